"""A stand-in for h5py, for the tests and for tests/golden/make_golden.py
(h5py is not installed where they run).

It keeps a file's groups, datasets and attributes in memory, and follows
h5py's rules for what the trajectory writers use:
* ``File(name, mode)``: 'w' creates or truncates the file at once (so a bad
  path raises), 'r' / 'a' read what an earlier ``close`` saved;
* ``create_group`` / ``create_dataset`` (from ``data=`` or from ``shape``,
  ``maxshape``, ``dtype``, ``chunks``, ``compression``), with names that
  may be paths ('topology/atoms/name'), membership and indexing by path,
  ``del``;
* ``Dataset.resize`` within ``maxshape`` (None = unlimited; new elements
  are zero, h5py's default fill value);
* assignment to an index or slice, whose value must broadcast to the
  selection (``TypeError`` otherwise) and is converted to the dataset's
  type; reading by index or slice;
* ``attrs`` as a dict; a ``File`` is true while it is open.

``close`` pickles the tree to the file name; ``load`` returns it flattened
to ``{path: {"data", "maxshape", "chunks", "compression", "attrs"}}`` for
datasets and ``{path: {"group": True, "attrs"}}`` for groups.
"""
import pickle
from pathlib import Path

import numpy as np

__version__ = "stand-in"


class Dataset(object):
    def __init__(self, data=None, shape=None, maxshape=None, dtype=None, chunks=None,
                 compression=None):
        if data is not None:
            arr = np.array(data, dtype=dtype) if dtype is not None else np.array(data)
        else:
            arr = np.zeros(tuple(shape), dtype=np.dtype(dtype) if dtype is not None
                           else np.float32)
        self._data = arr
        self.maxshape = tuple(maxshape) if maxshape is not None else arr.shape
        if len(self.maxshape) != arr.ndim:
            raise ValueError("maxshape and shape have different ranks")
        self.chunks = chunks
        self.compression = compression
        self.attrs = {}

    @property
    def shape(self):
        return self._data.shape

    @property
    def dtype(self):
        return self._data.dtype

    def __len__(self):
        return self._data.shape[0]

    def resize(self, size):
        size = tuple(int(s) for s in size)
        if len(size) != self._data.ndim:
            raise TypeError("new shape has the wrong rank")
        for s, m in zip(size, self.maxshape):
            if m is not None and s > m:
                raise ValueError("Unable to resize: new shape exceeds maxshape")
        new = np.zeros(size, dtype=self._data.dtype)
        keep = tuple(slice(0, min(a, b)) for a, b in zip(size, self._data.shape))
        new[keep] = self._data[keep]
        self._data = new

    def __setitem__(self, key, value):
        target = np.shape(self._data[key])
        v = np.asarray(value)
        try:
            v = np.broadcast_to(v, target)
        except ValueError:
            raise TypeError("Can't broadcast %s -> %s" % (v.shape, target))
        self._data[key] = v.astype(self._data.dtype)

    def __getitem__(self, key):
        return self._data[key]

    def _dump(self):
        return {"data": self._data.copy(), "maxshape": self.maxshape, "chunks": self.chunks,
                "compression": self.compression, "attrs": dict(self.attrs)}

    @classmethod
    def _load(cls, d):
        ds = cls(data=d["data"], maxshape=d["maxshape"], chunks=d["chunks"],
                 compression=d["compression"])
        ds.attrs.update(d["attrs"])
        return ds


class Group(object):
    def __init__(self):
        self._items = {}
        self.attrs = {}

    def _walk(self, path, make=False):
        parts = [p for p in str(path).split("/") if p]
        if not parts:
            raise ValueError("empty name")
        g = self
        for p in parts[:-1]:
            if p not in g._items:
                if not make:
                    raise KeyError(path)
                g._items[p] = Group()
            g = g._items[p]
            if not isinstance(g, Group):
                raise KeyError(path)
        return g, parts[-1]

    def create_group(self, name):
        g, last = self._walk(name, make=True)
        if last in g._items:
            raise ValueError("Unable to create group (name already exists)")
        g._items[last] = Group()
        return g._items[last]

    def create_dataset(self, name, shape=None, dtype=None, data=None, **kwargs):
        g, last = self._walk(name, make=True)
        if last in g._items:
            raise ValueError("Unable to create dataset (name already exists)")
        g._items[last] = Dataset(data=data, shape=shape, dtype=dtype, **kwargs)
        return g._items[last]

    def __contains__(self, name):
        try:
            g, last = self._walk(name)
        except (KeyError, ValueError):
            return False
        return last in g._items

    def __getitem__(self, name):
        g, last = self._walk(name)
        return g._items[last]

    def __delitem__(self, name):
        g, last = self._walk(name)
        del g._items[last]

    def keys(self):
        return self._items.keys()

    def _dump(self):
        return {"attrs": dict(self.attrs),
                "items": {k: (("group", v._dump()) if isinstance(v, Group)
                              else ("dataset", v._dump())) for k, v in self._items.items()}}

    @classmethod
    def _load(cls, d):
        g = cls()
        g.attrs.update(d["attrs"])
        for k, (kind, sub) in d["items"].items():
            g._items[k] = Group._load(sub) if kind == "group" else Dataset._load(sub)
        return g


class File(Group):
    def __init__(self, name, mode="r"):
        super().__init__()
        self.filename = str(name)
        self.mode = mode
        path = Path(name)
        if mode == "w":
            path.write_bytes(b"")
        elif mode in ("r", "r+", "a") and path.exists() and path.stat().st_size:
            with open(path, "rb") as fh:
                loaded = Group._load(pickle.load(fh))
            self._items, self.attrs = loaded._items, loaded.attrs
        elif mode in ("r", "r+"):
            raise FileNotFoundError(name)
        self._open = True

    def __bool__(self):
        return self._open

    def close(self):
        if self._open and self.mode != "r":
            with open(self.filename, "wb") as fh:
                pickle.dump(self._dump(), fh)
        self._open = False

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def load(path):
    """The saved tree of a stand-in file, flattened by path."""
    with open(path, "rb") as fh:
        tree = pickle.load(fh)
    out = {}

    def walk(d, prefix):
        for k, (kind, sub) in d["items"].items():
            p = prefix + "/" + k
            if kind == "group":
                out[p] = {"group": True, "attrs": sub["attrs"]}
                walk(sub, p)
            else:
                out[p] = sub
    walk(tree, "")
    return out
