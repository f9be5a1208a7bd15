"""Load the golden fixtures of tests/golden into this package's objects, and
the canonical array form of a hop-neighbour list shared with the generator."""
import hashlib
import json
import tempfile
from pathlib import Path

import numpy as np

from pycd_gb300.lattice import Material, Neighbors, ReturnValues

GOLDEN = Path(__file__).resolve().parent / "golden"


def load(name):
    cfg = json.loads((GOLDEN / f"{name}.json").read_text())
    arr = dict(np.load(GOLDEN / f"{name}.npz"))
    return cfg, arr


def hop_list(cfg, arr):
    out = {}
    for key, n_types_per_class in cfg["hop_meta"].items():
        per_class = []
        for ci, n_types in enumerate(n_types_per_class):
            per_type = []
            for ti in range(n_types):
                tag = f"hop|{key}|{ci}|{ti}"
                cnt = arr[tag + "|count"]
                idx, vec = arr[tag + "|idx"], arr[tag + "|vec"]
                nidx = np.empty(len(cnt), dtype=object)
                nvec = np.empty(len(cnt), dtype=object)
                o = 0
                for i, c in enumerate(cnt):
                    nidx[i] = idx[o:o + c]
                    nvec[i] = vec[o:o + c]
                    o += c
                per_type.append(ReturnValues(neighbor_system_element_indices=nidx,
                                             displacement_vector_list=nvec,
                                             num_neighbors=cnt))
            per_class.append(per_type)
        out[key] = per_class
    return out


def material(cfg, system_size=None):
    d = Path(tempfile.mkdtemp())
    (d / "POSCAR").write_text(cfg["poscar"])
    p = dict(cfg["params"])
    p.pop("precision_parameters", None)
    p["input_coord_file_location"] = d / "POSCAR"
    mat = Material(ReturnValues(**p))
    ss = np.asarray(system_size if system_size is not None else cfg["system_size"])
    nb = Neighbors(mat, ss, np.asarray(cfg["pbc"]))
    return mat, nb


def hop_to_arrays(hop):
    """A hop-neighbour list ({key: [class][type] -> neighbour record}) as
    (meta, arrays): per record the neighbour counts, the concatenated
    neighbour indices (int64) and displacement vectors (float64, (n, 3))."""
    meta, arrs = {}, {}
    for key, per_class in hop.items():
        meta[key] = []
        for ci, per_type in enumerate(per_class):
            meta[key].append(len(per_type))
            for ti, rv in enumerate(per_type):
                tag = f"hop|{key}|{ci}|{ti}"
                arrs[tag + "|count"] = np.asarray(rv.num_neighbors, np.int64)
                idx = [np.asarray(x, np.int64) for x in rv.neighbor_system_element_indices]
                vec = [np.asarray(x, np.float64).reshape(-1, 3)
                       for x in rv.displacement_vector_list]
                arrs[tag + "|idx"] = np.concatenate(idx) if idx else np.zeros(0, np.int64)
                arrs[tag + "|vec"] = np.concatenate(vec) if vec else np.zeros((0, 3))
    return meta, arrs


def hop_digest(hop):
    """sha256 over a hop-neighbour list's per-site counts, neighbour indices
    and displacement vectors, in key / class / type order."""
    meta, arrs = hop_to_arrays(hop)
    h = hashlib.sha256(json.dumps(meta, sort_keys=True).encode())
    for tag in sorted(arrs):
        h.update(tag.encode())
        h.update(np.ascontiguousarray(arrs[tag]).tobytes())
    return h.hexdigest()
