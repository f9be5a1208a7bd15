"""Load the golden fixtures of tests/golden into this package's objects."""
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
