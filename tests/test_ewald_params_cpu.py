"""CPU: the host side of the Ewald parameter search against the
reference's own get_ewald_parameters output (tests/golden/ewald_params.*):
the branches that only solve the cutoff-error models, and the error lines."""
import numpy as np
import pytest

import golden_io as gio
from pycd_gb300.core import System


def _system(name):
    cfg, arr = gio.load("ewald_params")
    hem_cfg, hem_arr = gio.load("hematite")
    case = cfg[name]
    mat, nb = gio.material(hem_cfg, system_size=case["system_size"])
    p = dict(cfg["base_params"], **case["params"])
    prec = dict(p["precision_parameters"], step_change_data_points=10)
    sysm = System(mat, nb, gio.hop_list(hem_cfg, hem_arr), hem_arr["pmiv"], p["alpha"],
                  p["r_cut"], p["k_cut"], prec)
    return sysm, case


def test_alpha_from_real_space_error_model(tmp_path):
    sysm, case = _system("alpha_optimal")
    alpha, r_cut, k_cut, choice, einsum, vdl, lines, _ = \
        sysm.get_cutoff_parameters(1.0, tmp_path, [])
    assert choice == {"alpha": "optimal", "r_cut": "user-specified",
                      "k_cut": "user-specified"}
    assert alpha == case["alpha"] and r_cut == case["r_cut"] and k_cut == case["k_cut"]
    errs = sysm.compute_cutoff_errors(einsum, alpha, r_cut, k_cut, vdl, [])
    assert "".join(errs) == "".join(case["lines"][3:5])


def test_step_change_analysis_counts_upward_steps_only():
    sysm, _ = _system("alpha_optimal")
    k = np.linspace(0.0, 1.0, 6)
    e = np.array([0.0, 0.0, 1e-3, 1e-3, 5e-4, 2e-3])
    k0, k1, de = sysm.get_step_change_analysis_with_k_cut(k, e)
    assert np.allclose(k0, [0.2, 0.8]) and np.allclose(k1, [0.4, 1.0])
    assert np.allclose(de, [1e-3, 1.5e-3])


def test_new_k_vectors_are_a_shell():
    sysm, _ = _system("alpha_optimal")
    b = sysm.reciprocal_lattice_vector_length.min()
    shell = np.asarray(sysm.get_new_k_vectors(1.5 * b, 2.5 * b))
    k = shell @ sysm.reciprocal_lattice_matrix
    k2 = (k * k).sum(axis=1)
    assert len(shell) > 0 and (k2 >= (1.5 * b) ** 2).all() and (k2 < (2.5 * b) ** 2).all()
