"""GPU: the Ewald parameter search (pycd_gb300.ewald_params, energy scans
on the device) against the reference's own get_ewald_parameters on the
Hematite example lattice: the chosen alpha / r_cut / k_cut, the report lines
after the timing lines, and the k_cut convergence and k-vector contribution
logs."""
import json

import numpy as np
import pytest

import golden_io as gio
from pycd_gb300 import constants as K
from pycd_gb300.core import System

pytestmark = pytest.mark.gpu

CASES = ["rcut_optimal", "rcut_kcut_optimal", "alpha_optimal", "kcut_converge"]


def _system(name):
    cfg, arr = gio.load("ewald_params")
    hem_cfg, hem_arr = gio.load("hematite")
    case = cfg[name]
    mat, nb = gio.material(hem_cfg, system_size=case["system_size"])
    pmiv = hem_arr["pmiv"] if case["system_size"] == [2, 2, 1] else arr[name + "|pmiv"]
    p = dict(cfg["base_params"], **case["params"])
    prec = dict(p["precision_parameters"], step_change_data_points=10)
    sysm = System(mat, nb, gio.hop_list(hem_cfg, hem_arr), pmiv, p["alpha"], p["r_cut"],
                  p["k_cut"], prec)
    return sysm, case


def _numbers(text):
    """Lines with their %.3e numbers parsed, to compare within the last digit."""
    out = []
    for line in text.splitlines():
        toks = []
        for t in line.replace("[", " ").replace("]", " ").replace(",", " ").split():
            try:
                toks.append(float(t))
            except ValueError:
                toks.append(t)
        out.append(toks)
    return out


def _same_lines(got, want):
    g, w = _numbers(got), _numbers(want)
    assert len(g) == len(w), (len(g), len(w))
    for a, b in zip(g, w):
        assert len(a) == len(b), (a, b)
        for x, y in zip(a, b):
            if isinstance(y, float) and isinstance(x, float):
                # printed with 4 significant digits: equal, or one unit of
                # the last digit apart when a value sits on a rounding edge
                assert x == y or abs(x - y) <= 1.01e-3 * abs(y), (a, b)
            else:
                assert x == y, (a, b)


def _same_contributions(got, want):
    """k-vectors sorted by decreasing energy contribution.  k and -k
    contribute exactly equally and NumPy's argsort is not stable, so the order
    inside ties depends on the last bits of the values: compare the lines as
    a set (energies within one unit of the printed digit) and check the order."""
    def parse(text):
        head, rows = [], {}
        for line in text.splitlines():
            if ":" in line and line.strip().endswith("eV"):
                k, e = line.split(":")
                rows[tuple(int(v) for v in k.split())] = float(e.split()[0])
            else:
                head.append(line)
        return head, rows
    gh, g = parse(got)
    wh, w = parse(want)
    assert gh == wh and g.keys() == w.keys()
    # each contribution is a sum of O(1) pair terms that nearly cancel: its
    # rounding is absolute, at ~1e-16 of the largest contribution
    floor = 1e-13 * max(abs(e) for e in w.values())
    for k, e in w.items():
        assert abs(g[k] - e) <= max(1.01e-3 * abs(e), floor), (k, g[k], e)
    order = [float(l.split(":")[1].split()[0]) for l in got.splitlines()
             if ":" in l and l.strip().endswith("eV")]
    assert all(a >= b for a, b in zip(order, order[1:]))


@pytest.mark.parametrize("name", CASES)
def test_parameter_search_matches_reference(cuda_ready, tmp_path, name):
    sysm, case = _system(name)
    dst = tmp_path / "InputFiles"
    dst.mkdir()
    params, lines, dst2 = sysm.get_ewald_parameters([], dst)
    assert not case["exit"]
    assert params["alpha"] == pytest.approx(case["alpha"], rel=1e-12)
    assert params["r_cut"] == pytest.approx(case["r_cut"], rel=1e-12)
    assert params["k_cut"] == pytest.approx(case["k_cut"], rel=1e-12)
    _same_lines("".join(lines[2:]), "".join(case["lines"]))
    assert str(dst2.relative_to(dst)) == case["dst_suffix"]
    for rel, text in case["files"].items():
        got = (dst / rel).read_text().split("Time elapsed")[0]
        if "k_vector_energy_contribution" in rel:
            _same_contributions(got, text)
        else:
            _same_lines(got, text)


def test_automatic_parameters_flow_into_the_build(cuda_ready, tmp_path):
    """get_precomputed_array with r_cut 'optimal' builds with the chosen
    r_cut and reports it on line 5 (alpha on line 4, read by material_run)."""
    sysm, case = _system("rcut_optimal")
    dst = tmp_path / "InputFiles"
    dst.mkdir()
    A, _ = sysm.get_precomputed_array(dst, 1, 0)
    assert A.shape == (120, 120) and np.isfinite(A).all()
    log = (dst / "precomputed_array.log").read_text().splitlines()
    assert log[3].startswith("alpha: ") and "(user-specified)" in log[3]
    assert log[4].startswith("r_cut: ") and "(optimal)" in log[4]
    assert float(log[4].split()[1]) == pytest.approx(case["r_cut"] * 0.529177210903, rel=2e-3)
    assert any(l.startswith("Total system energy (neutral): ") for l in log)


def test_kvector_energies_equal_one_vector_builds(cuda_ready):
    """pycd_ewald_kvector_energies (all k in one pass) against one Fourier
    build per k-vector, both the reference's get_k_vector_energy_contribution."""
    sysm, _ = _system("kcut_converge")
    ev = sysm._energy_evaluator()
    kv = np.array([[1, 0, 0], [0, 1, 0], [1, 1, 0], [-1, 2, 1], [2, 0, -3], [0, 0, 1]])
    batch = ev.k_vectors(sysm.alpha, kv)
    single = np.array([ev.k_vector(sysm.alpha, k) for k in kv])
    scale = np.abs(single).max()
    assert np.abs(batch - single).max() <= 1e-12 * scale


def test_fourier_energy_from_per_k_cache_equals_build(cuda_ready):
    """The cached per-k Fourier energy of a small system equals the energy of
    the part-only device build at several cutoffs."""
    sysm, _ = _system("kcut_converge")
    ev = sysm._energy_evaluator()
    for k_cut in (1.0, 2.5, 4.0):
        via_cache = ev.fourier(sysm.alpha, k_cut)
        via_build = ev._energy(sysm.alpha, 0.0, k_cut, 2)
        assert abs(via_cache - via_build) <= 1e-12 * max(abs(via_build), 1e-300)


def test_return_k_vector_data_matches_reference(cuda_ready, tmp_path):
    """get_precomputed_array(dst, 0, 1) on the Hematite example writes the
    reference's k_vector_energy_contribution_within_user_specified_k_cut.log
    (PyCD/core.py:1626-1653): the same k-vectors with the same contributions
    (ties compared as a set), sorted in decreasing order, and returns the
    shipped array."""
    ref = json.loads((gio.GOLDEN / "kvector_data.json").read_text())
    cfg, arr = gio.load("hematite")
    mat, nb = gio.material(cfg)
    p = ref["params"]
    sysm = System(mat, nb, gio.hop_list(cfg, arr), arr["pmiv"], p["alpha"], p["r_cut"],
                  p["k_cut"])
    dst = tmp_path / "InputFiles"
    A, _ = sysm.get_precomputed_array(dst, 0, 1)
    assert np.abs(A - arr["A"]).max() < 1e-10 * K.EV2HARTREE  # 1e-10 eV
    got = (dst / "k_vector_energy_contribution_within_user_specified_k_cut.log").read_text()
    assert "Time elapsed" not in got
    _same_contributions(got, ref["kvector_log"])
    log = (dst / "precomputed_array.log").read_text()
    for line in ref["report_lines"]:
        assert line in log
