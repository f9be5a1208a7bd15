"""CPU: host-side set-up (lattice, neighbour lists, k-vectors, process
tables) and the C-ABI library's exports.  No compute call needs a GPU."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

import golden_io as gio
from oracle import ewald_oracle as eo
from oracle import kmc_oracle as ko
from pycd_gb300 import _native as nat
from pycd_gb300 import ewald as ew
from pycd_gb300.core import Run, System

ROOT = Path(__file__).resolve().parent.parent


def test_library_exports_every_declared_symbol():
    lib = nat.lib()
    header = (ROOT / "include" / "pycd_gb300.h").read_text()
    declared = re.findall(r"PYCD_API\s+[\w\s\*]*?\b(pycd_\w+)\s*\(", header)
    assert len(declared) >= 12
    for name in declared:
        assert hasattr(lib, name), name
        assert name in nat.exported_symbols(), name
    assert lib.pycd_abi_version() == nat.ABI_VERSION == 4


def test_default_lanes_rule():
    """The launcher's default shape: at least one lane per carrier, about two
    processes per lane for large batches, a block of 4 warps for a single
    128-process trajectory, never more than 4 processes per lane in a block
    (whatever the SM count of the device, or 1 without one)."""
    from pycd_gb300.kmc import default_lanes
    assert default_lanes(16, 4, 10**6) == 8
    assert default_lanes(128, 32, 1) == 128
    assert default_lanes(64, 16, 1) == 128
    for npr, nc in ((4, 1), (16, 4), (32, 8), (64, 16), (128, 32), (96, 32)):
        for T in (1, 10, 100, 1000, 10**4, 10**6):
            g = default_lanes(npr, nc, T)
            assert g & (g - 1) == 0 and nc <= g <= 128
            assert -(-npr // g) <= (4 if g > 32 else 8)
    with pytest.raises(nat.NativeError):
        default_lanes(16, 33, 1)


def test_exp_table_is_correctly_rounded():
    """The kernels' table of 2^(j/4096), built by the library on the host from
    two seed tables: hi is 2^(j/4096) correctly rounded, hi + lo is within
    2^-100 of it, and |lo| < ulp(hi)/2 (so hi + lo rounds to hi, which the
    kernels' exp relies on)."""
    mp = pytest.importorskip("mpmath")
    import math
    mp.mp.prec = 200
    out = np.zeros(8192)
    nat.check(nat.lib().pycd_debug_exp_table(out.ctypes.data_as(ctypes.c_void_p)))
    hi, lo = out[0::2], out[1::2]
    for j in range(4096):
        exact = mp.mpf(2) ** (mp.mpf(j) / 4096)
        assert hi[j] == float(exact), j
        assert abs(mp.mpf(hi[j]) + mp.mpf(lo[j]) - exact) < exact * mp.mpf(2) ** -100, j
        assert abs(lo[j]) < math.ulp(hi[j]) / 2 and hi[j] + lo[j] == hi[j], j


def _exponent_bound(lu2, ktot):
    """The KMC kernels' per-step residence-time bound (TimeChain::push),
    restated: 2^(a - b + 1) as a float from the biased exponents a of lu2 and
    b of ktot; +inf for a subnormal ktot or above the float range, 2^-126
    below it."""
    a = (lu2.view(np.uint64) >> np.uint64(52)) & np.uint64(0x7FF)
    b = (ktot.view(np.uint64) >> np.uint64(52)) & np.uint64(0x7FF)
    k = a.astype(np.int64) - b.astype(np.int64) + 1
    out = np.ldexp(np.float32(1.0), np.clip(k, -126, 127).astype(np.int32)).astype(np.float32)
    out[(b == 0) | (k > 127)] = np.inf
    return out


def test_residence_time_bound_holds():
    """RN(-lu2 / ktot) <= the exponent-field bound for lu2 = log(u2), u2 in
    (0, 1], and ktot over the positive doubles (normal and subnormal): the
    deferred time chain may skip the exact time only while the summed bounds
    stay below the gap to the next grid row."""
    rng = np.random.default_rng(11)
    u2 = np.concatenate([rng.random(400_000), 1.0 - rng.random(2000) * 2.0 ** -40,
                         [1.0, np.nextafter(1.0, 0.0), 2.0 ** -53, 5e-324]])
    u2 = u2[u2 > 0]
    lu2 = np.log(u2)
    n = len(lu2)
    ktot = np.concatenate([
        np.exp(rng.uniform(np.log(1e-300), np.log(1e300), n // 2)),
        np.exp(rng.uniform(-40.0, 5.0, n - n // 2 - 4)),
        [5e-324, 2.2250738585072014e-308, 1.0, 1.7976931348623157e308]])
    rng.shuffle(ktot)
    with np.errstate(over="ignore"):  # tiny ktot: the quotient overflows, the bound is +inf
        q = (-lu2) / ktot
    bound = _exponent_bound(lu2, ktot).astype(np.float64)
    finite = np.isfinite(q)
    assert np.all(q[finite] <= bound[finite])
    assert np.all(np.isinf(bound[~finite]))
    # at most 4x loose where the bound is a normal float and the quotient is not tiny
    tight = np.isfinite(bound) & (bound > 2.0 ** -126) & (q > 0)
    assert np.all(bound[tight] <= 4.0 * q[tight])


def test_exp_fixed_table_is_correctly_rounded():
    """The integer exp's table: 2^(j/4096) 2^62 rounded to the nearest
    integer, built by the library from the (hi, lo) pairs with integer
    operations only (so every host builds the same table)."""
    mp = pytest.importorskip("mpmath")
    mp.mp.prec = 200
    out = np.zeros(4096, np.uint64)
    nat.check(nat.lib().pycd_debug_exp_table_fixed(out.ctypes.data_as(ctypes.c_void_p)))
    for j in range(4096):
        exact = int(mp.nint(mp.mpf(2) ** (mp.mpf(j) / 4096) * mp.mpf(2) ** 62))
        assert int(out[j]) == exact, j


def test_split_launch_fields_are_validated():
    """PycdEwaldDesc.split_form / split_raster: the defaults (0) and every
    allowed value size the workspace; values outside are rejected on the
    host with PYCD_ERR_INVALID_ARG (no device needed)."""
    d = nat.EwaldDesc()
    d.n_sites, d.n_kvec = 512, 100
    d.d_cart, d.d_kvec = 16, 16  # not dereferenced by the size query
    d.alpha, d.volume, d.dielectric = 0.1, 1000.0, 12.0
    size = nat.C.c_size_t()
    L = nat.lib()
    mode = nat.EWALD_MODES["bf16x3"]
    assert L.pycd_ewald_workspace_size(ctypes.byref(d), mode, ctypes.byref(size)) == 0
    base = size.value
    for form, raster in ((1, 1), (2, 64), (1, 0)):
        d.split_form, d.split_raster = form, raster
        assert L.pycd_ewald_workspace_size(ctypes.byref(d), mode, ctypes.byref(size)) == 0
        assert size.value == base
    for form, raster in ((3, 0), (-1, 0), (0, 65), (0, -1)):
        d.split_form, d.split_raster = form, raster
        rc = L.pycd_ewald_workspace_size(ctypes.byref(d), mode, ctypes.byref(size))
        assert rc == nat.ERR_INVALID_ARG, (form, raster)
        assert "split_" in nat.lib().pycd_last_error().decode()


def test_library_reports_missing_device_as_error():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(nat.NativeError) as e:
        nat.require_device()
    assert e.value.status == nat.ERR_NO_DEVICE


def test_neighbor_list_matches_reference_corundum324():
    cfg, arr = gio.load("corundum324")
    mat, nb = gio.material(cfg)
    ours = nb.generate_neighbor_list(None, (3, 3, 3), save=False)
    ref = gio.hop_list(cfg, arr)
    for key in ref:
        for ci, per_type in enumerate(ref[key]):
            for ti, rv in enumerate(per_type):
                mine = ours[key][ci][ti]
                assert np.array_equal(mine.num_neighbors, rv.num_neighbors)
                for i in range(len(rv.num_neighbors)):
                    assert np.array_equal(mine.neighbor_system_element_indices[i],
                                          rv.neighbor_system_element_indices[i])
                    assert np.array_equal(mine.displacement_vector_list[i],
                                          rv.displacement_vector_list[i])


def test_neighbor_list_matches_reference_corundum3600():
    """The 3,600-site lattice of the batched configuration (10x10x3 cells):
    our hop-neighbour list equals the reference's own (its digest over
    counts, indices and displacement vectors, generated by the reference)."""
    cfg, arr = gio.load("corundum3600")
    mat, nb = gio.material(cfg)
    ours = nb.generate_neighbor_list(None, (3, 3, 3), save=False)
    assert gio.hop_digest(ours) == cfg["hop_sha256"]


def test_pmiv_matches_reference_corundum324():
    import hashlib
    cfg, arr = gio.load("corundum324")
    mat, nb = gio.material(cfg)
    pmiv = nb.get_pairwise_min_image_vector_data(None)
    assert hashlib.sha256(pmiv.tobytes()).hexdigest() == cfg["pmiv_sha256"]


@pytest.mark.parametrize("name", ["corundum324", "hematite", "bvo"])
def test_k_vectors_match_oracle(name):
    cfg, arr = gio.load(name)
    mat, nb = gio.material(cfg)
    sysm = System(mat, nb, gio.hop_list(cfg, arr) if "hop_meta" in cfg else None,
                  None, cfg["params"]["alpha"], cfg["params"]["r_cut"],
                  cfg["params"]["k_cut"])
    kmax = ew.k_max_for(sysm, sysm.k_cut)
    ours = ew.effective_k_vectors(sysm.reciprocal_lattice_matrix, kmax, sysm.k_cut)
    ref = []
    for kv in eo.effective_k_vectors(kmax):
        k = np.dot(kv, sysm.reciprocal_lattice_matrix)
        if np.dot(k, k) < sysm.k_cut ** 2:
            ref.append(kv)
    assert np.array_equal(ours, np.asarray(ref, np.int32))
    # the C++ enumerator gives the same list
    L = nat.lib()
    recip = (ctypes.c_double * 9)(*sysm.reciprocal_lattice_matrix.ravel())
    km = (ctypes.c_int32 * 3)(*[int(v) for v in kmax])
    n = ctypes.c_int64()
    assert L.pycd_ewald_kvectors(recip, km, sysm.k_cut, None, 0, ctypes.byref(n)) == 0
    buf = (ctypes.c_int32 * (3 * n.value))()
    assert L.pycd_ewald_kvectors(recip, km, sysm.k_cut, buf, n.value,
                                 ctypes.byref(n)) == 0
    assert np.array_equal(np.frombuffer(buf, np.int32).reshape(-1, 3), ours)


def test_k_vector_cache_returns_the_enumerated_list():
    """effective_k_vectors keeps the last 64 lists by argument value: a kept
    list equals a fresh enumeration, comes back as the same read-only array
    and the cache stays bounded."""
    recip = np.array([[0.31, 0.0, 0.0], [0.02, 0.27, 0.0], [0.0, 0.0, 0.41]])
    km = np.array([4, 5, 3])
    first = {}
    for kc in (0.9, 1.3, 0.9):
        kv = ew.effective_k_vectors(recip, km, kc)
        half, keep = ew.half_space_k_vectors(recip, km, kc)
        assert np.array_equal(kv, half[keep]) and not kv.flags.writeable
        assert first.setdefault(kc, kv) is kv
    with pytest.raises(ValueError):
        kv[0, 0] = 1
    assert ew.effective_k_vectors(recip * 1.001, km, 1.3) is not first[1.3]
    for i in range(70):
        ew.effective_k_vectors(recip, km, 0.5 + 0.01 * i)
    assert len(ew._KV_CACHE) <= ew._KV_CACHE_MAX


def test_half_space_k_vectors_match_reference_k_vector_log():
    """The k-vectors listed by the reference's return_k_vector_data report
    (every half-space vector of the k_max box, those outside k_cut at zero)
    are the half-space list of pycd_gb300.ewald, and those with a non-zero
    contribution lie inside the cut."""
    import json
    cfg, arr = gio.load("hematite")
    ref = json.loads((gio.GOLDEN / "kvector_data.json").read_text())
    mat, nb = gio.material(cfg)
    p = ref["params"]
    sysm = System(mat, nb, gio.hop_list(cfg, arr), arr["pmiv"], p["alpha"], p["r_cut"],
                  p["k_cut"])
    kmax = ew.k_max_for(sysm, sysm.k_cut)
    kv, keep = ew.half_space_k_vectors(sysm.reciprocal_lattice_matrix, kmax, sysm.k_cut)
    rows = {}
    for line in ref["kvector_log"].splitlines()[1:]:
        k, e = line.split(":")
        rows[tuple(int(v) for v in k.split())] = float(e.split()[0])
    assert len(rows) == len(kv) == len(set(map(tuple, kv.tolist())))
    assert set(rows) == set(map(tuple, kv.tolist()))
    inside = set(map(tuple, kv[keep].tolist()))
    assert all(k in inside for k, e in rows.items() if e != 0.0)
    assert ref["report_lines"][0] == f"k_max: [{kmax[0]}, {kmax[1]}, {kmax[2]}]\n"


def test_corundum324_uses_feature_contraction():
    cfg, arr = gio.load("corundum324")
    mat, nb = gio.material(cfg)
    pmiv = nb.get_pairwise_min_image_vector_data(None)
    sysm = System(mat, nb, gio.hop_list(cfg, arr), pmiv, 0.25, 6.4, 1.6)
    assert ew.choose_mode(sysm, pmiv) == "fp64"
    assert ew.choose_mode(sysm, None) == "fp64"


def test_shipped_hematite_pmiv_needs_direct_mode():
    cfg, arr = gio.load("hematite")
    mat, nb = gio.material(cfg)
    sysm = System(mat, nb, gio.hop_list(cfg, arr), arr["pmiv"], 0.2667, 4.618, 6.998)
    assert ew.choose_mode(sysm, arr["pmiv"]) == "fp64_direct"
    with pytest.raises(ValueError):
        ew.choose_mode(sysm, arr["pmiv"], "fp64")


def _run(cfg, arr, mat, nb):
    run = cfg["run"]
    sysm = System(mat, nb, gio.hop_list(cfg, arr), None, cfg["params"]["alpha"],
                  cfg["params"]["r_cut"], cfg["params"]["k_cut"])
    return Run(sysm, arr["A"], run["temp"], run["ion_charge_type"],
               run["species_charge_type"], 1, run["t_final"], run["time_interval"],
               np.asarray(run["species_count"]), run["initial_occupancy"],
               run["relative_energies"], run["external_field"], run["doping"])


@pytest.mark.parametrize("name", ["hematite", "bvo"])
def test_site_tables_match_oracle_process_lists(name):
    cfg, arr = gio.load(name)
    mat, nb = gio.material(cfg)
    r = _run(cfg, arr, mat, nb)
    hop = gio.hop_list(cfg, arr)
    key = r.hop_element_type
    et = key.split(":")[0]
    ei = mat.element_types.index(et)
    t = ko.Tables(hop, key, np.tile(mat.unit_cell_class_list, int(nb.num_cells)),
                  int(mat.n_elements_per_unit_cell[ei]),
                  int(mat.n_elements_per_unit_cell[:ei].sum()),
                  int(mat.total_elements_per_unit_cell),
                  mat.lambda_values[key], mat.v_ab[key])
    n_checked = 0
    for site in range(nb.num_system_elements):
        if r.site_nbr[site, 0] < 0:
            continue
        procs = t.processes(site)
        assert len(procs) == r.n_slots == r.n_proc
        for s, (n, h, lam, vab, _) in enumerate(procs):
            assert r.site_nbr[site, s] == n
            assert np.array_equal(r.site_hop[site, s], h)
            assert r.site_lam[site, s] == lam and r.site_vab[site, s] == vab
        n_checked += 1
    assert n_checked == nb.num_cells * mat.n_elements_per_unit_cell[ei]


def test_multi_species_runs_are_rejected():
    cfg, arr = gio.load("hematite")
    mat, nb = gio.material(cfg)
    cfg = dict(cfg)
    cfg["run"] = dict(cfg["run"], species_count=[1, 1])
    with pytest.raises(NotImplementedError):
        _run(cfg, arr, mat, nb)


@pytest.mark.parametrize("name,cells", [("hematite", (2, 2, 1)), ("bvo", (3, 3, 3)),
                                        ("corundum324", (4, 3, 3))])
def test_translated_neighbor_list_equals_full_scan(name, cells):
    cfg, arr = gio.load(name)
    mat, nb = gio.material(cfg, system_size=cells)
    fast = nb.generate_neighbor_list(None, (3, 3, 3), save=False, method="auto")
    scan = nb.generate_neighbor_list(None, (3, 3, 3), save=False, method="scan")
    for key in scan:
        for ci in range(len(scan[key])):
            for ti in range(len(scan[key][ci])):
                a, b = fast[key][ci][ti], scan[key][ci][ti]
                assert np.array_equal(a.num_neighbors, b.num_neighbors)
                for i in range(len(b.num_neighbors)):
                    assert np.array_equal(a.neighbor_system_element_indices[i],
                                          b.neighbor_system_element_indices[i])
                    assert np.array_equal(np.asarray(a.displacement_vector_list[i]).reshape(-1, 3),
                                          np.asarray(b.displacement_vector_list[i]).reshape(-1, 3))


def test_mt19937_blocks_equal_cpython_random():
    """The drop-in KMC path draws each trajectory's uniforms in blocks with
    NumPy's MT19937: the values and the state after the used ones equal
    CPython's random.random() stream (PyCD/core.py:2799, 2802)."""
    import random
    from pycd_gb300.core import _Mt19937Stream
    r = random.Random(12345.678)
    st = _Mt19937Stream(r.getstate())
    out = np.empty(5000)
    st.fill(out)
    ref = np.array([r.random() for _ in range(5000)])
    assert np.array_equal(out, ref)
    st.used(1234)
    r2 = random.Random(12345.678)
    for _ in range(1234):
        r2.random()
    assert st.state() == r2.getstate()


def test_supercell_layout_of_synthetic_lattices():
    """The synthetic corundum and monoclinic supercells are described to the
    library as basis sites repeated over C-ordered cells; the shipped
    Hematite example (pmiv from an older min-image code) is not."""
    from pycd_gb300 import workloads as wl
    assert ew.supercell_layout(wl.corundum((3, 3, 3), neighbor_list=False)) == ([3, 3, 3], 12)
    assert ew.supercell_layout(wl.monoclinic((16, 16, 8), 0.9164)) == ([16, 16, 8], 4)
    cfg, arr = gio.load("hematite")
    mat, nb = gio.material(cfg)
    sysm = System(mat, nb, gio.hop_list(cfg, arr), arr["pmiv"], 0.2667, 4.618, 6.998)
    assert ew.supercell_layout(sysm, arr["pmiv"]) is None
