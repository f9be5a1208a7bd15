"""CPU: the oracle against the reference's golden vectors (pins the oracle)."""
import hashlib
import pickle
import random

import numpy as np
import pytest

import golden_io as gio
from oracle import ewald_oracle as eo
from oracle import kmc_oracle as ko
from oracle import philox
from pycd_gb300 import constants as K


def _geom(cfg, mat):
    p = cfg["params"]
    T, vol, recip = eo.ewald_geometry(mat.lattice_matrix, cfg["system_size"])
    return dict(alpha=p["alpha"] / K.ANG2BOHR, r_cut=p["r_cut"] * K.ANG2BOHR,
                k_cut=p["k_cut"] / K.ANG2BOHR, eps=p["dielectric_constant"],
                vol=vol, recip=recip)


@pytest.mark.parametrize("name", ["hematite", "bvo"])
def test_oracle_ewald_reproduces_shipped_array(name):
    cfg, arr = gio.load(name)
    mat, nb = gio.material(cfg)
    g = _geom(cfg, mat)
    A = eo.precomputed_array(arr["pmiv"], g["recip"], g["vol"], g["alpha"],
                             g["r_cut"], g["k_cut"], g["eps"])
    assert np.abs(A - arr["A"]).max() < 1e-15


def test_oracle_class_array_matches_reference_rows():
    cfg, arr = gio.load("corundum324")
    mat, nb = gio.material(cfg)
    g = _geom(cfg, mat)
    rows = np.asarray(cfg["A_rows"])
    A = eo.class_array(mat.cartesian_unit_cell_coords, mat.lattice_matrix,
                       cfg["system_size"], g["alpha"], g["r_cut"], g["k_cut"],
                       g["eps"], rows=rows)
    assert np.abs(A - arr["A_rows"]).max() < 1e-14


def _example_tables(cfg, arr, mat, nb):
    hop = gio.hop_list(cfg, arr)
    key = "Fe:Fe" if "Fe:Fe" in hop else "V:V"
    et = key.split(":")[0]
    ei = mat.element_types.index(et)
    ncls = np.tile(mat.unit_cell_class_list, int(nb.num_cells))
    lam = mat.lambda_values[key]
    vab = mat.v_ab[key]
    return ko.Tables(hop, key, ncls, int(mat.n_elements_per_unit_cell[ei]),
                     int(mat.n_elements_per_unit_cell[:ei].sum()),
                     int(mat.total_elements_per_unit_cell), lam, vab), ei


@pytest.mark.parametrize("name", ["bvo", "hematite"])
def test_oracle_kmc_reproduces_shipped_trajectory(name):
    cfg, arr = gio.load(name)
    mat, nb = gio.material(cfg)
    tables, ei = _example_tables(cfg, arr, mat, nb)
    run = cfg["run"]
    st = cfg["rnd_state"]
    random.setstate((st[0], tuple(st[1]), st[2]))
    # initial occupancy: rnd.sample over the hop-element sites (core.py:2527)
    n_cells = int(nb.num_cells)
    tpc = mat.total_elements_per_unit_cell
    head = mat.n_elements_per_unit_cell[:ei].sum()
    sites = [int(head + e + c * tpc) for c in range(n_cells)
             for e in range(mat.n_elements_per_unit_cell[ei])]
    sites = sorted(sites)
    occ = random.sample(sites, 1)
    n = cfg["n_steps"]
    u = np.array([random.random() for _ in range(2 * n + 2)])
    q = np.tile(np.array([mat.charge_types["full"][mat.element_types[e]]
                          for e in mat.element_type_index_list]), n_cells)
    e_rel = np.zeros(nb.num_system_elements)
    dt = run["time_interval"] * K.SEC2AUTIME
    n_path = int(run["t_final"] * K.SEC2AUTIME / dt) + 1
    out = ko.run(arr["A"], tables, occ, q, -1.0, e_rel, mat.vn,
                 run["temp"] * K.K2AUTEMP, u, dt, n_path)
    assert out["stop"] == "done" and out["steps"] == n
    u_sha = hashlib.sha256(np.ascontiguousarray(out["unwrapped"]).tobytes()).hexdigest()
    assert u_sha == cfg["unwrapped_sha256"]
    t = out["time"][::cfg["time_stride"]]
    ref = arr["time"]
    assert np.abs(t[1:] / ref[1:] - 1).max() < 1e-12


def test_oracle_kmc_reproduces_reference_doped_bvo():
    """The reference's doped BVO run (two W dopants of charge 6, shell
    energies from site_indices.npy, the electron drawn onto a dopant site by
    rnd.sample, core.py:2478-2528, 2723-2772): the oracle, given the
    reference's doped site energies, reproduces its occupancy list and its
    unwrapped rows bit for bit and its times within 1e-12."""
    cfg, arr = gio.load("bvo")
    ref, fix = gio.load("bvo_doped")
    mat, nb = gio.material(cfg)
    tables, ei = _example_tables(cfg, arr, mat, nb)
    run = cfg["run"]
    st = cfg["rnd_state"]
    random.setstate((st[0], tuple(st[1]), st[2]))
    si = fix["site_indices"]
    dopants = [int(x) for x in si[si[:, 3] == 0, 0]]
    occ = random.sample(dopants, 1)  # site_charge_initiation 'yes'
    n = ref["n_steps"]
    u = np.array([random.random() for _ in range(2 * n + 2)])
    n_cells = int(nb.num_cells)
    q = np.tile(np.array([mat.charge_types["full"][mat.element_types[e]]
                          for e in mat.element_type_index_list]), n_cells).astype(float)
    q[dopants] = ref["doping"]["charge"]["full"]["W"]
    dt = run["time_interval"] * K.SEC2AUTIME
    n_path = int(ref["t_final"] * K.SEC2AUTIME / dt) + 1
    out = ko.run(arr["A"], tables, occ, q, -1.0, fix["system_relative_energies"], mat.vn,
                 run["temp"] * K.K2AUTEMP, u, dt, n_path)
    assert out["stop"] == "done" and out["steps"] == n
    assert np.array_equal(np.asarray(out["sites"])[:, 0], fix["occupancy"][1:, 0])
    assert fix["occupancy"][0, 0] == occ[0]
    assert np.array_equal(out["unwrapped"], fix["unwrapped"])
    assert np.abs(out["time"][1:] / fix["time"][1:] - 1).max() < 1e-12


def test_oracle_energy_and_delg0_grids_match_reference_hematite():
    """The reference's Hematite run with the energy and dG0 path grids
    written (initial energy core.py:2663-2667; grids 2806-2808, 2848-2861):
    the oracle reproduces its rows bit for bit, its energies within 1e-12
    relative and its dG0 within 1e-14 Ha."""
    cfg, arr = gio.load("hematite")
    ref, fix = gio.load("hematite_outputs")
    mat, nb = gio.material(cfg)
    tables, ei = _example_tables(cfg, arr, mat, nb)
    run = cfg["run"]
    st = cfg["rnd_state"]
    random.setstate((st[0], tuple(st[1]), st[2]))
    n_cells = int(nb.num_cells)
    tpc = mat.total_elements_per_unit_cell
    head = mat.n_elements_per_unit_cell[:ei].sum()
    sites = sorted(int(head + e + c * tpc) for c in range(n_cells)
                   for e in range(mat.n_elements_per_unit_cell[ei]))
    occ = random.sample(sites, 1)
    n = ref["n_steps"]
    u = np.array([random.random() for _ in range(2 * n + 2)])
    q = np.tile(np.array([mat.charge_types["full"][mat.element_types[e]]
                          for e in mat.element_type_index_list]), n_cells).astype(float)
    # initial energy as the reference forms it: neutralising background plus
    # the pair sum over the charges with the carrier
    g = _geom(cfg, mat)
    qc = q.reshape(-1, 1).copy()
    qc[occ[0]] += -1.0
    ewald_neut = -(np.pi * 1.0 ** 2 / (2 * g["vol"] * g["alpha"]))
    energy0 = ewald_neut + np.sum(np.multiply(np.multiply(qc.transpose(), qc), arr["A"]))
    dt = run["time_interval"] * K.SEC2AUTIME
    n_path = int(ref["t_final"] * K.SEC2AUTIME / dt) + 1
    out = ko.run(arr["A"], tables, occ, q, -1.0, np.zeros(nb.num_system_elements), mat.vn,
                 run["temp"] * K.K2AUTEMP, u, dt, n_path, energy0=energy0)
    assert out["stop"] == "done" and out["steps"] == n
    assert np.array_equal(out["unwrapped"], fix["unwrapped_traj"])
    e, er = out["energy"], fix["energy"]
    assert np.abs(e - er).max() <= 1e-12 * np.abs(er).max()
    assert np.abs(out["delg0"] - fix["delg_0"]).max() <= 1e-14


def test_oracle_kmc_matches_reference_events_corundum324():
    cfg, arr = gio.load("corundum324")
    mat, nb = gio.material(cfg)
    hop = gio.hop_list(cfg, arr)
    tables = ko.Tables(hop, "Fe:Fe", np.zeros(324, int), 12, 0, 12,
                       mat.lambda_values["Fe:Fe"], mat.v_ab["Fe:Fe"])
    g = _geom(cfg, mat)
    pmiv = nb.get_pairwise_min_image_vector_data(None)
    assert hashlib.sha256(pmiv.tobytes()).hexdigest() == cfg["pmiv_sha256"]
    A = eo.precomputed_array(pmiv, g["recip"], g["vol"], g["alpha"], g["r_cut"],
                             g["k_cut"], g["eps"])
    rows = np.asarray(cfg["A_rows"])
    assert np.abs(A[rows] - arr["A_rows"]).max() < 1e-16
    n = 20000  # prefix: the full 1e5 steps run in the GPU test
    u = np.random.default_rng(cfg["uniform_seed"]).random(2 * n)
    dt = cfg["time_interval"] * K.SEC2AUTIME
    n_path = int(cfg["t_final"] * K.SEC2AUTIME / dt) + 1
    out = ko.run(A, tables, [cfg["carrier_site"]], np.zeros(324), -1.0,
                 np.zeros(324), mat.vn, 300 * K.K2AUTEMP, u, dt, n_path)
    assert out["steps"] == n
    assert np.array_equal(out["proc"], arr["proc"][:n])
    t = out["time"][::8]
    assert np.abs(t[1:] / arr["time"][1:len(t)] - 1).max() < 1e-12


def test_philox_known_answers():
    # Random123 known-answer vectors for Philox4x32-10
    assert philox.philox4x32_10((0, 0, 0, 0), (0, 0)) == \
        (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)
    m = 0xFFFFFFFF
    assert philox.philox4x32_10((m, m, m, m), (m, m)) == \
        (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)
    assert philox.philox4x32_10((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344),
                                (0xa4093822, 0x299f31d0)) == \
        (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1)
