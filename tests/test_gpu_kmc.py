"""GPU: the KMC kernel against the reference's trajectories, the oracle, and
itself (one trajectory alone vs inside a batch).

Events and carrier sites must match bit-exactly; residence times within
1e-12 relative; unwrapped displacement rows bit-identical."""
import hashlib
import pickle
import tempfile
from pathlib import Path

import numpy as np
import pytest

import golden_io as gio
from oracle import kmc_oracle as ko
from oracle import philox
from pycd_gb300 import _native as nat
from pycd_gb300 import constants as K
from pycd_gb300 import workloads as wl
from pycd_gb300.core import Run, System
from pycd_gb300.kmc import KmcBatch, KmcEngine, KmcTables

pytestmark = pytest.mark.gpu
TIME_RTOL = 1e-12


def _example_run(name, t_final=None, doping=None, n_traj=1):
    cfg, arr = gio.load(name)
    mat, nb = gio.material(cfg)
    p, r = cfg["params"], cfg["run"]
    sysm = System(mat, nb, gio.hop_list(cfg, arr), arr["pmiv"], p["alpha"],
                  p["r_cut"], p["k_cut"])
    run = Run(sysm, arr["A"], r["temp"], r["ion_charge_type"],
              r["species_charge_type"], n_traj, t_final or r["t_final"], r["time_interval"],
              np.asarray(r["species_count"]), r["initial_occupancy"],
              r["relative_energies"], r["external_field"], doping or r["doping"])
    return cfg, arr, run


@pytest.mark.parametrize("name", ["bvo", "hematite"])
def test_do_kmc_steps_reproduces_shipped_trajectory(cuda_ready, name):
    cfg, arr, run = _example_run(name)
    d = Path(tempfile.mkdtemp())
    st = cfg["rnd_state"]
    with open(d / "initial_rnd_state.dump", "wb") as fh:
        pickle.dump((st[0], tuple(st[1]), st[2]), fh)
    run.do_kmc_steps(d, cfg["run"]["output_data"], cfg["run"]["random_seed"],
                     "parallel")
    u = np.load(d / "unwrapped_traj.npy")
    t = np.load(d / "time_data.npy")
    assert len(t) == cfg["n_steps"] + 1
    assert hashlib.sha256(u.tobytes()).hexdigest() == cfg["unwrapped_sha256"]
    ts = t[::cfg["time_stride"]]
    assert np.abs(ts[1:] / arr["time"][1:] - 1).max() < TIME_RTOL
    assert abs(t[-1] / arr["time_last"][0] - 1) < TIME_RTOL
    assert (d / "Run.log").exists()


def test_do_kmc_steps_batched_trajectories_equal_runs_alone(cuda_ready, tmp_path):
    """n_traj = 8 in one call (serial mode: preproduction seeds traj1..traj8
    from random_seed, as core.py:2566-2580) advances the eight trajectories
    together.  Every file of every trajectory equals, byte for byte, the file
    of that trajectory run alone from its initial_rnd_state.dump, and the
    module's random state ends where the last trajectory's own run leaves
    it."""
    import random as rnd
    import shutil
    import time
    cfg, arr, run8 = _example_run("hematite", t_final=2e-6, n_traj=8)
    od = cfg["run"]["output_data"]
    d8 = tmp_path / "together"
    t0 = time.perf_counter()
    run8.do_kmc_steps(d8, od, 7, "serial")
    t_together = time.perf_counter() - t0
    state8 = rnd.getstate()
    t_alone = 0.0
    for i in range(8):
        d1 = tmp_path / f"alone{i + 1}"
        d1.mkdir()
        shutil.copy(d8 / f"traj{i + 1}" / "initial_rnd_state.dump", d1)
        _, _, run1 = _example_run("hematite", t_final=2e-6)
        t0 = time.perf_counter()
        run1.do_kmc_steps(d1, od, 7, "parallel")
        t_alone += time.perf_counter() - t0
        names = sorted(f.name for f in (d8 / f"traj{i + 1}").glob("*.npy"))
        assert "unwrapped_traj.npy" in names and "time_data.npy" in names
        for name in names:
            assert (d8 / f"traj{i + 1}" / name).read_bytes() == (d1 / name).read_bytes(), \
                (i, name)
        assert len(run8.last_run_steps[i]) == len(run1.last_run_steps[0])
    assert rnd.getstate() == state8
    print(f"8 trajectories of examples/Hematite to t = 2e-6: one call {t_together:.2f} s, "
          f"one call each {t_alone:.2f} s")


def test_do_kmc_steps_write_every_step_matches_reference(cuda_ready):
    """write_every_step = 1 (core.py:2832-2846): the per-step unwrapped rows
    of the reference's own run of examples/Hematite (~2,000 steps from the
    shipped random state), bit for bit, and its times."""
    ref, fix = gio.load("hematite_every_step")
    cfg, arr, run = _example_run("hematite", t_final=ref["t_final"])
    d = Path(tempfile.mkdtemp())
    st = cfg["rnd_state"]
    with open(d / "initial_rnd_state.dump", "wb") as fh:
        pickle.dump((st[0], tuple(st[1]), st[2]), fh)
    run.do_kmc_steps(d, ref["output_data"], cfg["run"]["random_seed"], "parallel")
    u = np.load(d / "unwrapped_traj.npy")
    t = np.load(d / "time_data.npy")
    assert len(t) == ref["n_steps"] + 1
    assert np.array_equal(u, fix["unwrapped"])
    assert np.abs(t[1:] / fix["time"][1:] - 1).max() < TIME_RTOL


def test_do_kmc_steps_hdf5_output_matches_reference(cuda_ready, monkeypatch):
    """hdf5_output enabled (core.py:2677-2691, 2882-2902), per step and on
    the time grid, written through the h5py stand-in: the layout, topology
    and float32 coordinates of the file the reference's own run of
    examples/Hematite wrote (tests/golden/hdf5.*), bit for bit.  /time holds
    each frame's time (the reference's is zero-filled: h5py refuses the
    time list it passes, as its recorded warning shows)."""
    import sys
    import fake_h5py
    monkeypatch.setitem(sys.modules, "h5py", fake_h5py)
    monkeypatch.delitem(sys.modules, "pycd_gb300.hdf5_io", raising=False)
    ref, arr = gio.load("hdf5")
    arrays = {k.replace("|", "/"): v for k, v in arr.items()}
    try:
        for label, every in (("run_every_step", 1), ("run_grid", 0)):
            meta = ref["runs"][label]
            assert meta["warnings"] and "Can't broadcast" in meta["warnings"][0]
            cfg, _, run = _example_run("hematite", t_final=ref["t_final"])
            d = Path(tempfile.mkdtemp())
            st = cfg["rnd_state"]
            with open(d / "initial_rnd_state.dump", "wb") as fh:
                pickle.dump((st[0], tuple(st[1]), st[2]), fh)
            run.do_kmc_steps(d, meta["output_data"], cfg["run"]["random_seed"], "parallel")
            got = fake_h5py.load(d / "trajectory.h5")
            rec = ref["records"][label]
            assert sorted(got) == sorted(rec)
            for key, want in rec.items():
                if want.get("group"):
                    continue
                assert got[key]["data"].dtype.str == want["dtype"], key
                assert list(got[key]["data"].shape) == want["shape"], key
                assert got[key]["attrs"] == want["attrs"], key
                if key != "/time":
                    assert np.array_equal(got[key]["data"], arrays[label + key]), key
            t = np.load(d / "time_data.npy")
            n = meta["rows"]
            want_t = (t[1:] if every else np.arange(n) * run.time_interval) * K.AUTIME2PS
            assert np.array_equal(got["/time"]["data"], want_t)
    finally:
        sys.modules.pop("pycd_gb300.hdf5_io", None)


def test_do_kmc_steps_doped_bvo_matches_reference(cuda_ready):
    """examples/BVO with two W dopants (charge 6) and shell-indexed site
    energies read from site_indices.npy, the electron starting on a dopant
    site (MT19937 rnd.sample): the doped site energies, the occupancy list,
    the unwrapped rows and the times of the reference's own run."""
    ref, fix = gio.load("bvo_doped")
    cfg, arr, run = _example_run("bvo", t_final=ref["t_final"], doping=ref["doping"])
    d = Path(tempfile.mkdtemp())
    st = cfg["rnd_state"]
    with open(d / "initial_rnd_state.dump", "wb") as fh:
        pickle.dump((st[0], tuple(st[1]), st[2]), fh)
    np.save(d / "site_indices.npy", fix["site_indices"])
    run.do_kmc_steps(d, ref["output_data"], cfg["run"]["random_seed"], "parallel")
    assert np.array_equal(np.asarray(run.system_relative_energies),
                          fix["system_relative_energies"])
    assert np.array_equal(np.load(d / "occupancy.npy"), fix["occupancy"])
    u = np.load(d / "unwrapped_traj.npy")
    t = np.load(d / "time_data.npy")
    assert len(t) == ref["n_steps"] + 1
    assert np.array_equal(u, fix["unwrapped"])
    assert np.abs(t[1:] / fix["time"][1:] - 1).max() < TIME_RTOL


def test_do_kmc_steps_energy_and_delg0_grids_match_reference(cuda_ready):
    """examples/Hematite, ~2,000 steps with the energy and dG0 path grids
    written: rows and events bit for bit; energies within 1e-12 relative;
    dG0 (a difference of ~1 Ha potentials, ~1e-8 Ha here) within 1e-14 Ha."""
    ref, fix = gio.load("hematite_outputs")
    cfg, arr, run = _example_run("hematite", t_final=ref["t_final"])
    d = Path(tempfile.mkdtemp())
    st = cfg["rnd_state"]
    with open(d / "initial_rnd_state.dump", "wb") as fh:
        pickle.dump((st[0], tuple(st[1]), st[2]), fh)
    od = ref["output_data"]
    run.do_kmc_steps(d, od, cfg["run"]["random_seed"], "parallel")
    got = {k: np.load(d / od[k]["file_name"])
           for k in ("unwrapped_traj", "time", "energy", "delg_0")}
    assert len(got["time"]) == ref["n_steps"] + 1
    assert np.array_equal(got["unwrapped_traj"], fix["unwrapped_traj"])
    assert np.abs(got["time"][1:] / fix["time"][1:] - 1).max() < TIME_RTOL
    e, er = got["energy"], fix["energy"]
    assert e.shape == er.shape and np.abs(e - er).max() <= 1e-12 * np.abs(er).max()
    g, gr = got["delg_0"], fix["delg_0"]
    assert g.shape == gr.shape and np.abs(g - gr).max() <= 1e-14


def _corundum324_engine(cfg, arr):
    import torch
    mat, nb = gio.material(cfg)
    sysm = System(mat, nb, gio.hop_list(cfg, arr), None, cfg["params"]["alpha"],
                  cfg["params"]["r_cut"], cfg["params"]["k_cut"])
    A = sysm.get_precomputed_array_device("fp64")
    tables, run = wl.batched_tables(sysm, A, 1, [], t_final=cfg["t_final"],
                                    time_interval=cfg["time_interval"])
    return tables, run


def test_plain_events_match_reference_corundum324(cuda_ready):
    import torch
    cfg, arr = gio.load("corundum324")
    tables, run = _corundum324_engine(cfg, arr)
    n = cfg["n_steps"]
    u = torch.as_tensor(np.random.default_rng(cfg["uniform_seed"]).random(2 * n)
                        ).cuda()[None, :]
    batch = KmcBatch([[cfg["carrier_site"]]], step_capacity=n,
                     unwrapped_rows=tables.n_path_steps)
    eng = KmcEngine(tables)
    eng.advance(batch, n + 10, eng.rng_struct(u))
    torch.cuda.synchronize()
    assert int(batch.status.item()) == nat.TRAJ_NEED_UNIFORMS
    assert int(batch.step.item()) == n
    proc = batch.step_proc[0].cpu().numpy()
    assert np.array_equal(proc, arr["proc"].astype(np.int32))
    t = batch.step_time[0].cpu().numpy()[7::8]
    assert np.abs(t / arr["time"][1:len(t) + 1] - 1).max() < TIME_RTOL


def _corundum3600(n_carriers=4):
    sysm = wl.corundum((10, 10, 3))
    A = sysm.get_precomputed_array_device("fp64")
    cfg, arr = gio.load("corundum3600")
    tables, run = wl.batched_tables(sysm, A, n_carriers, cfg["dopants"],
                                    cfg["dopant_charge"], t_final=cfg["t_final"],
                                    time_interval=cfg["time_interval"])
    return sysm, tables, run, cfg, arr


def test_batched_events_match_reference_corundum3600(cuda_ready):
    import torch
    sysm, tables, run, cfg, arr = _corundum3600()
    n = cfg["n_steps"]
    U = np.stack([np.random.default_rng(s).random(2 * n) for s in cfg["uniform_seeds"]])
    batch = KmcBatch([cfg["carriers"]] * 2, step_capacity=n)
    eng = KmcEngine(tables)
    eng.advance(batch, n, eng.rng_struct(torch.as_tensor(U).cuda()))
    torch.cuda.synchronize()
    assert batch.step.cpu().tolist() == [n, n]
    assert np.array_equal(batch.step_proc.cpu().numpy(), arr["proc"].astype(np.int32))
    t = batch.step_time.cpu().numpy()
    assert np.abs(t / arr["time"][:, 1:] - 1).max() < TIME_RTOL


def test_batch_equals_plain_and_oracle_on_sampled_trajectories(cuda_ready):
    """512 Philox trajectories advanced together; 8 of them re-run alone
    (plain form) must give identical events and times, and the oracle, fed
    the same Philox uniforms, the same events for a prefix."""
    import torch
    sysm, tables, run, cfg, arr = _corundum3600()
    T, n, seed = 512, 20000, 12345
    rng = np.random.default_rng(99)
    occ = np.stack([rng.choice(3600, size=4, replace=False) for _ in range(T)])
    eng = KmcEngine(tables)
    batch = KmcBatch(occ, step_capacity=n)
    # two chunks: resume from device state must not change anything
    eng.advance(batch, n // 2, eng.rng_struct(seed=seed))
    eng.advance(batch, n - n // 2, eng.rng_struct(seed=seed))
    torch.cuda.synchronize()
    assert (batch.step.cpu().numpy() == n).all()
    picks = rng.choice(T, size=8, replace=False)
    for t in picks:
        single = KmcBatch(occ[t:t + 1], step_capacity=n)
        eng.advance(single, n, eng.rng_struct(seed=seed, traj_offset=int(t)))
        torch.cuda.synchronize()
        assert np.array_equal(single.step_proc[0].cpu().numpy(),
                              batch.step_proc[t].cpu().numpy())
        assert np.array_equal(single.step_time[0].cpu().numpy(),
                              batch.step_time[t].cpu().numpy())
        assert np.array_equal(single.occ[0].cpu().numpy(), batch.occ[t].cpu().numpy())
    # oracle on a prefix of two sampled trajectories, same Philox stream
    A = tables.A.cpu().numpy()
    q_fixed = np.zeros(3600)
    q_fixed[cfg["dopants"]] = cfg["dopant_charge"]
    hop = sysm.hop_neighbor_list
    otab = ko.Tables(hop, "Fe:Fe", np.zeros(3600, int), 12, 0, 12,
                     sysm.material.lambda_values["Fe:Fe"], sysm.material.v_ab["Fe:Fe"])
    m = 1500
    for t in picks[:2]:
        u = np.array([v for s in range(m) for v in philox.step_uniforms(seed, int(t), s)])
        o = ko.run(A, otab, list(occ[t]), q_fixed, -1.0, np.zeros(3600),
                   sysm.material.vn, run.temp, u, run.time_interval,
                   tables.n_path_steps)
        assert np.array_equal(o["proc"], batch.step_proc[t, :m].cpu().numpy())
        assert np.abs(o["time"][1:] / batch.step_time[t, :m].cpu().numpy() - 1).max() \
            < TIME_RTOL


def test_device_philox_matches_host(cuda_ready):
    import torch
    out = torch.empty(2 * 64, dtype=torch.float64, device="cuda")
    nat.check(nat.lib().pycd_philox_uniforms(777, 5, 1000, 64, out.data_ptr(),
                                             nat.stream_handle()))
    torch.cuda.synchronize()
    ref = np.array([v for s in range(1000, 1064) for v in philox.step_uniforms(777, 5, s)])
    assert np.array_equal(out.cpu().numpy(), ref)


def test_zero_rates_stop_with_stalled_status(cuda_ready):
    """vn = 0 makes every rate 0: the kernel must report STALLED, not hang
    or index out of bounds (the reference raises IndexError here)."""
    import torch
    cfg, arr = gio.load("corundum324")
    tables, run = _corundum324_engine(cfg, arr)
    tables.vn = 0.0
    batch = KmcBatch([[5], [17]])
    eng = KmcEngine(tables)
    eng.advance(batch, 100, eng.rng_struct(seed=1))
    torch.cuda.synchronize()
    assert batch.status.cpu().tolist() == [nat.TRAJ_STALLED] * 2
    assert batch.step.cpu().tolist() == [0, 0]


def test_out_of_range_neighbour_stops_with_bad_index(cuda_ready):
    import torch
    cfg, arr = gio.load("corundum324")
    tables, run = _corundum324_engine(cfg, arr)
    tables.nbr[5, 2] = 10 ** 6  # a corrupt table entry, caught before any gather
    batch = KmcBatch([[5], [17]])
    eng = KmcEngine(tables)
    eng.advance(batch, 50, eng.rng_struct(seed=1))
    torch.cuda.synchronize()
    st = batch.status.cpu().tolist()
    assert st[0] == nat.TRAJ_BAD_INDEX
    assert st[1] in (nat.TRAJ_RUNNING, nat.TRAJ_BAD_INDEX)


def _ulp_diff(a, b):
    ia = a.view(np.int64)
    ib = b.view(np.int64)
    return np.abs(ia - ib)


def test_kernel_exp_within_ulps_of_cuda_and_libm(cuda_ready):
    """The kernels' table-driven exp against CUDA's exp and NumPy's exp on
    the range the rates use and across the whole finite range."""
    import torch
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.uniform(-80.0, 40.0, 400000),
                        rng.uniform(-745.0, 709.0, 200000),
                        np.array([0.0, -0.0, 1e-300, -1e-300, 709.78, -708.4, -744.9,
                                  -745.2, 709.8, 1.0, -1.0])])
    xd = torch.as_tensor(x).cuda()
    ours = torch.empty_like(xd)
    ref = torch.empty_like(xd)
    nat.check(nat.lib().pycd_debug_exp(xd.data_ptr(), len(x), ours.data_ptr(),
                                       ref.data_ptr(), nat.stream_handle()))
    torch.cuda.synchronize()
    o, r, h = ours.cpu().numpy(), ref.cpu().numpy(), np.exp(x)
    normal = np.isfinite(h) & (h > 2.3e-308)
    assert _ulp_diff(o[normal], r[normal]).max() <= 2
    assert _ulp_diff(o[normal], h[normal]).max() <= 2
    sub = (h > 0) & (h <= 2.3e-308)
    assert np.abs(o[sub] - h[sub]).max() <= 2 * 4.9e-324 or not sub.any()
    assert np.isinf(o[x >= 709.8]).all() and (o[x <= -745.2] == 0).all()


def test_kernel_exp_integer_path_edges(cuda_ready):
    """The integer-pipe exp (|x| < 704) at its internal edges: around
    |x| = 2^-13 (where the reduction starts), tiny and subnormal arguments,
    arguments half a step of ln2/4096 apart (the rounding of n), results
    whose 53-bit rounding carries into the exponent, and the switch to the
    FP64 form at |x| = 704.  Within 1 ulp of NumPy's exp (the kernels' exp is
    within ~0.502 ulp of exp(x))."""
    import math
    import torch
    rng = np.random.default_rng(11)
    step = math.log(2) / 4096
    k = rng.integers(-4_000_000, 4_000_000, 50000)
    x = np.concatenate([
        rng.uniform(-2.5e-4, 2.5e-4, 100000),
        np.array([s * np.ldexp(1.0, e) * (1 + 1e-9 * i) for s in (1, -1)
                        for e in range(-80, -9) for i in range(-3, 4)]),
        (k + 0.5) * step + rng.uniform(-1e-12, 1e-12, len(k)),
        # exp(x) just below a power of two (mantissa all ones before rounding)
        np.log(np.nextafter(np.ldexp(1.0, np.arange(-900, 1000, 7)), 0)),
        rng.uniform(703.0, 704.5, 20000), rng.uniform(-704.5, -703.0, 20000),
        np.array([5e-324, -5e-324, 2.2e-308, -2.2e-308, 2 ** -13, -2 ** -13,
                  np.nextafter(2 ** -13, 0), -np.nextafter(2 ** -13, 0), 703.99999999,
                  -703.99999999]),
    ])
    xd = torch.as_tensor(x).cuda()
    ours = torch.empty_like(xd)
    ref = torch.empty_like(xd)
    nat.check(nat.lib().pycd_debug_exp(xd.data_ptr(), len(x), ours.data_ptr(),
                                       ref.data_ptr(), nat.stream_handle()))
    torch.cuda.synchronize()
    o, h = ours.cpu().numpy(), np.exp(x)
    assert np.isfinite(o).all()
    assert _ulp_diff(o, h).max() <= 1


def test_event_stream_independent_of_launch_shape(cuda_ready):
    """Cumulative rates are balanced-tree sums over the process index, so
    the lanes-per-trajectory choice must not change any event or time."""
    import torch
    sysm, tables, run, cfg, arr = _corundum3600()
    T, n, seed = 64, 3000, 777
    rng = np.random.default_rng(5)
    occ = np.stack([rng.choice(3600, size=4, replace=False) for _ in range(T)])
    results = []
    shapes = [(4, 1), (8, 1), (8, 2), (16, 1), (16, 2), (32, 1), (32, 2), (64, 1),
              (128, 1)]
    for lanes, minb in shapes:  # minb 2: the 128-register variant; > 32: block form
        eng = KmcEngine(tables, launch={"lanes_per_traj": lanes,
                                        "min_blocks_per_sm": minb})
        b = KmcBatch(occ, step_capacity=n)
        eng.advance(b, n, eng.rng_struct(seed=seed))
        torch.cuda.synchronize()
        results.append((b.step_proc.cpu().numpy(), b.step_time.cpu().numpy(),
                        b.occ.cpu().numpy()))
    for r in results[1:]:
        assert np.array_equal(r[0], results[0][0])
        assert np.array_equal(r[1], results[0][1])
        assert np.array_equal(r[2], results[0][2])


def test_deferred_times_equal_exact_chain_across_shapes(cuda_ready):
    """The kernel defers the residence-time divisions (bounded in FP32, the
    exact FP64 chain at possible grid crossings and every G steps; a per-step
    time log is filled at each flush).  On a fine time grid (a crossing every
    ~50 steps) the rows, energies, final times and sites must be equal bit
    for bit for every launch shape, with and without a per-step log."""
    import torch
    cfg, arr = gio.load("corundum324")
    mat, nb = gio.material(cfg)
    sysm = System(mat, nb, gio.hop_list(cfg, arr), None, cfg["params"]["alpha"],
                  cfg["params"]["r_cut"], cfg["params"]["k_cut"])
    A = sysm.get_precomputed_array_device("fp64")
    tables, run = wl.batched_tables(sysm, A, 2, [], t_final=1e-9, time_interval=2e-12)
    rows = tables.n_path_steps
    rng = np.random.default_rng(3)
    occ = np.stack([rng.choice(324, size=2, replace=False) for _ in range(48)])

    def run_until_done(lanes, exact):
        eng = KmcEngine(tables, launch={"lanes_per_traj": lanes})
        b = KmcBatch(occ, unwrapped_rows=rows, energy_grid_rows=rows,
                     step_capacity=1 if exact else 0)
        for _ in range(100):
            eng.advance(b, 20000, eng.rng_struct(seed=31))
            if (b.status.cpu().numpy() == nat.TRAJ_DONE).all():
                break
        torch.cuda.synchronize()
        assert (b.status.cpu().numpy() == nat.TRAJ_DONE).all()
        return {k: getattr(b, k).cpu().numpy() for k in
                ("unwrapped", "energy_grid", "time", "occ", "step")}

    ref = run_until_done(8, exact=True)
    assert ref["step"].min() > 10 * rows  # many crossings per trajectory
    for lanes in (4, 8, 16, 32, 64, 128):  # 2 and 1 or 4 processes per lane
        got = run_until_done(lanes, exact=False)
        for k in ref:
            assert np.array_equal(got[k], ref[k]), (lanes, k)


@pytest.mark.parametrize("n_carriers", [16, 32])
def test_block_per_trajectory_equals_warp_form(cuda_ready, n_carriers):
    """One block of 2 or 4 warps per trajectory forms the same balanced trees
    as one warp (its warp totals are the top nodes of the process tree; its
    rebuild sums are the same carrier trees), so events, times, sites,
    energies, displacements and the stored carrier sums must equal the warp
    form's bit for bit, across a chunk boundary off the refresh period."""
    import torch
    sysm, tables, run, cfg, arr = _corundum3600(n_carriers)
    T, n, seed = 24, 2000, 4242
    rng = np.random.default_rng(11)
    occ = np.stack([rng.choice(3600, size=n_carriers, replace=False) for _ in range(T)])
    shapes = (16, 32, 64, 128) if n_carriers == 16 else (32, 64, 128)
    keys = ("step_proc", "step_time", "occ", "csum", "energy", "disp", "time")
    results = []
    for lanes in shapes:
        eng = KmcEngine(tables, launch={"lanes_per_traj": lanes})
        b = KmcBatch(occ, step_capacity=n)
        eng.advance(b, n // 3, eng.rng_struct(seed=seed))
        eng.advance(b, n - n // 3, eng.rng_struct(seed=seed))
        torch.cuda.synchronize()
        assert (b.step.cpu().numpy() == n).all(), lanes
        results.append({k: getattr(b, k).cpu().numpy() for k in keys})
    for lanes, r in zip(shapes[1:], results[1:]):
        for k in keys:
            assert np.array_equal(r[k], results[0][k]), (lanes, k)


def test_block_form_matches_oracle_with_32_carriers(cuda_ready):
    """A 32-carrier trajectory (128 processes) in the 4-warp block form
    against the oracle fed the same Philox uniforms: identical events,
    times within 1e-12 relative."""
    import torch
    sysm, tables, run, cfg, arr = _corundum3600(32)
    seed, m = 2024, 600
    occ0 = np.random.default_rng(21).choice(3600, size=32, replace=False)
    eng = KmcEngine(tables, launch={"lanes_per_traj": 128})
    b = KmcBatch(occ0[None], step_capacity=m)
    eng.advance(b, m, eng.rng_struct(seed=seed))
    torch.cuda.synchronize()
    assert int(b.step.item()) == m
    A = tables.A.cpu().numpy()
    q_fixed = np.zeros(3600)
    q_fixed[cfg["dopants"]] = cfg["dopant_charge"]
    otab = ko.Tables(sysm.hop_neighbor_list, "Fe:Fe", np.zeros(3600, int), 12, 0, 12,
                     sysm.material.lambda_values["Fe:Fe"], sysm.material.v_ab["Fe:Fe"])
    u = np.array([v for s in range(m) for v in philox.step_uniforms(seed, 0, s)])
    o = ko.run(A, otab, list(occ0), q_fixed, -1.0, np.zeros(3600), sysm.material.vn,
               run.temp, u, run.time_interval, tables.n_path_steps)
    assert np.array_equal(o["proc"], b.step_proc[0, :m].cpu().numpy())
    assert np.abs(o["time"][1:] / b.step_time[0, :m].cpu().numpy() - 1).max() < TIME_RTOL


def test_fourteen_slots_two_rebuild_rounds(cuda_ready):
    """Five corundum hop shells give 14 hop slots per carrier; 12 carriers
    give 168 processes.  The moved carrier's 15 rebuild jobs take two rounds
    in the warp form's many-carrier rebuild and in the block form, whose
    neighbour cache covers at most 4 slots (so it reads the neighbour table
    here).  Events, times and sites must agree across the forms, and the
    events with the oracle's."""
    import torch
    sysm = wl.corundum((3, 3, 3), shells=(2.90, 2.97, 3.364, 3.705, 3.986))
    A = sysm.get_precomputed_array_device("fp64")
    tables, run = wl.batched_tables(sysm, A, 12, [], 1.0, t_final=1e30, time_interval=1e27)
    assert tables.n_slots == 14
    T, n, seed = 4, 400, 515
    rng = np.random.default_rng(17)
    occ = np.stack([rng.choice(324, size=12, replace=False) for _ in range(T)])
    results = []
    for lanes in (32, 64, 128):
        eng = KmcEngine(tables, launch={"lanes_per_traj": lanes})
        b = KmcBatch(occ, step_capacity=n)
        eng.advance(b, n, eng.rng_struct(seed=seed))
        torch.cuda.synchronize()
        assert (b.step.cpu().numpy() == n).all(), lanes
        results.append((b.step_proc.cpu().numpy(), b.step_time.cpu().numpy(),
                        b.occ.cpu().numpy()))
    for r in results[1:]:
        for x, y in zip(r, results[0]):
            assert np.array_equal(x, y)
    m = sysm.material
    otab = ko.Tables(sysm.hop_neighbor_list, "Fe:Fe", np.zeros(324, int), 12, 0, 12,
                     m.lambda_values["Fe:Fe"], m.v_ab["Fe:Fe"])
    k = 300
    u = np.array([v for s in range(k) for v in philox.step_uniforms(seed, 0, s)])
    o = ko.run(A.cpu().numpy(), otab, list(occ[0]), np.zeros(324), -1.0, np.zeros(324),
               m.vn, run.temp, u, run.time_interval, tables.n_path_steps)
    assert o["steps"] == k
    assert np.array_equal(o["proc"], results[0][0][0, :k])
    assert np.abs(o["time"][1:] / results[0][1][0, :k] - 1).max() < TIME_RTOL


def test_field_drift_and_delg0_grid(cuda_ready):
    """An electric field shifts each rate by 0.5 E.hop (core.py:2041-2047).
    Events and the dG0 path grid (core.py:2806-2808) against the oracle; the
    drift sums (hop x rate of each event, core.py:2821-2824), the grids and
    the times equal across the warp and block forms."""
    import torch
    sysm = wl.corundum((3, 3, 3))
    A = sysm.get_precomputed_array_device("fp64")
    field = {"electric": {"active": 1, "dir": [1, 0, 0], "ld": 0, "mag": 5e-5}}
    run = Run(sysm, None, 300, "full", "full", 1, 5e-11, 1e-13, np.array([2]),
              {"electron": []}, {"class_index": {}, "doping": {}}, field,
              {"num_dopants": [0]})
    assert run.site_field_shift is not None and np.abs(run.site_field_shift).max() > 0
    n_path = int(run.t_final / run.time_interval) + 1
    q = run.base_charge_config()[:, 0].copy()
    tables = KmcTables(A, run.site_nbr, run.site_hop, run.site_lam, run.site_vab,
                       run.system_relative_energies, q, run.carrier_charge, 2,
                       run.material.vn, run.temp, run.time_interval, n_path,
                       field_shift=run.site_field_shift)
    T, n, seed = 4, 400, 808
    rng = np.random.default_rng(23)
    occ = np.stack([rng.choice(324, size=2, replace=False) for _ in range(T)])
    keys = ("step_proc", "step_time", "delg0_grid", "drift", "occ", "time")
    results = []
    for lanes in (8, 16, 64, 128):
        eng = KmcEngine(tables, launch={"lanes_per_traj": lanes})
        b = KmcBatch(occ, step_capacity=n, delg0_grid_rows=n_path, drift=True)
        eng.advance(b, n, eng.rng_struct(seed=seed))
        torch.cuda.synchronize()
        assert (b.step.cpu().numpy() == n).all(), lanes
        results.append({k: getattr(b, k).cpu().numpy() for k in keys})
    for r in results[1:]:
        for k in keys:
            assert np.array_equal(r[k], results[0][k]), k
    assert np.abs(results[0]["drift"]).max() > 0
    m = sysm.material
    otab = ko.Tables(sysm.hop_neighbor_list, "Fe:Fe", np.zeros(324, int), 12, 0, 12,
                     m.lambda_values["Fe:Fe"], m.v_ab["Fe:Fe"], field=run.electric_field)
    k = 300
    u = np.array([v for s in range(k) for v in philox.step_uniforms(seed, 0, s)])
    o = ko.run(A.cpu().numpy(), otab, list(occ[0]), q, run.carrier_charge,
               run.system_relative_energies, m.vn, run.temp, u, run.time_interval, n_path)
    assert o["steps"] == k
    assert np.array_equal(o["proc"], results[0]["step_proc"][0, :k])
    assert np.abs(o["time"][1:] / results[0]["step_time"][0, :k] - 1).max() < TIME_RTOL
    rows = np.nonzero(o["delg0"])[0]
    assert len(rows) > 3  # several grid crossings within the oracle's steps
    got = results[0]["delg0_grid"][0, rows]
    assert np.abs(got - o["delg0"][rows]).max() <= 1e-12 * np.abs(o["delg0"][rows]).max()


def _state(b):
    return {k: getattr(b, k).cpu().numpy().copy()
            for k in ("occ", "time", "step", "disp", "last_row", "energy", "csum")}


@pytest.mark.parametrize("lanes", [8, 64])
def test_time_limit_stops_and_resumes_with_the_same_events(cuda_ready, lanes):
    """A per-launch time limit stops every trajectory with TRAJ_TIMEOUT
    before its step budget; relaunching the stopped trajectories (status set
    back to RUNNING) until the budget is done gives the state of one
    uninterrupted launch bit for bit, in the warp form (8 lanes) and the
    block form (64 lanes)."""
    import torch
    sysm, tables, run, cfg, arr = _corundum3600()
    T, n = 32, 60000
    rng = np.random.default_rng(11)
    occ = np.stack([rng.choice(3600, size=4, replace=False) for _ in range(T)])
    eng = KmcEngine(tables, launch={"lanes_per_traj": lanes})
    ref = KmcBatch(occ, step_limit=n)
    eng.advance(ref, n, eng.rng_struct(seed=5))
    torch.cuda.synchronize()
    b = KmcBatch(occ, step_limit=n)
    b.time_limit_ns = 2_000_000  # 2 ms per launch
    b.poll_interval = 64
    launches, stopped = 0, 0
    while True:
        eng.advance(b, n, eng.rng_struct(seed=5))
        torch.cuda.synchronize()
        launches += 1
        st = b.status.cpu().numpy()
        stopped += int((st == nat.TRAJ_TIMEOUT).sum())
        if not (st == nat.TRAJ_TIMEOUT).any():
            break
        b.status[torch.as_tensor(st == nat.TRAJ_TIMEOUT, device=b.status.device)] = \
            nat.TRAJ_RUNNING
        assert launches < 10000
    assert launches > 1 and stopped > 0
    assert (b.step.cpu().numpy() == n).all()
    got, want = _state(b), _state(ref)
    for k in want:
        assert np.array_equal(got[k], want[k]), k


@pytest.mark.parametrize("lanes", [8, 64])
def test_cancel_flag_stops_one_trajectory_during_a_launch(cuda_ready, lanes):
    """The host raises one trajectory's cancel flag (pinned host memory)
    while a long launch runs: that trajectory stops with TRAJ_CANCELLED
    part-way, the others finish their budget, and the cancelled one's state
    equals the same trajectory advanced alone by the same number of steps."""
    import time
    import torch
    sysm, tables, run, cfg, arr = _corundum3600()
    T, n, victim = 16, 400000, 5
    rng = np.random.default_rng(12)
    occ = np.stack([rng.choice(3600, size=4, replace=False) for _ in range(T)])
    eng = KmcEngine(tables, launch={"lanes_per_traj": lanes})
    warm = KmcBatch(occ, step_limit=100)  # kernel loaded before the timed launch
    eng.advance(warm, 100, eng.rng_struct(seed=9))
    torch.cuda.synchronize()
    b = KmcBatch(occ, step_limit=n, cancellable=True)
    b.poll_interval = 128
    eng.advance(b, n, eng.rng_struct(seed=9))
    time.sleep(0.05)
    b.request_stop(victim)
    torch.cuda.synchronize()
    st, steps = b.status.cpu().numpy(), b.step.cpu().numpy()
    assert st[victim] == nat.TRAJ_CANCELLED
    assert 0 < steps[victim] < n
    others = np.arange(T) != victim
    assert (steps[others] == n).all()
    alone = KmcBatch(occ[victim:victim + 1], step_limit=int(steps[victim]))
    eng.advance(alone, n, eng.rng_struct(seed=9, traj_offset=victim))
    torch.cuda.synchronize()
    got, want = _state(b), _state(alone)
    for k in ("occ", "time", "step", "disp", "last_row", "energy"):
        assert np.array_equal(got[k][victim], want[k][0]), k
    # a cleared flag lets the trajectory go on
    b.request_stop(victim, False)
    b.status[victim] = nat.TRAJ_RUNNING
    eng.advance(b, n, eng.rng_struct(seed=9))
    torch.cuda.synchronize()
    assert b.step[victim].item() == n


@pytest.mark.parametrize("lanes,T", [(8, 600), (8, 16384), (4, 2000), (16, 3000)])
def test_queue_form_equals_static_form(cuda_ready, lanes, T):
    """The queue form (rounds of 128 steps handed to free warps, more sets
    than warps for T = 16,384) gives the static form's events, times and
    state bit for bit, with step budgets that end inside rounds, and no
    wait of the queue runs out."""
    import torch
    sysm, tables, run, cfg, arr = _corundum3600()
    n = 1500
    rng = np.random.default_rng(T + lanes)
    occ = np.stack([rng.choice(3600, size=4, replace=False) for _ in range(T)])
    limits = rng.integers(200, n + 1, T)
    out = []
    for sched in (0, 128):
        eng = KmcEngine(tables, launch={"lanes_per_traj": lanes}).schedule(sched)
        b = KmcBatch(occ, step_limit=limits, step_capacity=n)
        eng.advance(b, n, eng.rng_struct(seed=41))
        torch.cuda.synchronize()
        if sched:
            assert eng._sched[2].item() == 0
            assert eng._sched[0].item() >= eng._sched[1].item()
        st = _state(b)
        st["status"] = b.status.cpu().numpy()
        st["proc"] = b.step_proc.cpu().numpy()
        st["tlog"] = b.step_time.cpu().numpy()
        out.append(st)
    assert (out[0]["step"] == limits).all()
    for k in out[0]:
        assert np.array_equal(out[0][k], out[1][k]), k
