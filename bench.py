#!/usr/bin/env python
"""Benchmark: batched lattice KMC on one GB300 (steps/s aggregate).

Workload (per GPU): corundum 10x10x3 = 3,600 sites, 4 electrons and 4 fixed
+1 dopants on seeded sites, FP64 Ewald array (103.7 MB) built on the GPU,
4,096 trajectories with per-trajectory Philox streams.  One bench step = one
CUDA-graph launch of the persistent kernel advancing every trajectory by
10,000 KMC steps (100 such chunks = the 1e6-step job).

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]

Prints one JSON line (rank 0).  ``value`` is device-timed with inputs
resident; ``e2e`` runs the job through the host-buffer entry point
(``pycd_gb300.batch.run_batched``) with the array and tables copied from
pinned host memory and the final state copied back inside the timed region.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N_CELLS = (10, 10, 3)
N_TRAJ = 4096
N_CARRIERS, N_DOPANTS, Z = 4, 4, 4
CHUNK = 10000
# algorithmic bytes per KMC step: 8 n_c (z+1)(n_c+n_d) Ewald entries plus
# 16 n_c (z+1) for E_rel and phi_bg
B_STEP = 8 * N_CARRIERS * (Z + 1) * (N_CARRIERS + N_DOPANTS) + 16 * N_CARRIERS * (Z + 1)
T_FINAL, DT = 1e30, 1e27  # time grid wide enough that no trajectory ends by time
SEED = 20251203
# queue form of the warp-form launch: rounds of this many steps (0 = static)
SCHED_STEPS = 0
# FP64 thread instructions per KMC step on this workload, by launch shape
# (lanes per trajectory, register variant): ncu
# smsp__sass_thread_inst_executed_op_{dadd,dfma,dmul}_pred_on summed over one
# 1,000-step chunk launch, divided by its 4.096e6 KMC steps.  The autotuner
# picks (16, 2), i.e. kmc_advance_kernel<16, 1, 2>; with 8 lanes the step's
# shared FP64 work is repeated on fewer lanes.
FP64_INSTR_PER_STEP = {(16, 2): 428, (8, 1): 280}
# DRAM bytes per KMC step of kmc_advance_kernel<16, 1, 2> (ncu:
# dram__bytes_read.sum + dram__bytes_write.sum of one 10,000-step chunk launch
# of this workload, 7,420,928 + 3,072 bytes, divided by its 4.096e7 KMC steps)
DRAM_BYTES_PER_STEP = (7420928 + 3072) / 40960000


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d["hbm_gbs"], "measured"
    return 6800.0, "fallback"


class ClockSampler(object):
    """nvidia-smi samples of SM clock and throttle reasons while running."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index, self.rows, self.proc = index, [], None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([v.strip() for v in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4)
                          if len(r) > 4 + i and r[4 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


def fp64_peak_tflops(n=4096, reps=3):
    """Measured FP64 peak of this GPU: cuBLAS DGEMM n^3 (2 n^3 flops), best of
    `reps` after a warm-up, timed with CUDA events."""
    import torch
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = None
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        best = ms if best is None else min(best, ms)
    del a, b
    return 2.0 * n ** 3 / (best / 1e3) / 1e12


def build_workload(rank=0, n_traj=N_TRAJ):
    """System, device array, tables and initial carrier sites."""
    import torch
    from pycd_gb300 import workloads as wl
    system = wl.corundum(N_CELLS)
    A = system.get_precomputed_array_device("fp64")
    carriers0, dopants = wl.batched_uniform_sites(seed=3600)
    tables, run = wl.batched_tables(system, A, N_CARRIERS, dopants, 1.0,
                                    t_final=T_FINAL, time_interval=DT)
    rng = np.random.default_rng(SEED + rank)
    free = np.setdiff1d(np.arange(3600), dopants)
    occ = np.stack([rng.choice(free, size=N_CARRIERS, replace=False)
                    for _ in range(n_traj)]).astype(np.int32)
    torch.cuda.synchronize()
    return system, A, tables, run, dopants, occ


def time_plain(tables, occ, n_steps=20000):
    """The plain form: one trajectory advanced alone by the same kernel, at
    the fastest lane count for a single trajectory."""
    import torch
    from pycd_gb300.kmc import KmcBatch, KmcEngine
    best = 0.0
    for lanes in (4, 8, 16, 32, 64, 128):  # 64, 128: one block of 2 or 4 warps
        eng = KmcEngine(tables, launch={"lanes_per_traj": lanes})
        b = KmcBatch(occ[:1])
        eng.advance(b, 2000, eng.rng_struct(seed=SEED))
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        eng.advance(b, n_steps, eng.rng_struct(seed=SEED))
        e1.record()
        torch.cuda.synchronize()
        best = max(best, n_steps / (e0.elapsed_time(e1) / 1e3))
    return best


def cpu_port_steps(args):
    """Oracle port (the reference's algorithm, NumPy) on one trajectory;
    returns steps done and seconds."""
    a_path, tab_path, occ, n_steps, seed = args
    sys.path.insert(0, str(ROOT))
    import pickle
    from oracle import kmc_oracle as ko
    from oracle import philox
    A = np.load(a_path, mmap_mode="r")
    with open(tab_path, "rb") as fh:
        t = pickle.load(fh)
    u = np.array([v for s in range(n_steps) for v in philox.step_uniforms(seed, 0, s)])
    t0 = time.perf_counter()
    o = ko.run(A, t["tables"], list(occ), t["q_fixed"], -1.0, t["e_rel"], t["vn"],
               t["kT"], u, t["dt"], t["n_path"], max_steps=n_steps)
    return o["steps"], time.perf_counter() - t0


def write_cpu_inputs(system, run, dopants, tmpdir):
    """Oracle-side inputs: the oracle's own array (translation classes) and
    the oracle's process tables over the hop-neighbour list."""
    import pickle
    from oracle import ewald_oracle as eo
    from oracle import kmc_oracle as ko
    m = system.material
    A = eo.class_array(m.cartesian_unit_cell_coords, m.lattice_matrix, N_CELLS,
                       system.alpha, system.r_cut, system.k_cut,
                       m.dielectric_constant)
    a_path = Path(tmpdir) / "A.npy"
    np.save(a_path, A)
    q = np.zeros(3600)
    q[dopants] = 1.0
    tab = {"tables": ko.Tables(system.hop_neighbor_list, "Fe:Fe", np.zeros(3600, int),
                               12, 0, 12, m.lambda_values["Fe:Fe"], m.v_ab["Fe:Fe"]),
           "q_fixed": q, "e_rel": np.zeros(3600), "vn": m.vn, "kT": run.temp,
           "dt": run.time_interval, "n_path": int(run.t_final / run.time_interval) + 1}
    tab_path = Path(tmpdir) / "tables.pkl"
    with open(tab_path, "wb") as fh:
        pickle.dump(tab, fh)
    return str(a_path), str(tab_path)


def batched_config(args, world):
    """The workload both arms report (the reference arm times a sample of it,
    described in its cpu_baseline)."""
    return {"workload": "batched uniform: corundum 10x10x3 = 3,600 sites, "
                        "4 electrons + 4 fixed +1 dopants, FP64 Ewald array "
                        "(103.7 MB), Philox streams",
            "trajectories_per_gpu": args.traj, "steps_per_chunk": args.chunk,
            "chunk": "one CUDA-graph launch of the persistent kernel",
            "l2": "256 MiB buffer written between timed chunks",
            "parallelism": f"replicas x{world}"}


def reference_arm(args):
    """--impl reference: the reference's algorithm (oracle port) on all host
    cores, one trajectory per process as the reference's 'parallel' mode."""
    import multiprocessing as mp
    import tempfile
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from pycd_gb300 import workloads as wl
    system = wl.corundum(N_CELLS)
    run = wl.run_for(system, N_CARRIERS, T_FINAL, DT)
    _, dopants = wl.batched_uniform_sites(seed=3600)
    tmp = tempfile.mkdtemp()
    a_path, tab_path = write_cpu_inputs(system, run, dopants, tmp)
    cores = os.cpu_count() or 1
    rng = np.random.default_rng(SEED)
    free = np.setdiff1d(np.arange(3600), dopants)
    ctx = mp.get_context("spawn")
    budget = 150.0 / max(1, args.steps + args.warmup)  # seconds per bench step
    with ctx.Pool(cores) as pool:
        # calibrate the per-step sample so the whole run stays within minutes
        jobs = [(a_path, tab_path, rng.choice(free, N_CARRIERS, replace=False),
                 200, SEED + i) for i in range(cores)]
        res = pool.map(cpu_port_steps, jobs)
        per_step = max(r[1] / r[0] for r in res)
        m = max(50, int(0.8 * budget / per_step))
        total_steps, total_s = 0, 0.0
        for it in range(args.warmup + args.steps):
            jobs = [(a_path, tab_path, rng.choice(free, N_CARRIERS, replace=False),
                     m, SEED + 1000 * it + i) for i in range(cores)]
            t0 = time.perf_counter()
            res = pool.map(cpu_port_steps, jobs)
            dt = time.perf_counter() - t0
            if it >= args.warmup:
                total_steps += sum(r[0] for r in res)
                total_s += dt
    value = total_steps / total_s
    line = {"metric": "KMC steps/s (batched uniform, 3,600 sites, 4 e- + 4 dopants)",
            "value": value, "unit": "steps/s", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * total_s / max(1, args.steps),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": batched_config(args, int(os.environ.get("WORLD_SIZE", "1"))),
            "cpu_baseline": {"value": value, "unit": "steps/s", "cores": cores,
                             "kind": "port",
                             "sample": f"{cores} trajectories x {m} steps per bench "
                                       f"step, {args.steps} timed steps"},
            "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def cpu_baseline_1core(system, run, dopants, occ, seconds=10.0):
    import tempfile
    tmp = tempfile.mkdtemp()
    a_path, tab_path = write_cpu_inputs(system, run, dopants, tmp)
    s, t = cpu_port_steps((a_path, tab_path, occ[0], 200, SEED))
    n = max(200, int(seconds * s / t))
    s, t = cpu_port_steps((a_path, tab_path, occ[1], n, SEED + 1))
    return {"value": s / t, "unit": "steps/s", "cores": 1, "kind": "port",
            "sample": f"1 trajectory x {s} KMC steps of this workload, NumPy port "
                      "of the reference loop"}


# monoclinic supercells and the k_cut (1/A) that keeps K = 4,096 / 8,192 / 16,384
# half-space k-vectors with k^2 < k_cut^2
EWALD_SIZES = {8192: ((16, 16, 8), (0.9164, 1.1515, 1.4516)),
               16384: ((16, 16, 16), (0.7244, 0.9156, 1.1525)),
               32768: ((16, 16, 32), (0.5765, 0.7257, 0.9150))}


def cpu_fourier_ns_per_entry_k(system, rows=48, n_k=24):
    """The reference's pot_k_ewald arithmetic (oracle) on a row and k subset:
    seconds per (array entry x k-vector), to extrapolate a full build."""
    from oracle import ewald_oracle as eo
    coords = system.neighbors.bulk_sites.cell_coordinates
    n = len(coords)
    idx = np.arange(rows)
    d = coords[None, :, :] - coords[idx, None, :]
    pmiv = system.neighbors.apply_minimum_image_convention_vectorized(
        d.reshape(-1, 3)).reshape(rows, n, 3)
    kv = eo.effective_k_vectors(eo.k_max_for(system.k_cut,
                                             system.reciprocal_lattice_matrix))
    kv = kv[:n_k]
    out = np.zeros((rows, n))
    t0 = time.perf_counter()
    for v in kv:
        k = np.dot(v, system.reciprocal_lattice_matrix)
        k2 = np.dot(k, k)
        out += ((2 * np.pi) / system.system_volume * np.exp(-k2 / (4 * system.alpha))
                * np.cos(np.tensordot(pmiv, k, axes=([2], [0]))) / k2)
    dt = time.perf_counter() - t0
    return dt / (rows * n * len(kv))


def ewald_split_record(n, kk, kc, modes=("fp64", "bf16x3", "tf32x3"), cpu=True):
    """One (N, K) point of the split-precision build: FP64 feature build and
    the BF16x3 / TF32x3 tcgen05 builds timed end to end (best of 3 after a
    warm-up), their max / RMS error in eV against the FP64 array, and the
    error of the hop energy dE0 over sampled 16-carrier, 16-dopant
    configurations as a fraction of kT (300 K)."""
    import torch
    from pycd_gb300 import autotune
    from pycd_gb300 import constants as K
    from pycd_gb300 import ewald as ew
    from pycd_gb300 import workloads as wl
    peaks_file = ROOT / "MEASURED_PEAKS.json"
    bf16_peak = json.loads(peaks_file.read_text())["bf16_tflops"] if peaks_file.exists() else 1900.0
    cells = EWALD_SIZES[n][0]
    system = wl.monoclinic(cells, kc, neighbor_list=True)
    run1 = wl.run_for(system, 1)
    kT, nbr = run1.temp, run1.site_nbr
    line = {"workload": "ewald-split", "n_sites": n, "cells": list(cells),
            "k_cut_per_angstrom": kc, "k_target": kk}
    times = {}
    ref = None
    for mode in modes:
        reps = 1 if mode == "fp64" else 3
        if mode != "fp64":
            # launch shape of the tcgen05 contraction (untimed; same array)
            tuned = autotune.tune_split(system, mode, reps=1)
            times.setdefault("launch_shapes", {})[mode] = tuned["best"]
        system.get_precomputed_array_device(mode)  # warm-up / workspace
        torch.cuda.synchronize()
        best = None
        for _ in range(reps):
            t0 = time.perf_counter()
            A = system.get_precomputed_array_device(mode)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            best = dt if best is None else min(best, dt)
        info = system.last_build_info
        times[mode] = {"build_ms": 1e3 * best, "fourier_ms": info["fourier_ms"],
                       "real_ms": info["real_ms"]}
        line["n_kvec"] = info["n_kvec"]
        if mode == "fp64":
            ref = A
        elif ref is not None:
            err = (A - ref).abs()
            times[mode]["max_err_ev"] = err.max().item() / K.EV2HARTREE
            times[mode]["rms_err_ev"] = err.square().mean().sqrt().item() / K.EV2HARTREE
            del err
            de_max, de_rms = ew.hop_energy_error(ref, A, nbr, 16, 16, samples=2048, seed=1)
            times[mode]["dE_max_err_over_kT"] = de_max / kT
            times[mode]["dE_rms_err_over_kT"] = de_rms / kT
        if mode != "fp64":
            del A
    line["split_launch"] = times.pop("launch_shapes", {})
    kn = line["n_kvec"]
    flops = 4.0 * n * n * kn  # N x 2K by 2K x N
    for mode in modes:
        t = times[mode]
        t["algorithmic_tflops"] = flops / (t["fourier_ms"] / 1e3) / 1e12
        if mode != "fp64":
            if "fp64" in times:
                t["speedup_vs_fp64"] = times["fp64"]["build_ms"] / t["build_ms"]
            t["tensor_peak_tflops"] = bf16_peak if mode == "bf16x3" else bf16_peak / 2
    line["modes"] = times
    line["algorithmic_flops"] = "4 N^2 K (N x 2K features times their transpose)"
    del ref
    torch.cuda.empty_cache()
    if cpu:
        ns = cpu_fourier_ns_per_entry_k(system)
        line["cpu_reference_fourier"] = {
            "s_per_entry_k": ns, "extrapolated_build_s": ns * n * n * kn,
            "cores": 1, "kind": "port",
            "sample": "48 rows x all N columns x 24 k-vectors of pot_k_ewald"}
    return line


def ewald_split_bench(args):
    """Split-precision (BF16x3 / TF32x3 tcgen05) vs FP64 GPU Ewald build on
    the monoclinic supercells; one JSON line per (N, K)."""
    import torch
    from pycd_gb300 import _native as nat
    torch.cuda.set_device(0)
    nat.require_device()
    sizes = [int(s) for s in args.sizes.split(",")] if args.sizes else sorted(EWALD_SIZES)
    ks = [int(k) for k in args.kvecs.split(",")] if args.kvecs else [4096, 8192, 16384]
    for n in sizes:
        for kk, kc in zip((4096, 8192, 16384), EWALD_SIZES[n][1]):
            if kk in ks:
                print(json.dumps(ewald_split_record(n, kk, kc, cpu=not args.no_cpu_baseline)),
                      flush=True)


def _lattice_tables(cache, lattice, cells, precision):
    from pycd_gb300 import workloads as wl
    key = (lattice, tuple(cells), precision)
    if key not in cache:
        system = wl.system_for(lattice, cells)
        A = system.get_precomputed_array_device(precision)
        base, _ = wl.batched_tables(system, A, 1, [], 1.0, T_FINAL, DT)
        base.share_rate_coefficients()
        cache[key] = (system, base)
    return cache[key]


def _job_occupancy(n_sites, n_carriers, dopants, seed, width):
    free = np.setdiff1d(np.arange(n_sites), dopants)
    occ = np.zeros(width, np.int32)
    occ[:n_carriers] = np.random.default_rng(seed).choice(free, n_carriers, replace=False)
    return occ


def diffusivity(disp, t):
    """D = <|dr|^2> / (6 t) per carrier (Einstein relation at the end of
    each trajectory); returns mean and standard error over carriers."""
    r2 = (disp ** 2).sum(-1)
    d = (r2 / (6.0 * t[:, None])).ravel()
    return float(d.mean()), float(d.std(ddof=1) / np.sqrt(len(d)))


def uneven_bench(args):
    """64 systems of both lattices (300-20,000 sites), 2,048 trajectories with
    1-16 carriers, 0-16 dopants and 1e4-1e6 steps, split-precision arrays,
    bucketed autotuned launches; plus FP64-vs-split diffusivity checks."""
    import torch
    from pycd_gb300 import _native as nat
    from pycd_gb300 import constants as K
    from pycd_gb300 import workloads as wl
    from pycd_gb300.batch import BatchedKmc
    torch.cuda.set_device(0)
    nat.require_device()
    specs, traj_sys, steps = wl.uneven_systems()
    cache, tables = {}, []
    t0 = time.perf_counter()
    for spec in specs:
        system, base = _lattice_tables(cache, spec["lattice"], spec["cells"], "bf16x3")
        n = system.neighbors.num_system_elements
        _, dop = wl.sites_for(n, spec["carriers"], spec["dopants"], spec["seed"])
        q = np.zeros(n)
        q[dop] = 1.0
        tables.append(base.with_charges(q, spec["carriers"]))
        spec["n_sites"], spec["dopant_sites"] = n, dop
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    occ = np.stack([_job_occupancy(specs[s]["n_sites"], specs[s]["carriers"],
                                   specs[s]["dopant_sites"], 7000 + i, 16)
                    for i, s in enumerate(traj_sys)])
    bk = BatchedKmc(tables, occ, sys_index=traj_sys, seed=SEED, chunk_steps=args.chunk,
                    step_limit=steps, autotune=True)
    tuned = [(bkt.engine.launch.lanes_per_traj, bkt.engine.launch.warps_per_block,
              bkt.engine.launch.min_blocks_per_sm, len(bkt.idx)) for bkt in bk.buckets]
    torch.cuda.synchronize()
    with ClockSampler(0) as clocks:
        t0 = time.perf_counter()
        chunks = 0
        while True:
            bk.step_chunk()
            chunks += 1
            if chunks % 10 == 0 or chunks * args.chunk >= int(steps.max()):
                torch.cuda.synchronize()
                st = bk.status_counts()
                if st.get(nat.TRAJ_RUNNING, 0) == 0:
                    break
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    total = bk.steps_done()
    arrays_gb = sum(8.0 * s["n_sites"] ** 2 for s in specs) / 1e9
    # diffusivity: FP64 vs split arrays on the six smallest lattices, no dopants
    checks = []
    small = sorted({(s["lattice"], tuple(s["cells"]), s["n_sites"]) for s in specs},
                   key=lambda x: x[2])[:6]
    for lattice, cells, n in small:
        res = {}
        for prec in ("fp64", "bf16x3"):
            system, base = _lattice_tables(cache, lattice, cells, prec)
            tab = base.with_charges(np.zeros(n), 4)
            o = np.stack([_job_occupancy(n, 4, [], 9000 + i, 4) for i in range(256)])
            b2 = BatchedKmc(tab, o, seed=SEED + 1, chunk_steps=20000, step_limit=100000)
            b2.run(100000)
            torch.cuda.synchronize()
            disp = (b2.batch.last_row + b2.batch.disp).cpu().numpy().reshape(256, 4, 3)
            t = b2.batch.time.cpu().numpy()
            res[prec] = diffusivity(disp, t)
        d64, s64 = res["fp64"]
        ds, ss = res["bf16x3"]
        checks.append({"lattice": lattice, "n_sites": n, "D_fp64": d64, "sem_fp64": s64,
                       "D_split": ds, "sem_split": ss,
                       "z": abs(d64 - ds) / max(1e-300, np.hypot(s64, ss))})
    line = {"workload": "batched uneven", "metric": "KMC steps/s (uneven batch)",
            "value": total / wall, "unit": "steps/s", "steps": int(total),
            "wall_s": wall, "systems": len(specs), "trajectories": int(len(traj_sys)),
            "site_range": [int(min(s["n_sites"] for s in specs)),
                           int(max(s["n_sites"] for s in specs))],
            "arrays_gb": arrays_gb, "setup_s": setup_s, "chunk_steps": args.chunk,
            "buckets_lanes_warps_minblocks_trajs": tuned, "status_counts": bk.status_counts(),
            "diffusivity_fp64_vs_split": checks, "clocks": clocks.summary()}
    print(json.dumps(line), flush=True)


def serving_record(args):
    """Poisson arrivals (200 jobs/s) of single-trajectory KMC jobs over both
    lattices; continuous batching; p50/p99 latency and aggregate steps/s;
    a sample of jobs re-run alone must give identical results."""
    import torch
    from pycd_gb300 import _native as nat
    from pycd_gb300.batch import BatchedKmc
    from pycd_gb300.serving import KmcServer, poisson_jobs
    jobs = poisson_jobs(args.jobs, rate=200.0, seed=11, max_steps=args.max_job_steps)
    server = KmcServer(budget_bytes=150e9, chunk_steps=args.chunk, precision="bf16x3",
                       seed=SEED)
    t0 = time.perf_counter()
    keys = sorted({(j["lattice"], tuple(j["cells"])) for j in jobs},
                  key=lambda k: np.prod(k[1]))
    for i, k in enumerate(keys):  # warm the lattice cache (arrays are shared)
        server.cache.get(*k)
        if i % 8 == 0:
            print(f"[serving] lattice {i + 1}/{len(keys)} {k} "
                  f"{time.perf_counter() - t0:.1f}s", file=sys.stderr, flush=True)
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    warm_s = time.perf_counter() - t0
    print(f"[serving] cache warm in {warm_s:.1f}s, {server.cache.bytes_in_use() / 1e9:.1f} GB",
          file=sys.stderr, flush=True)
    t0 = time.perf_counter()
    n_warm = server.warm_up(jobs)  # one short job per carrier class, discarded
    warm_jobs_s = time.perf_counter() - t0
    print(f"[serving] {n_warm} warm-up jobs in {warm_jobs_s:.1f}s", file=sys.stderr, flush=True)
    with ClockSampler(0) as clocks:
        stats = server.run([dict(j) for j in jobs], max_seconds=420.0, log=sys.stderr)
    # alone vs in the mix
    rng = np.random.default_rng(3)
    same = []
    served = [j for j in server.done if j["status"] == nat.TRAJ_STEP_LIMIT]
    for j in rng.choice(served, size=min(6, len(served)), replace=False):
        lat = server.cache.get(j["lattice"], j["cells"])
        n = lat["n_sites"]
        q = np.zeros(n)
        q[j["dopant_sites"]] = 1.0
        tab = lat["tables"].with_charges(q, j["carriers"])
        alone = BatchedKmc(tab, np.asarray(j["carrier_sites"])[None, :], seed=SEED,
                           chunk_steps=j["steps"], step_limit=j["steps"],
                           traj_offset=j["id"], use_graph=False)
        alone.run(j["steps"])
        torch.cuda.synchronize()
        disp = (alone.batch.last_row + alone.batch.disp).cpu().numpy()[0, :3 * j["carriers"]]
        same.append(bool(np.array_equal(alone.batch.occ.cpu().numpy()[0, :j["carriers"]],
                                        j["occupancy"])
                         and alone.batch.time.item() == j["time"]
                         and np.array_equal(disp.reshape(-1, 3), j["displacement"])))
    line = {"workload": "serving", "metric": "KMC job latency p50/p99 and steps/s",
            "arrival_rate_jobs_per_s": 200.0, "jobs": len(jobs), "arrival_seed": 11,
            "lattice_cache_warm_s": warm_s, "warm_up_jobs": n_warm,
            "warm_up_jobs_s": warm_jobs_s, **stats,
            "alone_equals_mix": same, "chunk_steps": args.chunk,
            "clocks": clocks.summary()}
    del server
    torch.cuda.empty_cache()
    return line


def serving_bench(args):
    import torch
    from pycd_gb300 import _native as nat
    torch.cuda.set_device(0)
    nat.require_device()
    print(json.dumps(serving_record(args)), flush=True)


def heavy_bench(args):
    """Trajectories of many carriers (corundum 10x10x3 = 3,600 sites, 16 and
    32 electrons, no dopants): per-step latency and aggregate steps/s of the
    warp form (one warp per trajectory) and the block forms (2 or 4 warps
    per trajectory) for 1, 152 and 608 trajectories, and the shape the
    default launcher picks.  Events are the same in every form; the line
    also checks that on the first trajectory."""
    import torch
    from pycd_gb300 import _native as nat
    from pycd_gb300 import workloads as wl
    from pycd_gb300.kmc import KmcBatch, KmcEngine, default_lanes
    nat.require_device()
    system = wl.corundum(N_CELLS)
    A = system.get_precomputed_array_device("fp64")
    n_steps, warm = args.heavy_steps, 300
    trajs = [args.traj] if args.traj != N_TRAJ else [1, 152, 608]
    rows = []
    for nc in (16, 32):
        tables, run = wl.batched_tables(system, A, nc, [], 1.0, t_final=1e30,
                                        time_interval=1e27)
        shapes = [args.lanes] if args.lanes else [32, 64, 128]
        for T in trajs:
            occ = np.stack([np.random.default_rng(SEED + i).choice(3600, nc, replace=False)
                            for i in range(T)]).astype(np.int32)
            procs = {}
            for lanes in shapes:
                eng = KmcEngine(tables, launch={"lanes_per_traj": lanes})
                b = KmcBatch(occ, step_capacity=warm)
                eng.advance(b, warm, eng.rng_struct(seed=SEED))
                torch.cuda.synchronize()
                procs[lanes] = b.step_proc[0].cpu().numpy()
                # timed steps record no per-step output (no exact time per step)
                b.step_time = b.step_proc = None
                b.step_capacity = 0
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                eng.advance(b, n_steps, eng.rng_struct(seed=SEED))
                e1.record()
                torch.cuda.synchronize()
                ms = e0.elapsed_time(e1)
                rows.append({"carriers": nc, "trajectories": T, "lanes": lanes,
                             "us_per_step": 1e3 * ms / n_steps,
                             "steps_per_s": T * n_steps / (ms / 1e3)})
            same = all(np.array_equal(v, procs[shapes[0]]) for v in procs.values())
            rows.append({"carriers": nc, "trajectories": T,
                         "default_lanes": default_lanes(4 * nc, nc, T),
                         "events_equal_across_forms": bool(same)})
    line = {"workload": "heavy", "metric": "KMC step latency and steps/s, many carriers",
            "unit": "us/step", "dtype": "f64", "data": "synthetic",
            "config": {"lattice": "corundum 10x10x3 = 3,600 sites", "slots": 4,
                       "timed_steps": n_steps, "warmup_steps": warm,
                       "lanes": "32 = one warp; 64 / 128 = one block of 2 / 4 warps"},
            "rows": rows}
    if not args.no_cpu_baseline:
        from oracle import kmc_oracle as ko
        from oracle import philox
        tables, run = wl.batched_tables(system, A, 32, [], 1.0, t_final=1e30,
                                        time_interval=1e27)
        m = system.material
        otab = ko.Tables(system.hop_neighbor_list, "Fe:Fe", np.zeros(3600, int), 12, 0, 12,
                         m.lambda_values["Fe:Fe"], m.v_ab["Fe:Fe"])
        occ0 = np.random.default_rng(SEED).choice(3600, 32, replace=False)
        k = 200
        u = np.array([v for st in range(k) for v in philox.step_uniforms(SEED, 0, st)])
        Ah = A.cpu().numpy()
        t0 = time.perf_counter()
        ko.run(Ah, otab, list(occ0), np.zeros(3600), -1.0, np.zeros(3600), m.vn, run.temp,
               u, run.time_interval, tables.n_path_steps, max_steps=k)
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": 1e6 * dt / k, "unit": "us/step", "cores": 1,
                                "kind": "port", "sample": "one 32-carrier trajectory, "
                                "%d steps, oracle port of the reference loop" % k}
    print(json.dumps(line), flush=True)


def msd_bench(args):
    """MSD analysis (Analysis.compute_msd) on device: the parameters of the
    reference's Hematite example (t_final 1e-4 s, interval 1e-8 s -> 10,001
    rows; msd_t_final 5,000 ns -> 501 lags; trim 50) for args.traj
    trajectories of 4 carriers, synthetic random-walk rows."""
    import torch
    from pycd_gb300 import _native as nat
    from pycd_gb300 import constants as K
    from pycd_gb300.analysis import msd_device
    torch.cuda.set_device(0)
    nat.require_device()
    T, S = args.traj, 4
    dt = 1e-8 * K.SEC2AUTIME
    R = int(1e-4 * K.SEC2AUTIME / dt) + 1
    L = int(5000.0 / K.AUTIME2NS / dt) + 1
    trim = 50
    gen = torch.Generator(device="cuda").manual_seed(SEED)
    rows = torch.randn((T, R, 3 * S), generator=gen, dtype=torch.float64, device="cuda")
    rows.mul_(5.5).cumsum_(1)
    call = dict(species_count=[S], n_rows=R, n_lags=L, trim_length=trim,
                dist_conversion=1 / K.ANG2BOHR, time_interval=dt,
                time_conversion=K.AUTIME2NS)
    reps = max(1, min(args.steps, 5))
    for _ in range(max(1, args.warmup)):
        msd_device(rows, **call)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    times = []
    with ClockSampler(0) as clocks:
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            res = msd_device(rows, **call)
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
    t = float(np.median(times))
    pairs = T * sum(R - l for l in range(1, L))
    flops = 9.0 * S * pairs  # per (row pair, carrier): 3 DSUB + 3 DFMA
    line = {"workload": "msd", "metric": "MSD analysis throughput (trajectories/s)",
            "value": T / t, "unit": "trajectories/s", "higher_is_better": True,
            "seconds_per_analysis": t, "dtype": "f64", "data": "synthetic",
            "config": {"trajectories": T, "rows": R, "lags": L, "carriers": S,
                       "trim": trim, "source": "examples/Hematite MSD parameters, "
                       "random-walk rows (normal steps, 5.5 bohr)"},
            "fp64_gflops_algorithmic": flops / t / 1e9, "gpu_launches_per_analysis": 6,
            "clocks": clocks.summary()}
    if not args.no_e2e:
        host = rows.cpu().pin_memory()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        dev = host.to("cuda", non_blocking=True)
        res = msd_device(dev, **call)
        out = {k: res[k].cpu() for k in ("msd_data", "sem_data", "slopes", "slope_stats")}
        e2e = time.perf_counter() - t0
        line["e2e"] = {"value": T / e2e, "unit": "trajectories/s",
                       "h2d_bytes": host.numel() * 8,
                       "d2h_bytes": sum(v.numel() * 8 for v in out.values())}
        del dev, host
    if not args.no_cpu_baseline:
        from oracle import msd_oracle as mo
        one = (rows[0].cpu().numpy() * (1 / K.ANG2BOHR)).reshape(R, S, 3)
        t0 = time.perf_counter()
        sd = mo.squared_displacements(one, L)
        cpu = time.perf_counter() - t0
        ref = res["sd"][0].cpu().numpy()
        line["cpu_baseline"] = {"value": 1.0 / cpu, "unit": "trajectories/s", "cores": 1,
                                "kind": "port", "sample": "1 trajectory, NumPy port of "
                                "the reference's lag loop (core.py:2991-3005)",
                                "max_rel_diff_vs_gpu": float(np.abs(sd - ref).max()
                                                             / np.abs(sd).max())}
    print(json.dumps(line), flush=True)


def plain_bench(args):
    """The plain configuration as its own JSON line (plain_record)."""
    print(json.dumps(plain_record()), flush=True)


def plain_record():
    """The plain, CPU-runnable configuration: corundum 3x3x3 = 324 sites, one
    electron on site default_rng(0).integers(324), FP64 Ewald array, 1e5 steps
    with injected uniforms default_rng(0).random(2e5) (time grid 1e-9 s up to
    1e-6 s).  The plain GPU form's steps/s, the FP64 array build, and the
    NumPy port of the reference loop on one host core over the same 1e5
    steps, with the event streams compared step by step."""
    import torch
    from oracle import ewald_oracle as eo
    from oracle import kmc_oracle as ko
    from pycd_gb300 import _native as nat
    from pycd_gb300 import constants as K
    from pycd_gb300 import workloads as wl
    from pycd_gb300.kmc import KmcBatch, KmcEngine
    nat.require_device()
    n_steps = 100_000
    system = wl.corundum((3, 3, 3))
    n = system.neighbors.num_system_elements
    system.get_precomputed_array_device("fp64")  # loads the kernels
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    A = system.get_precomputed_array_device("fp64")
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    tables, run = wl.batched_tables(system, A, 1, [], 1.0, t_final=1e-6, time_interval=1e-9)
    site = int(np.random.default_rng(0).integers(n))
    u = np.random.default_rng(0).random(2 * n_steps)
    u_dev = torch.as_tensor(u).cuda()[None, :]
    best, proc, times = None, None, None
    for lanes in (2, 4, 8, 16, 32, 64, 128):  # the plain form at its fastest lane count
        eng = KmcEngine(tables, launch={"lanes_per_traj": lanes})
        for rep in range(2):
            b = KmcBatch([[site]], step_capacity=n_steps,
                         unwrapped_rows=tables.n_path_steps)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            eng.advance(b, n_steps, eng.rng_struct(u_dev))
            e1.record()
            torch.cuda.synchronize()
            dt = e0.elapsed_time(e1) / 1e3
            if rep and (best is None or dt < best):
                best = dt
                proc = b.step_proc[0].cpu().numpy()
                times = b.step_time[0].cpu().numpy()
                steps = int(b.step.item())
    m = system.material
    A_host = eo.class_array(m.cartesian_unit_cell_coords, m.lattice_matrix, (3, 3, 3),
                            system.alpha, system.r_cut, system.k_cut, m.dielectric_constant)
    A_err_ev = float(np.abs(A.cpu().numpy() - A_host).max()) / K.EV2HARTREE
    otab = ko.Tables(system.hop_neighbor_list, "Fe:Fe", np.zeros(n, int), 12, 0, 12,
                     m.lambda_values["Fe:Fe"], m.v_ab["Fe:Fe"])
    t0 = time.perf_counter()
    o = ko.run(A_host, otab, [site], np.zeros(n), -1.0, np.zeros(n), m.vn, run.temp, u,
               run.time_interval, tables.n_path_steps, max_steps=n_steps)
    cpu_s = time.perf_counter() - t0
    same_events = bool(np.array_equal(o["proc"], proc[:len(o["proc"])]))
    t_rel = float(np.abs(o["time"][1:len(times) + 1] / times[:len(o["time"]) - 1] - 1).max())
    flops = 4.0 * n * n * (system.last_build_info["n_kvec"])
    return {
        "workload": "plain", "metric": "KMC steps/s (plain form, one trajectory)",
        "value": n_steps / best, "unit": "steps/s", "steps": n_steps, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": "plain: corundum 3x3x3 = 324 sites, 1 electron on site "
                   f"{site}, FP64 Ewald array, 1e5 steps, uniforms default_rng(0)"},
        "ewald_build": {"seconds": build_s, "n_kvec": system.last_build_info["n_kvec"],
                        "mode": system.last_build_info["mode"],
                        "algorithmic_gflops": flops / build_s / 1e9,
                        "max_abs_err_vs_oracle_ev": A_err_ev},
        "events_equal_oracle": same_events, "oracle_steps": int(o["steps"]),
        "time_max_rel_diff": t_rel, "gpu_steps_recorded": steps,
        "cpu_baseline": {"value": o["steps"] / cpu_s, "unit": "steps/s", "cores": 1,
                         "kind": "port", "sample": "the same 1e5 steps, NumPy port of the "
                         "reference loop"}}


OUTPUT_DATA = {"unwrapped_traj": {"file_name": "unwrapped_traj.npy", "write": 1,
                                  "write_every_step": 0},
               "time": {"file_name": "time_data.npy", "write": 1},
               "wrapped_traj": {"file_name": "wrapped_traj.npy", "write": 0},
               "energy": {"file_name": "energy_traj.npy", "write": 0},
               "delg_0": {"file_name": "delG0_traj.npy", "write": 0},
               "potential": {"file_name": "potential_traj.npy", "write": 0}}


def dropin_bench(args):
    """Run.do_kmc_steps, the drop-in call, on the plain configuration's
    lattice (corundum 3x3x3 = 324 sites, one electron drawn by the Run's
    MT19937 stream, FP64 array, time grid 1e-11 s up to 2e-9 s, about
    5e4 steps per trajectory): n_traj trajectories in one call, where they
    advance together, against one call per trajectory (the reference's
    one-after-another order), wall time of the whole call with set-up and
    file writes.  Both write the same files."""
    import shutil
    import tempfile
    import torch
    from pycd_gb300 import _native as nat
    from pycd_gb300 import workloads as wl
    nat.require_device()
    system = wl.corundum((3, 3, 3))
    A, _ = system.get_precomputed_array(None, precision="fp64")
    rows = []
    for n_traj in (1, 8, 64):
        d = Path(tempfile.mkdtemp(prefix="pycd_dropin_"))
        run = wl.run_for(system, 1, t_final=2e-9, time_interval=1e-11, n_traj=n_traj,
                         precomputed_array=A)
        run.do_kmc_steps(d, OUTPUT_DATA, 11, "serial")  # untimed: loads the kernels
        shutil.rmtree(d)
        d = Path(tempfile.mkdtemp(prefix="pycd_dropin_"))
        t0 = time.perf_counter()
        run.do_kmc_steps(d, OUTPUT_DATA, 11, "serial")
        torch.cuda.synchronize()
        together = time.perf_counter() - t0
        steps = int(sum(len(s) for s in run.last_run_steps))
        t_each = 0.0
        same = True
        for i in range(n_traj):
            one = wl.run_for(system, 1, t_final=2e-9, time_interval=1e-11, n_traj=1,
                             precomputed_array=A)
            e = Path(tempfile.mkdtemp(prefix="pycd_dropin_"))
            shutil.copy(d / f"traj{i + 1}" / "initial_rnd_state.dump", e)
            t0 = time.perf_counter()
            one.do_kmc_steps(e, OUTPUT_DATA, 11, "parallel")
            torch.cuda.synchronize()
            t_each += time.perf_counter() - t0
            for name in ("unwrapped_traj.npy", "time_data.npy"):
                same &= (d / f"traj{i + 1}" / name).read_bytes() == (e / name).read_bytes()
            shutil.rmtree(e)
        shutil.rmtree(d)
        rows.append({"n_traj": n_traj, "steps": steps, "one_call_s": together,
                     "one_call_steps_per_s": steps / together,
                     "call_per_trajectory_s": t_each,
                     "call_per_trajectory_steps_per_s": steps / t_each,
                     "speedup": t_each / together, "files_identical": bool(same)})
    print(json.dumps({"workload": "dropin", "metric": "Run.do_kmc_steps wall time",
                      "config": "corundum 3x3x3 (324 sites), 1 electron, t_final 2e-9 s, "
                                "dt 1e-11 s, FP64 array", "rows": rows}), flush=True)


def ewald_params_bench(args):
    """Ewald parameter selection (get_ewald_parameters) on the Hematite
    example lattice with device energy scans: the cases of the fixtures in
    tests/golden/ewald_params.json, timed end to end (host logic included).
    The reference's own NumPy run of the same cases, recorded when the
    fixtures were made (1 core, x86 host), is given beside each."""
    import contextlib
    import io
    import tempfile
    sys.path.insert(0, str(ROOT / "tests"))
    import golden_io as gio
    from pycd_gb300 import _native as nat
    from pycd_gb300.core import System
    nat.require_device()
    cfg, arr = gio.load("ewald_params")
    hem_cfg, hem_arr = gio.load("hematite")
    hop = gio.hop_list(hem_cfg, hem_arr)
    for name in ("rcut_optimal", "rcut_kcut_optimal", "kcut_converge"):
        case = cfg[name]
        mat, nb = gio.material(hem_cfg, system_size=case["system_size"])
        pmiv = hem_arr["pmiv"] if case["system_size"] == [2, 2, 1] else arr[name + "|pmiv"]
        p = dict(cfg["base_params"], **case["params"])
        prec = dict(p["precision_parameters"], step_change_data_points=10)
        best, builds, chosen = None, 0, None
        for _ in range(2):  # the first run also loads the kernels
            sysm = System(mat, nb, hop, pmiv, p["alpha"], p["r_cut"], p["k_cut"], prec)
            dst = Path(tempfile.mkdtemp()) / "InputFiles"
            dst.mkdir()
            t0 = time.perf_counter()
            with contextlib.redirect_stdout(io.StringIO()):
                chosen, _, _ = sysm.get_ewald_parameters([], dst)
            dt = time.perf_counter() - t0
            best = dt if best is None else min(best, dt)
            builds = sysm._energy_evaluator().builds
        ok = all(abs(chosen[k] / case[k] - 1) < 1e-12 for k in ("alpha", "r_cut", "k_cut"))
        print(json.dumps({"workload": "ewald-params", "case": name,
                          "n_sites": int(nb.num_system_elements), "seconds": best,
                          "device_builds": builds, "same_choice_as_reference": ok,
                          "reference_recorded_seconds": case["reference_seconds"],
                          "reference_recorded_on": "NumPy, 1 core, x86 host of this build"}),
              flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="batched",
                    choices=["batched", "plain", "ewald-split", "uneven", "serving",
                             "msd", "ewald-params", "heavy", "dropin"])
    ap.add_argument("--heavy-steps", type=int, default=2000)
    ap.add_argument("--jobs", type=int, default=2000)
    ap.add_argument("--max-job-steps", type=int, default=1_000_000)
    ap.add_argument("--sizes", default="")
    ap.add_argument("--kvecs", default="")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--traj", type=int, default=N_TRAJ)
    ap.add_argument("--chunk", type=int, default=CHUNK)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-serving", action="store_true",
                    help="leave the serving record out of the default line")
    ap.add_argument("--no-plain", action="store_true",
                    help="leave the plain configuration's record out of the default line")
    ap.add_argument("--no-ewald", action="store_true",
                    help="leave the split-precision build record out of the default line")
    ap.add_argument("--lanes", type=int, default=0)
    ap.add_argument("--warps", type=int, default=0)
    ap.add_argument("--min-blocks", type=int, default=0,
                    help="2 = the 128-register kernel variant")
    ap.add_argument("--sched-steps", type=int, default=-1,
                    help="queue form of the warp-form launch: steps per round "
                         "(0 = static form, -1 = the default)")
    args = ap.parse_args()
    if args.impl == "reference":
        return reference_arm(args)
    if args.workload == "ewald-split":
        return ewald_split_bench(args)
    if args.workload == "uneven":
        return uneven_bench(args)
    if args.workload == "serving":
        return serving_bench(args)
    if args.workload == "msd":
        return msd_bench(args)
    if args.workload == "plain":
        return plain_bench(args)
    if args.workload == "ewald-params":
        return ewald_params_bench(args)
    if args.workload == "heavy":
        return heavy_bench(args)
    if args.workload == "dropin":
        return dropin_bench(args)

    import torch
    import torch.distributed as dist
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from pycd_gb300 import _native as nat
    from pycd_gb300.batch import BatchedKmc, run_batched
    from pycd_gb300.replicas import stream_offset
    nat.require_device()
    system, A, tables, run, dopants, occ = build_workload(rank, args.traj)
    launch = {}
    if args.lanes:
        launch["lanes_per_traj"] = args.lanes
    if args.warps:
        launch["warps_per_block"] = args.warps
    if args.min_blocks:
        launch["min_blocks_per_sm"] = args.min_blocks
    # launch shape: autotuned (untimed) unless given; it never changes events
    sched = SCHED_STEPS if args.sched_steps < 0 else args.sched_steps
    bk = BatchedKmc(tables, occ, seed=SEED, chunk_steps=args.chunk,
                    traj_offset=stream_offset(rank, args.traj), launch=launch,
                    autotune=0 if (args.lanes or args.warps) else 2000,
                    schedule_steps=sched)
    tuned = {"lanes_per_traj": bk.buckets[0].engine.launch.lanes_per_traj,
             "warps_per_block": bk.buckets[0].engine.launch.warps_per_block,
             "min_blocks_per_sm": bk.buckets[0].engine.launch.min_blocks_per_sm,
             "sched_steps": bk.buckets[0].engine.launch.sched_steps}
    flush = torch.empty(256 * 2 ** 20, dtype=torch.uint8, device="cuda")
    for _ in range(args.warmup):
        bk.step_chunk()
    torch.cuda.synchronize()
    steps0 = bk.batch.step.sum().item()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        t0 = time.perf_counter()
        for i in range(args.steps):
            flush.fill_(i & 0xFF)  # write 256 MiB (> L2) between chunks
            ev[i][0].record()
            bk.step_chunk()
            ev[i][1].record()
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        wall = time.perf_counter() - t0
    kernel_ms = [a.elapsed_time(b) for a, b in ev]
    steps_done = bk.batch.step.sum().item() - steps0
    status = bk.status_counts()
    from pycd_gb300 import replicas
    wall_max, total_steps = replicas.aggregate(wall, steps_done, device="cuda")
    value = total_steps / wall_max

    # plain one-trajectory form (same kernel, same events)
    plain = time_plain(tables, occ)

    # end to end through the host-buffer entry point
    e2e = None
    if not args.no_e2e:
        A_host = A.cpu().numpy()
        th = {"nbr": run.site_nbr, "hop": run.site_hop, "lam": run.site_lam,
              "vab": run.site_vab, "e_rel": run.system_relative_energies,
              "q_fixed": np.where(np.isin(np.arange(3600), dopants), 1.0, 0.0),
              "carrier_charge": -1.0, "n_carriers": N_CARRIERS, "vn": run.material.vn,
              "kT": run.temp, "time_interval": run.time_interval,
              "n_path_steps": int(run.t_final / run.time_interval) + 1}
        e2e_steps = args.chunk * args.steps
        # untimed warm-up through the same call: one-time process costs (the
        # first pinned host allocation, kernel loading) are not per-step work
        run_batched(A_host, th, occ, args.chunk, seed=SEED + 1, chunk_steps=args.chunk,
                    launch=tuned)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = run_batched(A_host, th, occ, e2e_steps, seed=SEED + 1,
                          chunk_steps=args.chunk, launch=tuned)
        torch.cuda.synchronize()
        e2e_wall = time.perf_counter() - t0
        e2e = {"value": float(res["step"].sum()) * world / e2e_wall, "unit": "steps/s",
               "h2d_bytes_per_step": res["h2d_bytes"] / max(1, res["launches"]),
               "d2h_bytes_per_step": res["d2h_bytes"] / max(1, res["launches"]),
               "wall_s": e2e_wall}

    hbm, peak_kind = peaks()
    launch_ms = float(np.mean(kernel_ms))
    steps_per_launch = steps_done / max(1, args.steps)
    bytes_per_launch = B_STEP * steps_per_launch
    achieved = bytes_per_launch / (launch_ms / 1e3) / 1e9
    # the binding resource: FP64 issue.  One DFMA, DADD or DMUL thread
    # instruction takes one FP64 lane slot; the peak slot rate is half the
    # measured DGEMM flop rate (2 flops per DFMA slot).
    fp64_tf = fp64_peak_tflops()
    fp64_peak_instr = fp64_tf * 1e12 / 2.0
    fp64_per_step = FP64_INSTR_PER_STEP.get(
        (tuned["lanes_per_traj"], tuned["min_blocks_per_sm"]))
    fp64_achieved = (fp64_per_step * steps_per_launch / (launch_ms / 1e3)
                     if fp64_per_step else None)
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline_1core(system, run, dopants, occ)
    extra = {}
    if rank == 0 and not args.no_plain:
        extra["plain_config"] = plain_record()
    if rank == 0 and not args.no_ewald:
        n, kk = 8192, 4096
        extra["ewald_split"] = ewald_split_record(n, kk, EWALD_SIZES[n][1][0], cpu=False)
    if rank == 0 and not args.no_serving:
        del bk
        torch.cuda.empty_cache()
        extra["serving"] = serving_record(args)
    if rank == 0:
        line = {
            "metric": "KMC steps/s (batched uniform, 3,600 sites, 4 e- + 4 dopants)",
            "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * wall_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": batched_config(args, world),
            "plain_steps_per_s": plain, "batched_over_plain": value / world / plain,
            "launch_shape": tuned,
            "status_counts": status,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm,
                         "unit": "GB/s", "frac": achieved / hbm,
                         "traffic": DRAM_BYTES_PER_STEP * steps_per_launch,
                         "traffic_source": "ncu dram bytes per KMC step of one chunk "
                                           "launch, scaled by this launch's steps",
                         "peak_kind": peak_kind,
                         "bytes_per_step": B_STEP, "launch_ms": launch_ms,
                         "fp64_issue": {
                             "instr_per_step": fp64_per_step,
                             "achieved": fp64_achieved, "peak": fp64_peak_instr,
                             "unit": "FP64 thread instr/s",
                             "frac": (fp64_achieved / fp64_peak_instr
                                      if fp64_achieved else None),
                             "peak_kind": "measured: cuBLAS DGEMM 4096^3 this run, "
                                          f"{fp64_tf:.3f} TFLOP/s / 2 flops per DFMA"}},
            "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": args.steps,
            "clocks": clocks.summary(), **extra}
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
