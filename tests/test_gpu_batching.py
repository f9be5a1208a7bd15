"""GPU: uneven multi-system batches (buckets, autotuned shapes) and the
continuous-batching server: every trajectory's result equals the same
trajectory advanced alone."""
import numpy as np
import pytest

from pycd_gb300 import _native as nat
from pycd_gb300 import workloads as wl
from pycd_gb300.batch import BatchedKmc

pytestmark = pytest.mark.gpu


def _tables(lattice, cells, n_carriers, dopants, precision="fp64"):
    system = wl.system_for(lattice, cells)
    A = system.get_precomputed_array_device(precision)
    base, _ = wl.batched_tables(system, A, 1, [], 1.0, 1e30, 1e27)
    base.share_rate_coefficients()
    n = system.neighbors.num_system_elements
    q = np.zeros(n)
    q[dopants] = 1.0
    return base.with_charges(q, n_carriers), n


def test_uneven_buckets_equal_alone_runs(cuda_ready):
    """Trajectories of four systems in process-count buckets with autotuned
    shapes, widened between chunks as they finish, equal the same
    trajectories run alone."""
    import torch
    specs = [("corundum", (3, 3, 1), 1, [5]), ("monoclinic", (3, 3, 3), 3, []),
             ("corundum", (3, 3, 2), 6, [1, 2, 3]), ("monoclinic", (4, 4, 3), 12, [7])]
    tables = [_tables(*s)[0] for s in specs]
    rng = np.random.default_rng(0)
    occ, sys_index, limits = [], [], []
    for t in range(40):
        s = t % len(specs)
        n = tables[s].n_sites
        row = np.zeros(16, np.int32)
        row[:tables[s].n_carriers] = rng.choice(n, tables[s].n_carriers, replace=False)
        occ.append(row)
        sys_index.append(s)
        limits.append(int(rng.integers(500, 3000)))
    bk = BatchedKmc(tables, np.stack(occ), sys_index=sys_index, seed=77,
                    chunk_steps=1000, step_limit=limits, autotune=True)
    assert len(bk.buckets) >= 3
    # chunk by chunk, re-picking the buckets' shapes for the trajectories
    # still running (widening, up to the block forms): results must not move
    changed = 0
    for _ in range(3):
        bk.step_chunk()
        torch.cuda.synchronize()
        changed += bk.adapt_shapes()
    assert changed > 0
    torch.cuda.synchronize()
    assert (bk.gather("status").cpu().numpy() == nat.TRAJ_STEP_LIMIT).all()
    assert (bk.gather("step").cpu().numpy() == np.array(limits)).all()
    for t in (0, 1, 2, 3, 17, 38):
        s = sys_index[t]
        alone = BatchedKmc(tables[s], occ[t][None, :tables[s].n_carriers], seed=77,
                           chunk_steps=limits[t], step_limit=limits[t],
                           traj_offset=t, use_graph=False)
        alone.run(limits[t])
        torch.cuda.synchronize()
        nc = tables[s].n_carriers
        assert np.array_equal(alone.batch.occ.cpu().numpy()[0, :nc],
                              bk.gather("occ").cpu().numpy()[t, :nc])
        assert alone.batch.time.item() == bk.gather("time")[t].item()


def test_server_results_equal_alone_runs(cuda_ready):
    import torch
    from pycd_gb300.serving import KmcServer, poisson_jobs
    jobs = poisson_jobs(24, rate=400.0, seed=5, median_sites=400, max_sites=2000,
                        max_carriers=8, min_steps=2000, max_steps=20000)
    server = KmcServer(budget_bytes=20e9, chunk_steps=1500, slots_per_bucket=8, seed=9)
    # warm-up jobs pass through the same buckets first and are discarded
    n_warm = server.warm_up(jobs, steps=700)
    assert n_warm == len({int(j["carriers"] - 1).bit_length() for j in jobs})
    assert server.done == [] and all(not b.jobs for b in server.buckets.values())
    stats = server.run([dict(j) for j in jobs], max_seconds=300)
    assert stats["jobs"] == 24 and stats["unfinished"] == 0
    assert stats["latency_p99_s"] >= stats["latency_p50_s"] > 0
    for j in server.done[:6]:
        assert j["status"] == nat.TRAJ_STEP_LIMIT and j["steps_done"] == j["steps"]
        lat = server.cache.get(j["lattice"], j["cells"])
        q = np.zeros(lat["n_sites"])
        q[j["dopant_sites"]] = 1.0
        tab = lat["tables"].with_charges(q, j["carriers"])
        alone = BatchedKmc(tab, np.asarray(j["carrier_sites"])[None, :], seed=9,
                           chunk_steps=j["steps"], step_limit=j["steps"],
                           traj_offset=j["id"], use_graph=False)
        alone.run(j["steps"])
        torch.cuda.synchronize()
        nc = j["carriers"]
        assert np.array_equal(alone.batch.occ.cpu().numpy()[0, :nc], j["occupancy"])
        assert alone.batch.time.item() == j["time"]
        disp = (alone.batch.last_row + alone.batch.disp).cpu().numpy()[0, :3 * nc]
        assert np.array_equal(disp.reshape(nc, 3), j["displacement"])


def _diffusivity(bk, n_traj, n_carriers):
    """D = <|dr|^2> / (6 t) per carrier at the end of each trajectory; the
    mean and its standard error over carriers."""
    disp = (bk.batch.last_row + bk.batch.disp).cpu().numpy()[:, :3 * n_carriers]
    r2 = (disp.reshape(n_traj, n_carriers, 3) ** 2).sum(-1)
    d = (r2 / (6.0 * bk.batch.time.cpu().numpy()[:, None])).ravel()
    return float(d.mean()), float(d.std(ddof=1) / np.sqrt(len(d)))


@pytest.mark.parametrize("lattice,target", [("corundum", 6000), ("monoclinic", 8192)])
def test_split_array_diffusivity_matches_fp64(cuda_ready, lattice, target):
    """Above 5,000 sites: 256 trajectories of 4 electrons, 1e5 steps each, on
    the FP64 array and on the BF16x3 split-precision array (independent
    Philox streams).  The diffusivities agree within statistical error
    (|z| < 4 on the carriers' standard errors)."""
    import torch
    cells = wl.supercell_for(lattice, target)
    system = wl.system_for(lattice, cells)
    n = system.neighbors.num_system_elements
    assert n > 5000
    res = {}
    for seed, prec in ((101, "fp64"), (202, "bf16x3")):
        A = system.get_precomputed_array_device(prec)
        tab, _ = wl.batched_tables(system, A, 4, [], 1.0, 1e30, 1e27)
        rng = np.random.default_rng(seed)
        occ = np.stack([rng.choice(n, 4, replace=False) for _ in range(256)]).astype(np.int32)
        bk = BatchedKmc(tab, occ, seed=seed, chunk_steps=25000, step_limit=100000)
        bk.run(100000)
        torch.cuda.synchronize()
        assert (bk.batch.step.cpu().numpy() == 100000).all()
        res[prec] = _diffusivity(bk, 256, 4)
        del bk, tab, A
    (d64, s64), (ds, ss) = res["fp64"], res["bf16x3"]
    z = abs(d64 - ds) / np.hypot(s64, ss)
    print(f"{lattice} N={n}: D_fp64 {d64:.4e} +- {s64:.1e}, D_split {ds:.4e} +- {ss:.1e}, "
          f"|z| = {z:.2f}")
    assert z < 4.0


def _alone_equals_mix(server, jobs, seed):
    import torch
    for j in jobs:
        lat = server.cache.get(j["lattice"], j["cells"])
        q = np.zeros(lat["n_sites"])
        q[j["dopant_sites"]] = 1.0
        tab = lat["tables"].with_charges(q, j["carriers"])
        alone = BatchedKmc(tab, np.asarray(j["carrier_sites"])[None, :], seed=seed,
                           chunk_steps=j["steps"], step_limit=j["steps"],
                           traj_offset=j["id"], use_graph=False)
        alone.run(j["steps"])
        torch.cuda.synchronize()
        nc = j["carriers"]
        assert np.array_equal(alone.batch.occ.cpu().numpy()[0, :nc], j["occupancy"])
        assert alone.batch.time.item() == j["time"]


def test_server_under_hbm_pressure_evicts_and_defers(cuda_ready):
    """An HBM budget that holds the largest lattice but never all of them:
    the lattice cache evicts idle lattices (least recently used) and defers
    jobs whose lattice does not fit yet; every job finishes, the cache never
    holds more than the budget, and results equal the jobs run alone."""
    from pycd_gb300.serving import KmcServer, LatticeCache, poisson_jobs
    jobs = poisson_jobs(40, rate=400.0, seed=21, median_sites=800, max_sites=3000,
                        max_carriers=6, min_steps=1000, max_steps=6000, size_grid=12)
    probe = LatticeCache(1e30)
    fps = sorted({probe.footprint((12 if j["lattice"] == "corundum" else 4)
                                  * int(np.prod(j["cells"])), 4)
                  for j in jobs})
    assert len(fps) >= 4
    budget = fps[-1] + 0.5 * fps[-2]
    server = KmcServer(budget_bytes=budget, chunk_steps=1000, slots_per_bucket=8, seed=3)
    stats = server.run([dict(j) for j in jobs], max_seconds=300)
    assert stats["jobs"] == 40 and stats["unfinished"] == 0 and stats["rejected"] == 0
    assert stats["lattice_evictions"] > 0 and stats["admission_deferrals"] > 0
    assert server.cache.peak_bytes <= budget
    assert all(j["status"] == nat.TRAJ_STEP_LIMIT for j in server.done)
    _alone_equals_mix(server, server.done[:4] + server.done[-2:], seed=3)


def test_server_rejects_a_lattice_larger_than_the_budget(cuda_ready):
    from pycd_gb300.serving import KmcServer, poisson_jobs
    jobs = poisson_jobs(3, rate=100.0, seed=2, median_sites=400, max_sites=800,
                        max_carriers=2, min_steps=500, max_steps=800)
    server = KmcServer(budget_bytes=1e5, chunk_steps=500, slots_per_bucket=4, seed=1)
    stats = server.run([dict(j) for j in jobs], max_seconds=60)
    assert stats["rejected"] == 3 and stats["unfinished"] == 0


def test_server_cancels_a_running_and_a_pending_job(cuda_ready):
    """A long job is cancelled while its chunk runs on the GPU: it stops
    within a poll interval, retires with TRAJ_CANCELLED and its partial
    state, and its bucket's other jobs finish as if alone.  A job that has
    not arrived yet is cancelled with no steps."""
    import time
    from pycd_gb300.serving import KmcServer, poisson_jobs
    jobs = poisson_jobs(12, rate=200.0, seed=8, median_sites=400, max_sites=1000,
                        max_carriers=4, min_steps=2000, max_steps=4000)
    jobs[2]["steps"] = 50_000_000
    jobs[11]["arrival"] = 30.0
    server = KmcServer(budget_bytes=20e9, chunk_steps=1_000_000, slots_per_bucket=16,
                       seed=4, long_work=0)
    for j in jobs:
        server.submit(dict(j))
    server.start()
    assert server.cancel(11)
    t_cancel = None
    while server.busy() and server.now() < 120:
        server.step()
        running = any(j["id"] == 2 for b in server.buckets.values() for j in b.jobs.values()
                      if b.running)
        if t_cancel is None and running and server.now() > 1.0:
            assert server.cancel(2)
            t_cancel = server.now()
        time.sleep(0.001)
    assert t_cancel is not None and not server.busy()
    done = {j["id"]: j for j in server.done}
    assert done[11]["status"] == nat.TRAJ_CANCELLED and done[11]["steps_done"] == 0
    assert done[2]["status"] == nat.TRAJ_CANCELLED
    assert 0 < done[2]["steps_done"] < 50_000_000
    assert done[2]["finished"] - t_cancel < 2.0
    rest = [j for i, j in done.items() if i not in (2, 11)]
    assert len(rest) == 10 and all(j["status"] == nat.TRAJ_STEP_LIMIT for j in rest)
    _alone_equals_mix(server, rest[:4], seed=4)
