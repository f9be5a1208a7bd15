"""Continuous-batching KMC job server on one GPU.

Jobs (a lattice supercell, carriers, fixed dopant charges, a step budget and
a seed) arrive over time.  The server keeps:

* a cache of lattice systems: host set-up, the split-precision Ewald array
  and the device tables, shared by every job on that supercell and evicted
  least-recently-used when the HBM budget needs the room;
* per-job device tables that share the lattice's array, neighbour tables and
  rate coefficients and add only the job's background potential (dopants);
* trajectory slots in buckets keyed by (process count, carrier count), each
  a resident ``KmcBatch`` advanced by the persistent kernel.

Buckets run independently on their own streams: whenever a bucket's chunk
has finished, its finished jobs retire, arrived jobs of its class take the
free slots and its next chunk is launched, while the other buckets keep
running.  A job's uniforms come from the Philox stream of its job id, so its
result is the same alone and in any mix.  Latency = retirement time -
arrival time.
"""
import time

import numpy as np

from . import _native as nat
from .kmc import KmcBatch, KmcEngine, default_lanes


# status of a job whose lattice alone is larger than the HBM budget
REJECTED = -1


def _pow2(v):
    p = 1
    while p < v:
        p <<= 1
    return p


class LatticeCache(object):
    """(lattice, cells) -> lattice system with its device array and tables."""

    def __init__(self, budget_bytes, precision="bf16x3", t_final=1e30,
                 time_interval=1e27):
        self.budget = float(budget_bytes)
        self.precision = precision
        self.t_final, self.time_interval = t_final, time_interval
        self.entries = {}
        self.clock = 0
        self.builds = 0
        self.evictions = 0
        self.deferrals = 0        # get() calls the budget could not serve yet
        self.peak_bytes = 0.0     # largest bytes_in_use() after any build

    def bytes_in_use(self):
        return sum(e["bytes"] for e in self.entries.values())

    def fits(self, lattice, cells):
        """Whether the lattice could ever be held within the budget."""
        per = 12 if lattice == "corundum" else 4
        n = per * int(np.prod(cells))
        return self.footprint(n, 4) <= self.budget

    def footprint(self, n_sites, n_slots):
        # array + neighbour/hop/lambda/V/coefficient tables + per-job potentials
        return 8.0 * n_sites * n_sites + 8.0 * n_sites * n_slots * 9 + 64.0 * n_sites

    def _evict(self, need):
        while self.bytes_in_use() + need > self.budget:
            idle = [(e["used"], k) for k, e in self.entries.items() if e["refs"] == 0]
            if not idle:
                return False
            del self.entries[min(idle)[1]]
            self.evictions += 1
        return True

    def get(self, lattice, cells):
        """Entry for (lattice, cells), building it if needed; None when the
        budget cannot hold it now."""
        from . import workloads as wl
        key = (lattice, tuple(int(c) for c in cells))
        self.clock += 1
        e = self.entries.get(key)
        if e is not None:
            e["used"] = self.clock
            return e
        per = 12 if lattice == "corundum" else 4
        n = per * int(np.prod(cells))
        need = self.footprint(n, 4)
        if not self._evict(need):
            self.deferrals += 1
            return None
        system = wl.system_for(lattice, cells)
        A = system.get_precomputed_array_device(self.precision)
        tables, run = wl.batched_tables(system, A, 1, [], 1.0, self.t_final,
                                        self.time_interval)
        tables.share_rate_coefficients()
        e = {"key": key, "system": system, "tables": tables, "run": run,
             "n_sites": n, "bytes": self.footprint(n, tables.n_slots), "refs": 0,
             "used": self.clock}
        self.entries[key] = e
        self.builds += 1
        self.peak_bytes = max(self.peak_bytes, self.bytes_in_use())
        return e


class _Bucket(object):
    """Slots of one (process count, carrier count) class with their own
    system table, engine, stream and completion event.  A bucket is touched
    by the host (retire, admit, table upload) only between its chunks."""

    def __init__(self, np_bound, nc_bound, capacity, max_carriers, long_jobs=False):
        import torch
        self.np_bound, self.nc_bound = np_bound, nc_bound
        self.long_jobs = long_jobs
        self.capacity = capacity
        self.batch = KmcBatch(np.zeros((capacity, max_carriers), np.int32),
                              sys_index=np.zeros(capacity, np.int32),
                              max_carriers=max_carriers,
                              step_limit=np.zeros(capacity, np.int64),
                              cancellable=True)
        self.batch.status.fill_(nat.TRAJ_DONE)  # free slots are never advanced
        self.ids = torch.zeros(capacity, dtype=torch.int64, device="cuda")
        self.free = list(range(capacity - 1, -1, -1))
        self.jobs = {}            # slot -> job
        self.tables = []          # this bucket's per-job tables (sys_index space)
        self.table_free = []
        self.engine = None
        self.dirty = True
        self.stream = torch.cuda.Stream()
        self.event = None         # recorded after the chunk in flight
        self.running = False

    def add_table(self, tab):
        if self.table_free:
            ti = self.table_free.pop()
            self.tables[ti] = tab
        else:
            ti = len(self.tables)
            self.tables.append(tab)
        self.dirty = True
        return ti

    def drop_table(self, ti):
        self.tables[ti] = None
        self.table_free.append(ti)

    def upload(self):
        """Rebuild this bucket's system table (only between its chunks)."""
        live = [t for t in self.tables if t is not None]
        self.engine = KmcEngine([t if t is not None else live[0] for t in self.tables])
        self.engine.launch.max_processes = self.np_bound
        self.engine.launch.max_carriers = self.nc_bound
        self.engine.upload(self.stream)
        self.engine.launch.max_processes = self.np_bound
        self.engine.launch.max_carriers = self.nc_bound
        self.dirty = False


class KmcServer(object):
    """Buckets run independently: whenever one bucket's chunk has finished,
    its finished jobs are retired, arrived jobs of its class are admitted and
    its next chunk is launched on its own stream, while the other buckets keep
    running.  No bucket waits for another."""

    # a job whose steps x carriers reach this is "long": it goes to a bucket
    # of long jobs of its class, whose few trajectories get the wider (block)
    # launch forms, the fastest per step; the longest jobs set the latency
    # tail, so they are served first in per-step speed
    LONG_WORK = 1.6e7

    def __init__(self, budget_bytes=150e9, chunk_steps=5000, slots_per_bucket=1024,
                 precision="bf16x3", seed=0, max_carriers=32, long_work=LONG_WORK):
        self.cache = LatticeCache(budget_bytes, precision)
        self.chunk_steps = int(chunk_steps)
        self.slots = int(slots_per_bucket)
        self.seed = int(seed)
        self.max_carriers = int(max_carriers)
        self.long_work = float(long_work) if long_work else float("inf")
        self.buckets = {}
        self.pending = []
        self.waiting = {}         # bucket key -> prepared jobs waiting for a slot
        self.done = []
        self.t0 = None

    # -- jobs ------------------------------------------------------------
    def submit(self, job):
        """job: dict(id, lattice, cells, carriers, dopants, steps, seed,
        arrival) with `arrival` in seconds since start()."""
        self.pending.append(job)

    def start(self):
        self.t0 = time.perf_counter()

    def now(self):
        return time.perf_counter() - self.t0

    def _bucket(self, n_proc, n_car, long_jobs=False):
        key = (_pow2(n_proc), _pow2(n_car), bool(long_jobs))
        b = self.buckets.get(key)
        if b is None:
            b = _Bucket(key[0], key[1], self.slots, self.max_carriers, key[2])
            self.buckets[key] = b
        return b

    def _finish_unadmitted(self, job, status):
        """A job that leaves before it had a slot (cancelled or rejected)."""
        t = self.now()
        job.update(status=status, finished=t, latency=t - job["arrival"], steps_done=0,
                   time=0.0, occupancy=None, displacement=None)
        for k in ("bucket", "lattice_entry", "tab"):
            job.pop(k, None)
        self.done.append(job)

    def _prepare(self, job):
        """Lattice and job tables of an arrived job; False when the HBM
        budget cannot hold its lattice now.  A job whose lattice alone
        exceeds the budget is rejected (status REJECTED)."""
        if not self.cache.fits(job["lattice"], job["cells"]):
            self._finish_unadmitted(job, REJECTED)
            return True
        lat = self.cache.get(job["lattice"], job["cells"])
        if lat is None:
            return False
        n = lat["n_sites"]
        sites = np.random.default_rng(job["seed"]).choice(
            n, size=job["carriers"] + job["dopants"], replace=False)
        carriers, dopants = sites[:job["carriers"]], sites[job["carriers"]:]
        q = np.zeros(n)
        q[dopants] = 1.0
        tab = lat["tables"].with_charges(q, job["carriers"])
        long_job = job["steps"] * job["carriers"] >= self.long_work
        b = self._bucket(job["carriers"] * tab.n_slots, job["carriers"], long_job)
        lat["refs"] += 1
        job.update(lattice_entry=lat, bucket=b, tab=tab, carrier_sites=carriers,
                   dopant_sites=dopants)
        self.waiting.setdefault(id(b), []).append(job)
        return True

    def _admit_into(self, b):
        """Give free slots of idle bucket b to its waiting jobs."""
        queue = self.waiting.get(id(b), [])
        new = []
        while queue and b.free:
            job = queue.pop(0)
            slot = b.free.pop()
            job.update(slot=slot, table_index=b.add_table(job.pop("tab")),
                       admitted=self.now())
            b.jobs[slot] = job
            new.append(job)
        self._write_slots(b, new)
        return new

    def _write_slots(self, b, new):
        import torch
        if not new:
            return
        idx = torch.as_tensor([j["slot"] for j in new], device="cuda")
        occ = np.zeros((len(new), b.batch.max_carriers), np.int32)
        for r, j in enumerate(new):
            occ[r, :len(j["carrier_sites"])] = j["carrier_sites"]
        bt = b.batch
        dev = lambda a, dt: torch.as_tensor(np.asarray(a), dtype=dt, device="cuda")
        bt.occ[idx] = dev(occ, torch.int32)
        bt.sys_index[idx] = dev([j["table_index"] for j in new], torch.int32)
        bt.step_limit[idx] = dev([j["steps"] for j in new], torch.int64)
        b.ids[idx] = dev([j["id"] for j in new], torch.int64)
        for name in ("time", "energy"):
            getattr(bt, name)[idx] = 0.0
        bt.step[idx] = 0
        bt.path_index[idx] = 1
        bt.u_cursor[idx] = 0
        bt.disp[idx] = 0.0
        bt.last_row[idx] = 0.0
        bt.status[idx] = nat.TRAJ_RUNNING
        for j in new:  # the bucket is idle: no kernel reads these flags now
            bt.request_stop(j["slot"], False)

    def _launch(self, b):
        """Next chunk of idle bucket b on its stream (after the host-side
        writes and table builds made on the current stream)."""
        import torch
        b.stream.wait_stream(torch.cuda.current_stream())
        if b.dirty:
            b.upload()
        # launch shape for the jobs now in the bucket, not its slot count
        # (a bucket of long jobs holds few, which widens it to block forms)
        b.engine.launch.lanes_per_traj = default_lanes(b.np_bound, b.nc_bound,
                                                       max(1, len(b.jobs)))
        b.engine.advance(b.batch, self.chunk_for(b),
                         b.engine.rng_struct(seed=self.seed, traj_ids=b.ids),
                         stream=b.stream)
        b.event = torch.cuda.Event()
        b.event.record(b.stream)
        b.running = True

    def _collect(self, b):
        """Retire the finished jobs of bucket b, whose chunk has completed."""
        b.running = False
        st = b.batch.status.cpu().numpy()
        t_ret = self.now()
        out = []
        for slot, job in list(b.jobs.items()):
            if st[slot] != nat.TRAJ_RUNNING:
                self._retire(b, slot, job, int(st[slot]), t_ret)
                out.append(job)
        return out

    def cancel(self, job_id):
        """Cancel a job.  A job on the GPU stops at its next poll (the
        kernel reads its slot's flag in pinned host memory while the chunk
        runs) and retires with TRAJ_CANCELLED and its state so far; a job
        not yet admitted leaves at once with no steps.  Returns False for
        an unknown or finished job."""
        for j in self.pending:
            if j["id"] == job_id:
                self.pending.remove(j)
                self._finish_unadmitted(j, nat.TRAJ_CANCELLED)
                return True
        for queue in self.waiting.values():
            for j in queue:
                if j["id"] == job_id:
                    queue.remove(j)
                    j["lattice_entry"]["refs"] -= 1
                    self._finish_unadmitted(j, nat.TRAJ_CANCELLED)
                    return True
        for b in self.buckets.values():
            for slot, j in b.jobs.items():
                if j["id"] == job_id:
                    b.batch.request_stop(slot)
                    return True
        return False

    def step(self):
        """One scheduling pass: prepare arrived jobs, then for every bucket
        whose chunk has finished retire, admit and relaunch.  Returns the
        jobs retired."""
        now = self.now()
        arrived = [j for j in self.pending if j["arrival"] <= now]
        for j in arrived:
            if self._prepare(j):
                self.pending.remove(j)
        retired = []
        for b in list(self.buckets.values()):
            if b.running and b.event.query():
                retired += self._collect(b)
            if not b.running:
                self._admit_into(b)
                if b.jobs:
                    self._launch(b)
        return retired

    def _retire(self, b, slot, job, status, t_ret):
        bt = b.batch
        nc = job["carriers"]
        disp = (bt.last_row[slot] + bt.disp[slot]).cpu().numpy()[:3 * nc]
        job.update(status=status, finished=t_ret, latency=t_ret - job["arrival"],
                   steps_done=int(bt.step[slot].item()),
                   time=float(bt.time[slot].item()),
                   occupancy=bt.occ[slot].cpu().numpy()[:nc].copy(),
                   displacement=disp.reshape(nc, 3))
        bt.status[slot] = nat.TRAJ_DONE
        del b.jobs[slot]
        b.free.append(slot)
        b.drop_table(job["table_index"])
        job["lattice_entry"]["refs"] -= 1
        for k in ("bucket", "lattice_entry"):
            job.pop(k, None)
        self.done.append(job)

    def chunk_for(self, b):
        """Steps per chunk for bucket b: a step costs roughly in proportion
        to the carriers it sums over, so lighter buckets take longer chunks
        and every bucket's chunk lasts about as long."""
        return max(500, int(self.chunk_steps * 8 / max(8, b.nc_bound)))

    def warm_up(self, jobs, steps=1000):
        """Serve a short copy of one job per carrier class of `jobs` (each
        alone in its bucket, so the block launch forms run too) and discard
        it, so that one-time costs of the first admission, launch and
        retirement (first use of device code and host libraries) fall before
        traffic is taken.  Buckets stay allocated; the lattice cache and the
        served-job list are left as they were."""
        if self.pending or any(self.waiting.values()):
            raise RuntimeError("warm_up() runs before jobs are submitted")
        sample = {}
        for j in jobs:
            sample.setdefault(_pow2(j["carriers"]), j)
        done = self.done
        self.done = []
        self.run([dict(j, steps=min(int(j["steps"]), int(steps)), arrival=0.0)
                  for j in sample.values()])
        self.done = done
        return len(sample)

    def busy(self):
        return (bool(self.pending) or any(self.waiting.values())
                or any(b.jobs for b in self.buckets.values()))

    def run(self, jobs, max_seconds=600.0, log=None):
        """Serve `jobs` (arrival-time ordered) to completion; `log` is an
        optional file for a progress line every ~2 s."""
        for j in jobs:
            self.submit(j)
        self.start()
        steps = 0
        next_log = 2.0
        while self.busy() and self.now() < max_seconds:
            if log is not None and self.now() >= next_log:
                next_log += 2.0
                active = sum(len(b.jobs) for b in self.buckets.values())
                print(f"[serving] t={self.now():.1f}s done={len(self.done)} "
                      f"active={active} pending={len(self.pending)}", file=log, flush=True)
            retired = self.step()
            for j in retired:
                steps += j["steps_done"]
            if not retired:
                if not any(b.running for b in self.buckets.values()) and self.pending:
                    wait = min(j["arrival"] for j in self.pending) - self.now()
                    if wait > 0:
                        time.sleep(min(wait, 0.05))
                else:
                    time.sleep(0.0005)  # chunks in flight: poll their events
        for b in self.buckets.values():
            if b.running:
                b.event.synchronize()
                b.running = False
        wall = self.now()
        served = [j for j in self.done if j["status"] not in (REJECTED, nat.TRAJ_CANCELLED)]
        lat = np.array([j["latency"] for j in served]) if served else np.zeros(1)
        return {"jobs": len(self.done), "wall_s": wall, "steps": steps,
                "steps_per_s": steps / wall if wall else 0.0,
                "latency_p50_s": float(np.percentile(lat, 50)),
                "latency_p99_s": float(np.percentile(lat, 99)),
                "lattice_builds": self.cache.builds,
                "lattice_evictions": self.cache.evictions,
                "admission_deferrals": self.cache.deferrals,
                "peak_lattice_bytes": self.cache.peak_bytes,
                "long_job_buckets": sum(1 for b in self.buckets.values() if b.long_jobs),
                "cancelled": sum(1 for j in self.done if j["status"] == nat.TRAJ_CANCELLED),
                "rejected": sum(1 for j in self.done if j["status"] == REJECTED),
                "unfinished": len(self.pending) + sum(len(q) for q in self.waiting.values())
                + sum(len(b.jobs) for b in self.buckets.values())}


def poisson_jobs(n_jobs, rate=200.0, seed=0, median_sites=2000, min_sites=300,
                 max_sites=50000, max_carriers=32, min_steps=10_000,
                 max_steps=1_000_000, sigma=1.0, size_grid=24):
    """Arrival stream of the serving workload: exponential inter-arrival
    times at `rate` jobs/s, either lattice, log-normal site counts (clipped),
    carriers U{1..max_carriers}, dopants U{0..16}, steps U[min, max].
    With ``size_grid`` the drawn site count is snapped to the nearest of that
    many log-spaced sizes, so that jobs share a catalogue of lattices whose
    arrays stay cached (otherwise nearly every job needs its own array)."""
    from . import workloads as wl
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, n_jobs))
    grid = (np.exp(np.linspace(np.log(min_sites), np.log(max_sites), size_grid))
            if size_grid else None)
    jobs = []
    for i in range(n_jobs):
        lattice = "corundum" if rng.random() < 0.5 else "monoclinic"
        target = float(np.clip(np.exp(rng.normal(np.log(median_sites), sigma)),
                               min_sites, max_sites))
        if grid is not None:
            target = float(grid[np.argmin(np.abs(np.log(grid / target)))])
        jobs.append({"id": i, "lattice": lattice,
                     "cells": wl.supercell_for(lattice, target),
                     "carriers": int(rng.integers(1, max_carriers + 1)),
                     "dopants": int(rng.integers(0, 17)),
                     "steps": int(rng.integers(min_steps, max_steps + 1)),
                     "seed": int(rng.integers(1 << 31)), "arrival": float(t[i])})
    return jobs
