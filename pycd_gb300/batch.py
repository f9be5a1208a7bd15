"""Batched persistent KMC: many trajectories over one or many systems.

``BatchedKmc`` keeps the state of T trajectories resident in HBM and
advances them in chunks of ``chunk_steps`` KMC steps.  Trajectories are
grouped into buckets by their process count (carriers x slots, rounded up to
a power of two); each bucket has its own launch shape, picked by the
autotuner, and all buckets of a chunk run concurrently on forked streams.
One chunk is captured once into a CUDA graph and replayed.  Uniforms come
from per-trajectory Philox streams keyed by the trajectory's global id, so a
trajectory's events do not depend on its bucket, the batch it runs in, the
chunking or the launch shape.

``run_batched`` is the host-buffer entry point: NumPy inputs are copied to
the device, the whole job runs, and NumPy results come back.
"""
import numpy as np

from . import _native as nat
from .kmc import KmcBatch, KmcEngine, KmcTables, default_lanes


def _bucket_of(n_proc):
    b = 1
    while b < n_proc:
        b <<= 1
    return b


class _Bucket(object):
    def __init__(self, idx, batch, engine, ids):
        self.idx, self.batch, self.engine, self.ids = idx, batch, engine, ids
        self.stream = None
        self.tuning = None


class BatchedKmc(object):
    def __init__(self, tables, occupancy, sys_index=None, seed=0,
                 chunk_steps=10000, unwrapped=False, step_capacity=0,
                 launch=None, use_graph=True, traj_offset=0, step_limit=None,
                 autotune=False, n_carriers=None, schedule_steps=0):
        """``occupancy``: T x max_carriers initial sites (rows padded beyond
        each system's carrier count); ``sys_index``: system of each
        trajectory (default 0); ``step_limit``: per-trajectory step budget;
        ``schedule_steps``: > 0 runs the warp-form launches in the queue form
        (rounds of that many steps handed to free warps; same results)."""
        import torch
        self.tables = list(tables) if isinstance(tables, (list, tuple)) else [tables]
        occ = np.asarray(occupancy, dtype=np.int32)
        if occ.ndim == 1:
            occ = occ[None, :]
        T = occ.shape[0]
        sys_index = (np.zeros(T, np.int32) if sys_index is None
                     else np.asarray(sys_index, np.int32))
        limits = (None if step_limit is None else
                  np.broadcast_to(np.asarray(step_limit, np.int64), (T,)))
        self.n_traj = T
        self.seed = int(seed)
        self.chunk_steps = int(chunk_steps)
        self.use_graph = use_graph
        self.launches = 0
        self.master = KmcEngine(self.tables)
        self.master.upload()
        mc = max(max(t.n_carriers for t in self.tables), occ.shape[1])
        rows = max(t.n_path_steps for t in self.tables) if unwrapped else None
        n_proc = np.array([self.tables[s].n_carriers * self.tables[s].n_slots
                           for s in sys_index])
        keys = np.array([_bucket_of(p) for p in n_proc])
        self.buckets = []
        self.order = np.zeros(T, np.int64)  # bucket-major position of traj t
        pos = 0
        for key in sorted(set(keys.tolist())):
            idx = np.nonzero(keys == key)[0]
            sub_occ = np.zeros((len(idx), mc), np.int32)
            sub_occ[:, :occ.shape[1]] = occ[idx]
            b = KmcBatch(sub_occ, sys_index=sys_index[idx], max_carriers=mc,
                         max_processes=int(n_proc.max()),
                         unwrapped_rows=rows, step_capacity=step_capacity,
                         step_limit=None if limits is None else limits[idx])
            eng = KmcEngine(None, launch, share=self.master)
            eng.restrict_shape(sys_index[idx])
            if schedule_steps:
                eng.schedule(schedule_steps)
            ids = torch.as_tensor((idx + int(traj_offset)).astype(np.uint64).view(np.int64)
                                  ).cuda()
            bk = _Bucket(idx, b, eng, ids)
            bk.stream = torch.cuda.Stream()
            self.buckets.append(bk)
            self.order[idx] = np.arange(pos, pos + len(idx))
            pos += len(idx)
        self.graph = None
        self.stream = torch.cuda.Stream()
        if autotune:  # True, or the probe length in steps
            self.autotune(probe_steps=int(autotune) if int(autotune) > 1 else 200)

    def _rng(self, bk):
        return bk.engine.rng_struct(seed=self.seed, traj_ids=bk.ids)

    def autotune(self, probe_steps=200):
        from . import autotune as at
        out = []
        for bk in self.buckets:
            bk.tuning = at.tune(bk.engine, bk.batch, self._rng(bk), probe_steps)
            out.append(bk.tuning["best"])
        self.graph = None
        return out

    def adapt_shapes(self):
        """Re-pick each bucket's launch shape for the trajectories still
        running, by the launcher's default rule (wider, up to one block of 4
        warps per trajectory, while the launch keeps <= 2 warps per SM
        sub-partition).  A shape is only widened, so a full bucket keeps its
        tuned shape; results do not depend on it.  Call between chunks (it
        reads the statuses); the next chunk recaptures its graph if a shape
        changed.  Returns the number of buckets whose shape changed."""
        changed = 0
        for bk in self.buckets:
            running = int((bk.batch.status == nat.TRAJ_RUNNING).sum().item())
            if running == 0:
                continue
            L = bk.engine.launch
            cur = L.lanes_per_traj or default_lanes(L.max_processes, L.max_carriers,
                                                    len(bk.idx))
            lanes = default_lanes(L.max_processes, L.max_carriers, running)
            if lanes > cur:
                L.lanes_per_traj = lanes
                if lanes > 32:
                    L.warps_per_block = 0
                    L.min_blocks_per_sm = 0
                changed += 1
        if changed:
            self.graph = None
        return changed

    def _launch_all(self):
        import torch
        cur = torch.cuda.current_stream()
        if len(self.buckets) == 1:
            bk = self.buckets[0]
            bk.engine.advance(bk.batch, self.chunk_steps, self._rng(bk), stream=cur)
            return
        ev = torch.cuda.Event()
        ev.record(cur)
        for bk in self.buckets:
            bk.stream.wait_event(ev)
            bk.engine.advance(bk.batch, self.chunk_steps, self._rng(bk),
                              stream=bk.stream)
        for bk in self.buckets:
            done = torch.cuda.Event()
            done.record(bk.stream)
            cur.wait_event(done)

    def capture(self):
        import torch
        g = torch.cuda.CUDAGraph()
        # capture records the launches (state pointers, chunk length, RNG key)
        # without executing them; every replay advances the resident state
        with torch.cuda.graph(g, stream=self.stream):
            self._launch_all()
        self.graph = g

    def step_chunk(self):
        """Advance every running trajectory by up to chunk_steps steps
        (asynchronous on the current stream)."""
        if self.use_graph:
            if self.graph is None:
                self.capture()
            self.graph.replay()
        else:
            self._launch_all()
        self.launches += len(self.buckets)

    def run(self, total_steps):
        n = (int(total_steps) + self.chunk_steps - 1) // self.chunk_steps
        for _ in range(n):
            self.step_chunk()

    def _gather(self, attr):
        import torch
        parts = [getattr(bk.batch, attr) for bk in self.buckets]
        cat = torch.cat(parts, 0)
        return cat[torch.as_tensor(self.order, device=cat.device)]

    @property
    def batch(self):
        """Single-bucket convenience: the KmcBatch of the only bucket."""
        assert len(self.buckets) == 1, "several buckets: use gather()"
        return self.buckets[0].batch

    def gather(self, attr):
        """Device tensor of one state/output field in trajectory order."""
        return self._gather(attr)

    def steps_done(self):
        return int(sum(bk.batch.step.sum().item() for bk in self.buckets))

    def status_counts(self):
        s = np.concatenate([bk.batch.status.cpu().numpy() for bk in self.buckets])
        return {int(k): int(v) for k, v in zip(*np.unique(s, return_counts=True))}


def run_batched(A, tables_host, occupancy, total_steps, seed=0, chunk_steps=10000,
                unwrapped=False, launch=None, pinned=True):
    """Host-buffer entry point: ``A`` and the tables are NumPy arrays; the
    job runs on the current GPU and the final state comes back as NumPy.

    ``tables_host`` is a dict with the KmcTables fields other than A (nbr,
    hop, lam, vab, e_rel, q_fixed, carrier_charge, n_carriers, vn, kT,
    time_interval, n_path_steps).  Returns a dict of host arrays (occupancy,
    time, step, status, and unwrapped rows when requested) and the bytes
    moved each way."""
    import torch
    dev = torch.device("cuda", torch.cuda.current_device())
    h2d = 0
    A_host = torch.from_numpy(np.ascontiguousarray(A, np.float64))
    if pinned:
        A_host = A_host.pin_memory()
    A_dev = A_host.to(dev, non_blocking=True)
    h2d += A_host.numel() * 8
    t = dict(tables_host)
    for k in ("nbr", "hop", "lam", "vab", "e_rel", "q_fixed"):
        h2d += np.asarray(t[k]).nbytes
    occ = np.asarray(occupancy)
    h2d += occ.nbytes
    tables = KmcTables(A_dev, t["nbr"], t["hop"], t["lam"], t["vab"], t["e_rel"],
                       t["q_fixed"], t["carrier_charge"], t["n_carriers"], t["vn"],
                       t["kT"], t["time_interval"], t["n_path_steps"])
    bk = BatchedKmc(tables, occ, seed=seed, chunk_steps=chunk_steps,
                    unwrapped=unwrapped, launch=launch)
    bk.run(total_steps)
    out = {"occupancy": bk.gather("occ").cpu().numpy(),
           "time": bk.gather("time").cpu().numpy(),
           "step": bk.gather("step").cpu().numpy(),
           "status": bk.gather("status").cpu().numpy()}
    if unwrapped:
        out["unwrapped"] = bk.gather("unwrapped").cpu().numpy()
    d2h = sum(v.nbytes for v in out.values())
    out["h2d_bytes"], out["d2h_bytes"], out["launches"] = h2d, d2h, bk.launches
    return out
