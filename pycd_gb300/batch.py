"""Batched persistent KMC: many trajectories, one kernel, CUDA-graph chunks.

``BatchedKmc`` keeps the state of T trajectories (over one or several
systems) resident in HBM and advances them in chunks of ``chunk_steps`` KMC
steps; each chunk is one launch of the persistent kernel, captured once into
a CUDA graph and replayed.  Uniforms come from per-trajectory Philox streams
(counter = (step, trajectory)), so a trajectory's events do not depend on
the batch it runs in, the chunking, or the launch shape.

``run_batched`` is the host-buffer entry point: it takes NumPy inputs,
copies them to the device, runs the whole job and returns NumPy results.
"""
import numpy as np

from . import _native as nat
from .kmc import KmcBatch, KmcEngine, KmcTables


class BatchedKmc(object):
    def __init__(self, tables, occupancy, sys_index=None, seed=0,
                 chunk_steps=10000, unwrapped=False, step_capacity=0,
                 launch=None, use_graph=True, traj_offset=0):
        import torch
        self.tables = list(tables) if isinstance(tables, (list, tuple)) else [tables]
        occ = np.asarray(occupancy)
        mc = max(t.n_carriers for t in self.tables)
        rows = max(t.n_path_steps for t in self.tables) if unwrapped else None
        self.batch = KmcBatch(occ, sys_index=sys_index, max_carriers=mc,
                              unwrapped_rows=rows, step_capacity=step_capacity)
        self.engine = KmcEngine(self.tables, launch)
        self.engine.upload()
        self.seed = int(seed)
        self.traj_offset = int(traj_offset)
        self.chunk_steps = int(chunk_steps)
        self.use_graph = use_graph
        self.graph = None
        self.stream = torch.cuda.Stream()
        self.launches = 0

    @property
    def n_traj(self):
        return self.batch.n_traj

    def _launch(self):
        self.engine.advance(self.batch, self.chunk_steps,
                            self.engine.rng_struct(seed=self.seed,
                                                   traj_offset=self.traj_offset))

    def capture(self):
        import torch
        g = torch.cuda.CUDAGraph()
        # capture records the launch (state pointers, chunk length, RNG key)
        # without executing it; every replay advances the resident state
        with torch.cuda.graph(g, stream=self.stream):
            self._launch()
        self.graph = g

    def step_chunk(self):
        """Advance every running trajectory by up to chunk_steps steps
        (asynchronous on the current stream)."""
        import torch
        if self.use_graph:
            if self.graph is None:
                self.capture()
            self.graph.replay()
        else:
            self._launch()
        self.launches += 1

    def run(self, total_steps):
        n = (int(total_steps) + self.chunk_steps - 1) // self.chunk_steps
        for _ in range(n):
            self.step_chunk()

    def steps_done(self):
        return int(self.batch.step.sum().item())

    def status_counts(self):
        s = self.batch.status.cpu().numpy()
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
    out = {"occupancy": bk.batch.occ.cpu().numpy(),
           "time": bk.batch.time.cpu().numpy(),
           "step": bk.batch.step.cpu().numpy(),
           "status": bk.batch.status.cpu().numpy()}
    if unwrapped:
        out["unwrapped"] = bk.batch.unwrapped.cpu().numpy()
    d2h = sum(v.nbytes for v in out.values())
    out["h2d_bytes"], out["d2h_bytes"], out["launches"] = h2d, d2h, bk.launches
    return out
