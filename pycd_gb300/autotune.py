"""Launch-shape autotuners: the KMC kernel (``tune``) and the tcgen05
split-precision Ewald contraction (``tune_split``).

The kernel's event streams do not depend on its launch shape (cumulative
rates are fixed balanced-tree sums over the process index), so the shape is
a pure performance choice.  ``tune`` times short probes of every candidate
(lanes per trajectory x warps per block x register variant, and one block
of 2 or 4 warps per trajectory) on the real batch, restoring the
batch state after each probe, and keeps the fastest.  Results are cached
in-process per (each system's site-count bucket, slots and number of
charged sites; process count, carrier count, trajectory count): the array's
size sets how much of it the L2 holds, so a shape tuned on a 300-site
lattice is not reused for a 20,000-site one.
"""
import numpy as np

_CACHE = {}


def candidates(max_processes, max_carriers):
    out = []
    for lanes in (4, 8, 16, 32):
        if lanes < max_carriers:
            continue
        per_lane = -(-max_processes // lanes)
        if per_lane > 8:
            continue
        for warps in (1, 2, 4, 8):
            for minb in ((1, 2) if per_lane <= 2 else (1,)):
                out.append({"lanes_per_traj": lanes, "warps_per_block": warps,
                            "min_blocks_per_sm": minb})
    # one block of 2 or 4 warps per trajectory (more than 32 processes)
    if max_processes > 32 and max_carriers <= 32:
        for lanes in (64, 128):
            if -(-max_processes // lanes) <= 4:
                out.append({"lanes_per_traj": lanes, "warps_per_block": lanes // 32,
                            "min_blocks_per_sm": 1})
    return out


def _size_bucket(n_sites):
    """Site counts in factors of two (300-599, 600-1,199, ...)."""
    return int(np.floor(np.log2(max(1, n_sites) / 300.0))) if n_sites >= 300 else -1


def cache_key(engine, batch):
    systems = tuple(sorted({(_size_bucket(t.n_sites), int(t.n_slots),
                             int(getattr(t, "q_fixed", None) is not None
                                 and int((t.q_fixed != 0).sum().item())))
                            for t in engine.tables}))
    return (systems, int(engine.launch.max_processes), int(engine.launch.max_carriers),
            int(batch.n_traj))


def _apply(engine, shape):
    engine.launch.lanes_per_traj = shape["lanes_per_traj"]
    engine.launch.warps_per_block = shape["warps_per_block"]
    engine.launch.min_blocks_per_sm = shape.get("min_blocks_per_sm", 1)


def tune(engine, batch, rng, probe_steps=200, reps=2, stream=None):
    """Pick the fastest launch shape for (engine, batch); sets it on the
    engine and returns ``{"best": shape, "table": [(shape, ms), ...]}``."""
    import torch
    key = cache_key(engine, batch)
    if key in _CACHE:
        best = _CACHE[key]
        _apply(engine, best)
        return {"best": best, "table": [], "cached": True}
    snap = batch.snapshot()
    limit = batch.step_limit
    batch.step_limit = None  # probes must not stop early
    table = []
    s = stream or torch.cuda.current_stream()
    for cand in candidates(engine.launch.max_processes, engine.launch.max_carriers):
        _apply(engine, cand)
        times = []
        for r in range(reps + 1):
            batch.restore(snap)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(s)
            engine.advance(batch, probe_steps, rng, stream=s)
            e1.record(s)
            e1.synchronize()
            if r:
                times.append(e0.elapsed_time(e1))
        table.append((cand, float(np.median(times))))
    batch.restore(snap)
    batch.step_limit = limit
    best = min(table, key=lambda x: x[1])[0]
    _apply(engine, best)
    _CACHE[key] = best
    return {"best": best, "table": table, "cached": False}


# ---------------------------------------------------------------------------
# Split-precision Ewald build
# ---------------------------------------------------------------------------
_SPLIT_CACHE = {}

# (form, raster): CTA pairs or single CTAs, super-tiles per raster block side
SPLIT_CANDIDATES = (("pair", 4), ("pair", 8), ("pair", 16), ("single", 8))


def split_cache_key(system, precision):
    """(precision, site-count bucket, k-count bucket): factors of two of N and
    of the k list length (enumerated on the host, as the build does), which
    set the tile count and the operand panels' length, so the L2 reuse the
    raster order buys."""
    from . import ewald as ew
    n = int(system.neighbors.num_system_elements)
    _, _, k_cut, _ = system._ewald_parameters()
    k_max = ew.k_max_for(system, k_cut)
    k = len(ew.effective_k_vectors(system.reciprocal_lattice_matrix, k_max, k_cut))
    return (precision, int(np.log2(max(1, n))), int(np.log2(max(1, k))))


def tune_split(system, precision="bf16x3", reps=2, candidates=SPLIT_CANDIDATES):
    """Pick the fastest launch shape of the split-precision build of
    ``system`` by timing each candidate's whole build (the array does not
    depend on the shape), set it as ``system.split_launch`` and return
    ``{"best": shape, "table": [(shape, ms), ...]}``.  Cached in-process per
    ``split_cache_key``."""
    import torch
    key = split_cache_key(system, precision)
    if key in _SPLIT_CACHE:
        system.split_launch = dict(_SPLIT_CACHE[key])
        return {"best": system.split_launch, "table": [], "cached": True}
    table = []
    for form, raster in candidates:
        system.split_launch = {"form": form, "raster": raster}
        times = []
        for r in range(reps + 1):
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            A = system.get_precomputed_array_device(precision)
            e1.record()
            e1.synchronize()
            del A
            if r:
                times.append(e0.elapsed_time(e1))
        table.append(({"form": form, "raster": raster}, float(np.median(times))))
    best = min(table, key=lambda x: x[1])[0]
    system.split_launch = dict(best)
    _SPLIT_CACHE[key] = dict(best)
    return {"best": best, "table": table, "cached": False}
