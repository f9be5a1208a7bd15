"""Device build of the Ewald precomputed array (System.get_precomputed_array,
PyCD/core.py:1611-1679) through ``pycd_ewald_build``.

Host work here is the k-vector list (integer, PyCD/core.py:816-838 with the
k^2 < k_cut^2 filter of core.py:868) and the choice of algorithm:

* ``fp64_direct`` - per-pair cos(k . d_ij) from the pairwise minimum-image
  vectors; the reference's exact formula for any pmiv.
* ``fp64``        - feature contraction F F^T in FP64.  Valid when every
  pmiv_ij equals r_j - r_i plus a supercell translation and the Ewald cell
  (``System.translational_matrix``) is that supercell.
* ``bf16x3`` / ``tf32x3`` - the same contraction on tcgen05 tensor cores.
"""
import numpy as np

from . import _native as nat


def k_max_for(system, k_cut):
    """k_max = ceil(k_cut / |b_i|) (PyCD/core.py:1599)."""
    return np.ceil(k_cut / system.reciprocal_lattice_vector_length).astype(int)


def half_space_k_vectors(recip, k_max, k_cut):
    """(k, keep): every half-space integer k-vector of the k_max box in the
    reference's order (get_effective_k_vectors, PyCD/core.py:816-838) and the
    mask of those with k^2 < k_cut^2 (core.py:868).

    The grid [-k_max, k_max]^3 in C order with the first member of every +-m
    pair kept is exactly the set of points before the origin.  k^2 is
    compared vectorised and every vector within rounding of the cut is
    re-evaluated with the reference's per-vector ``np.dot`` so the kept set
    is the reference's.
    """
    k_max = np.asarray(k_max, dtype=int)
    g = np.mgrid[-k_max[0]:k_max[0] + 1, -k_max[1]:k_max[1] + 1,
                 -k_max[2]:k_max[2] + 1].reshape(3, -1).T
    half = g[: len(g) // 2]  # points strictly before the origin
    kv = np.dot(half.astype(np.float64), recip)
    k2 = np.einsum("ij,ij->i", kv, kv)
    kc2 = k_cut ** 2
    keep = k2 < kc2
    near = np.abs(k2 - kc2) <= 1e-12 * kc2
    for i in np.nonzero(near)[0]:
        kk = np.dot(half[i], recip)
        keep[i] = np.dot(kk, kk) < kc2
    return np.ascontiguousarray(half.astype(np.int32)), keep


_KV_CACHE = {}      # (recip, k_max, k_cut) values -> kept k list
_KV_CACHE_MAX = 64


def effective_k_vectors(recip, k_max, k_cut):
    """Half-space integer k list kept by the reference, in its order: the
    k-vectors of ``half_space_k_vectors`` inside the cut.

    The list depends on the values of the three arguments alone; the last
    64 lists are kept (as read-only arrays), so that rebuilding an array, or
    scanning alpha at a fixed cut, does not enumerate the k grid again
    (0.65 ms of host time at K = 4,095)."""
    key = (np.asarray(recip, dtype=np.float64).tobytes(),
           tuple(int(v) for v in np.ravel(k_max)), float(k_cut))
    kv = _KV_CACHE.get(key)
    if kv is None:
        half, keep = half_space_k_vectors(recip, k_max, k_cut)
        kv = np.ascontiguousarray(half[keep])
        kv.flags.writeable = False
        if len(_KV_CACHE) >= _KV_CACHE_MAX:
            _KV_CACHE.pop(next(iter(_KV_CACHE)))
        _KV_CACHE[key] = kv
    return kv


def pmiv_is_lattice_consistent(system, pmiv, tol=1e-8):
    """True when pmiv_ij - (r_j - r_i) is a supercell translation for all
    pairs and the Ewald cell equals the supercell (no column-broadcast quirk),
    i.e. cos(k . pmiv_ij) = cos(k . r_j - k . r_i) for every kept k."""
    if not ewald_cell_matches_supercell(system):
        return False
    return lattice_deviation(system, pmiv) <= tol


def lattice_deviation(system, pmiv):
    """Largest distance (in supercell fractional units) of any
    pmiv_ij - (r_j - r_i) from a supercell translation; inf for non-finite
    input."""
    coords = np.asarray(system.neighbors.bulk_sites.cell_coordinates, np.float64)
    inv = np.asarray(system.neighbors.simulation_cell_matrix_inv, np.float64)
    pmiv = np.asarray(pmiv, dtype=np.float64)
    n = len(coords)
    if pmiv.shape != (n, n, 3):
        raise ValueError("pmiv must have shape (N, N, 3), got %r" % (pmiv.shape,))
    worst = 0.0
    chunk = max(1, 2_000_000 // max(1, n))
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        d = pmiv[s:e] - (coords[None, :, :] - coords[s:e, None, :])
        f = d.reshape(-1, 3) @ inv
        dev = np.abs(f - np.rint(f))
        if not np.all(np.isfinite(dev)):
            return float("inf")
        worst = max(worst, float(dev.max()))
    return worst


def ewald_cell_matches_supercell(system, rtol=1e-12):
    a = system.translational_matrix
    b = system.neighbors.simulation_cell_matrix
    return bool(np.allclose(a, b, rtol=rtol, atol=rtol * np.abs(b).max()))


def choose_mode(system, pmiv, requested="auto"):
    if requested != "auto":
        if requested not in nat.EWALD_MODES:
            raise ValueError("unknown Ewald precision %r" % (requested,))
        if requested != "fp64_direct":
            ok = (pmiv_is_lattice_consistent(system, pmiv) if pmiv is not None
                  else ewald_cell_matches_supercell(system))
            if not ok:
                raise ValueError(
                    "precision %r needs a lattice-consistent pmiv and an Ewald "
                    "cell equal to the supercell; use 'fp64_direct'" % requested)
        return requested
    if pmiv is not None:
        return "fp64" if pmiv_is_lattice_consistent(system, pmiv) else "fp64_direct"
    return "fp64" if ewald_cell_matches_supercell(system) else "fp64_direct"


def build_device_array(system, alpha, r_cut, k_cut, precision="auto",
                       pmiv="system", stream=None, out=None, parts=0, kvecs=None,
                       split_launch=None):
    """Build the N x N FP64 array on the current CUDA device.

    Returns ``(A, info)``: ``A`` a CUDA float64 tensor, ``info`` a dict with
    ``mode``, ``k_max``, ``n_kvec`` and the real / Fourier phase times (ms).
    ``pmiv='system'`` uses ``system.pairwise_min_image_vector_data``.
    ``parts``: a mask of ``_native.EWALD_PART_*`` (0 = the whole array).
    ``kvecs``: an explicit (K, 3) integer k list instead of the one k_cut
    selects.
    ``split_launch``: launch shape of the split modes, ``{"form": "auto" |
    "pair" | "single", "raster": super-tiles per raster block side (0 =
    default)}`` (``autotune.tune_split`` picks one); the array does not
    depend on it.
    """
    import torch
    nat.require_device()
    if isinstance(pmiv, str) and pmiv == "system":
        pmiv = system.pairwise_min_image_vector_data
    n = int(system.neighbors.num_system_elements)
    mode = choose_mode(system, pmiv, precision)
    desc, keep, k_max = make_desc(system, alpha, r_cut, k_cut, pmiv, kvecs)
    desc.parts = int(parts)
    if split_launch:
        desc.split_form = nat.SPLIT_FORMS[split_launch.get("form", "auto")]
        desc.split_raster = int(split_launch.get("raster", 0))
    dev = keep[0].device
    L = nat.lib()
    code = nat.EWALD_MODES[mode]
    ws_bytes = nat.C.c_size_t()
    nat.check(L.pycd_ewald_workspace_size(nat.C.byref(desc), code,
                                          nat.C.byref(ws_bytes)))
    ws = torch.empty(max(1, ws_bytes.value), dtype=torch.uint8, device=dev)
    if out is None:
        out = torch.empty((n, n), dtype=torch.float64, device=dev)
    rms, fms = nat.C.c_float(), nat.C.c_float()
    nat.check(L.pycd_ewald_build(nat.C.byref(desc), code, out.data_ptr(),
                                 ws.data_ptr(), ws_bytes.value,
                                 nat.stream_handle(stream), nat.C.byref(rms),
                                 nat.C.byref(fms)))
    info = {"mode": mode, "k_max": k_max, "n_kvec": int(desc.n_kvec),
            "real_ms": rms.value, "fourier_ms": fms.value}
    return out, info


def make_desc(system, alpha, r_cut, k_cut, pmiv=None, kvecs=None):
    """PycdEwaldDesc for `system` on the current CUDA device.  Returns
    (desc, tensors the descriptor points into, k_max)."""
    import torch
    n = int(system.neighbors.num_system_elements)
    k_max = k_max_for(system, k_cut)
    if kvecs is None:
        kv = effective_k_vectors(system.reciprocal_lattice_matrix, k_max, k_cut)
    else:
        kv = np.ascontiguousarray(np.asarray(kvecs, dtype=np.int32).reshape(-1, 3))
    dev = torch.device("cuda", torch.cuda.current_device())
    cart = torch.as_tensor(system.neighbors.bulk_sites.cell_coordinates,
                           dtype=torch.float64).contiguous().to(dev)
    d_pmiv = None
    if pmiv is not None:  # the real-space term uses |pmiv_ij| as given
        d_pmiv = torch.as_tensor(np.ascontiguousarray(pmiv, dtype=np.float64)
                                 ).to(dev)
    d_kv = torch.tensor(kv).to(dev) if len(kv) else torch.zeros(  # kv may be read-only
        (1, 3), dtype=torch.int32, device=dev)
    desc = nat.EwaldDesc()
    desc.n_sites = n
    desc.n_kvec = len(kv)
    desc.d_cart = cart.data_ptr()
    desc.d_pmiv = d_pmiv.data_ptr() if d_pmiv is not None else None
    desc.d_kvec = d_kv.data_ptr()
    desc.recip[:] = [float(v) for v in np.asarray(
        system.reciprocal_lattice_matrix, dtype=np.float64).ravel()]
    desc.sim_cell[:] = [float(v) for v in system.neighbors.simulation_cell_matrix.ravel()]
    desc.sim_cell_inv[:] = [float(v) for v in system.neighbors.simulation_cell_matrix_inv.ravel()]
    desc.pbc[:] = [int(v) for v in system.pbc]
    desc.alpha = float(alpha)
    desc.r_cut = float(r_cut)
    desc.volume = float(system.system_volume)
    desc.dielectric = float(system.material.dielectric_constant)
    layout = supercell_layout(system, pmiv)
    if layout is not None:
        desc.supercell[:] = layout[0]
        desc.basis_sites = layout[1]
    keep = [cart, d_kv] + ([d_pmiv] if d_pmiv is not None else [])
    return desc, keep, k_max


def supercell_layout(system, pmiv=None, tol=1e-6):
    """((s0, s1, s2), n_basis) when site i is basis site i % n_basis of cell
    i // n_basis (cells in C order, the last index fastest), every site
    sits at its unit-cell position plus its cell's translation (to `tol`
    bohr), the Ewald cell is that supercell and any given pmiv is
    lattice-consistent; otherwise None.  The array is then translation
    invariant and its real-space rows repeat with the cells."""
    if not ewald_cell_matches_supercell(system):
        return None
    if pmiv is not None and not pmiv_is_lattice_consistent(system, pmiv):
        return None
    m = system.material
    uc = np.asarray(m.cartesian_unit_cell_coords, dtype=np.float64)
    ss = np.asarray(system.system_size, dtype=int)
    cart = np.asarray(system.neighbors.bulk_sites.cell_coordinates, dtype=np.float64)
    nb = len(uc)
    if nb == 0 or len(cart) != nb * int(np.prod(ss)):
        return None
    # cell indices in C order, as doubles (an integer matmul misses BLAS);
    # translation + basis position, site by site, as one contiguous addition
    cells = np.indices(tuple(int(v) for v in ss), dtype=np.float64).reshape(3, -1).T
    trans = cells @ np.asarray(m.lattice_matrix, dtype=np.float64)
    want = np.repeat(trans, nb, axis=0) + np.tile(uc, (len(trans), 1))
    if np.abs(want - cart).max() > tol:
        return None
    return [int(v) for v in ss], int(nb)


def hop_energy_error(A_ref, A, nbr, n_carriers, n_dopants, samples=4096, seed=0,
                     carrier_charge=-1.0, dopant_charge=1.0):
    """Error of the hop energy dE0 (PyCD/core.py:2004-2026) computed from the
    array ``A`` instead of ``A_ref`` (both CUDA (N, N) float64), over
    ``samples`` seeded charge configurations of ``n_carriers`` carriers and
    ``n_dopants`` fixed dopants on distinct sites, each with one hop of a
    carrier from its site o to a neighbour n = nbr[o, s] (``nbr``: (N, S)
    int array, -1 for no neighbour):

        dE0 = 2 q_s [sum_j q_j (A[n, j] - A[o, j]) + q_s (A[o, o] - A[o, n])]
              + E_rel[n] - E_rel[o]

    with q holding every charge before the move.  E_rel cancels.  Returns
    (max, rms) of |dE0(A) - dE0(A_ref)| in Hartree."""
    import torch
    nbr = np.asarray(nbr)
    n = nbr.shape[0]
    rng = np.random.default_rng(seed)
    m = n_carriers + n_dopants
    sites = np.stack([rng.choice(n, size=m, replace=False) for _ in range(samples)])
    q = np.concatenate([np.full(n_carriers, carrier_charge),
                        np.full(n_dopants, dopant_charge)])
    o = sites[np.arange(samples), rng.integers(0, n_carriers, samples)]
    slots = nbr[o]
    pick = np.array([rng.choice(np.nonzero(r >= 0)[0]) for r in slots])
    dst = slots[np.arange(samples), pick]
    dev = A.device
    t = lambda a: torch.as_tensor(a, device=dev)
    S, O, D, Q = t(sites), t(o), t(dst), t(q)

    def de(M):
        rows_n = M[D[:, None], S]          # A[n, j] at the charged sites
        rows_o = M[O[:, None], S]
        term = (Q[None, :] * (rows_n - rows_o)).sum(1)
        return 2 * carrier_charge * (term + carrier_charge * (M[O, O] - M[O, D]))

    err = (de(A) - de(A_ref)).abs()
    return float(err.max().item()), float(err.square().mean().sqrt().item())
