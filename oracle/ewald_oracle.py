"""ORACLE (test infrastructure only) - CPU restatement of PyCD's Ewald
precomputed array.  Never imported by the product package; used by tests/,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` leg of bench.py as the
checker.

Pinned: ``precomputed_array`` reproduces the reference's shipped
examples/Hematite and examples/BVO arrays (tests/golden, built by
tests/golden/make_golden.py) and the reference's own build of the 324-site
corundum lattice.

Functions follow, in NumPy:
  real_space         PyCD/core.py:799-814 then / eps (core.py:1594-1596)
  effective_k_vectors PyCD/core.py:816-838
  fourier_space      PyCD/core.py:853-878 then / eps (core.py:1598-1602)
  self_term          PyCD/core.py:1659
  precomputed_array  PyCD/core.py:1624-1661
  class_array        the same formula evaluated once per translation class
                     (site pair up to a supercell translation), for N where
                     the all-pairs form is too slow
"""
import numpy as np
from scipy.special import erfc


def real_space(pmiv, alpha, r_cut, eps):
    n = pmiv.shape[0]
    out = np.zeros((n, n))
    dr = np.linalg.norm(pmiv, axis=2)
    inside = dr < r_cut
    out[inside] += erfc(np.sqrt(alpha) * dr[inside]) / 2
    np.fill_diagonal(dr, 1)
    out[inside] /= dr[inside]
    return out / eps


def effective_k_vectors(k_max):
    """All integer triples in [-k_max, k_max]^3 except 0, C order, keeping the
    first member of each +-pair."""
    grid = np.mgrid[-k_max[0]:k_max[0] + 1, -k_max[1]:k_max[1] + 1,
                    -k_max[2]:k_max[2] + 1].reshape(3, -1).T
    kept, seen = [], set()
    for v in grid:
        t = tuple(v)
        if t == (0, 0, 0):
            continue
        if t not in seen:
            kept.append(v)
            seen.add(tuple(-v))
    return np.array(kept)


def k_max_for(k_cut, recip):
    return np.ceil(k_cut / np.linalg.norm(recip, axis=1)).astype(int)


def fourier_space(pmiv, recip, volume, alpha, k_cut, eps):
    n = pmiv.shape[0]
    out = np.zeros((n, n))
    a4 = 4 * alpha
    coeff = (2 * np.pi) / volume
    kc2 = k_cut ** 2
    for kv in effective_k_vectors(k_max_for(k_cut, recip)):
        k = np.dot(kv, recip)
        k2 = np.dot(k, k)
        if k2 < kc2:
            out += (coeff * np.exp(-k2 / a4)
                    * np.cos(np.tensordot(pmiv, k, axes=([2], [0]))) / k2)
    out *= 2
    return out / eps


def self_term(n, alpha, eps):
    return -np.eye(n) * np.sqrt(alpha / np.pi) / eps


def precomputed_array(pmiv, recip, volume, alpha, r_cut, k_cut, eps):
    n = pmiv.shape[0]
    return (real_space(pmiv, alpha, r_cut, eps)
            + fourier_space(pmiv, recip, volume, alpha, k_cut, eps)
            + self_term(n, alpha, eps))


def ewald_geometry(lattice_bohr, system_size):
    """Ewald cell, volume and reciprocal basis as PyCD/core.py:709-724
    (column-broadcast supercell kept)."""
    T = np.multiply(np.asarray(system_size), lattice_bohr)
    vol = abs(np.dot(T[0], np.cross(T[1], T[2])))
    recip = 2 * np.pi / vol * np.array([np.cross(T[1], T[2]),
                                        np.cross(T[2], T[0]),
                                        np.cross(T[0], T[1])])
    return T, vol, recip


def min_image(d, cell, cell_inv, pbc=(1, 1, 1)):
    """Vectorised minimum image: nearest fractional image then its 26
    neighbours, first strictly shorter wins (PyCD/core.py:304-361)."""
    f = d @ cell_inv
    base = np.zeros_like(f)
    pm = np.asarray(pbc, bool)
    base[:, pm] = -np.round(f[:, pm])
    best = (f + base) @ cell
    bd = np.einsum("ij,ij->i", best, best)
    for dx in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dz in (-1, 0, 1):
                o = np.array([dx, dy, dz]) * pm
                if not o.any():
                    continue
                c = (f + base + o) @ cell
                cd = np.einsum("ij,ij->i", c, c)
                better = cd < bd
                best[better] = c[better]
                bd[better] = cd[better]
    return best


def class_array(uc_cart, lattice_bohr, system_size, alpha, r_cut, k_cut, eps,
                rows=None):
    """A for a periodic supercell whose Ewald cell equals the supercell
    (s_i = s_j wherever lattice[i][j] != 0), from the same formula as
    ``precomputed_array`` evaluated on the minimum-image vector of every
    translation class; returns the full N x N array (or the given rows)."""
    ss = np.asarray(system_size)
    nb = len(uc_cart)
    T, vol, recip = ewald_geometry(lattice_bohr, ss)
    cell = lattice_bohr * ss[:, None]
    cell_inv = np.linalg.inv(cell)
    cells = np.stack(np.meshgrid(np.arange(ss[0]), np.arange(ss[1]),
                                 np.arange(ss[2]), indexing="ij"), -1).reshape(-1, 3)
    nc = len(cells)
    n = nc * nb
    # class vectors: site b2 in cell c relative to site b1 in cell 0
    trans = cells @ lattice_bohr
    d = (uc_cart[None, None, :, :] + trans[None, :, None, :]
         - uc_cart[:, None, None, :]).reshape(-1, 3)
    d = min_image(d, cell, cell_inv)
    dr = np.linalg.norm(d, axis=1)
    real = np.zeros(len(d))
    inside = dr < r_cut
    safe = np.where(dr > 0, dr, 1.0)
    real[inside] = erfc(np.sqrt(alpha) * dr[inside]) / 2 / safe[inside]
    real /= eps
    kv = effective_k_vectors(k_max_for(k_cut, recip))
    k = kv @ recip
    k2 = np.einsum("ij,ij->i", k, k)
    keep = k2 < k_cut ** 2
    k, k2 = k[keep], k2[keep]
    w = 2 * (2 * np.pi / vol) * np.exp(-k2 / (4 * alpha)) / k2 / eps
    four = np.zeros(len(d))
    for s in range(0, len(k), 256):
        four += np.cos(d @ k[s:s + 256].T) @ w[s:s + 256]
    vals = (real + four).reshape(nb, nc, nb)
    # A[(c1, b1), (c2, b2)] = vals[b1, (c2 - c1) mod ss, b2]
    if rows is None:
        rows = np.arange(n)
    rows = np.asarray(rows)
    c1 = cells[rows // nb]
    b1 = rows % nb
    out = np.empty((len(rows), n))
    for r, (cc, bb) in enumerate(zip(c1, b1)):
        rel = (cells - cc) % ss
        ci = (rel[:, 0] * ss[1] + rel[:, 1]) * ss[2] + rel[:, 2]
        out[r] = vals[bb][ci].reshape(-1)
    diag = rows
    out[np.arange(len(rows)), diag] += -np.sqrt(alpha / np.pi) / eps
    return out
