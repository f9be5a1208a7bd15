"""Host-side lattice setup: ``Material`` and ``Neighbors``.

These classes define the site order that is the index order of the
precomputed Ewald array, and they produce the hop-neighbor tables that the
KMC kernels consume.  Their public attributes and methods mirror
PyCD/core.py:37-241 (``Material``) and PyCD/core.py:244-668 (``Neighbors``).
The all-pairs work is vectorised NumPy; the minimum-image choice and the
hop-distance windows are re-evaluated with the reference's per-vector
arithmetic wherever a vectorised comparison is within rounding of a tie, so
that neighbour indices and displacement vectors come out as the reference's.
"""
import itertools
from collections import defaultdict
from datetime import datetime
from pathlib import Path

import numpy as np

from . import constants
from .io import read_poscar, generate_report


class ReturnValues(object):
    """Attribute bag (PyCD/core.py:3457-3462)."""

    def __init__(self, *args, **kwargs):
        if args:
            (input_dict,) = args
            kwargs = dict(input_dict, **kwargs)
        for key, value in kwargs.items():
            setattr(self, key, value)


class Material(object):
    """Material parameters and unit-cell sites (PyCD/core.py:37-152).

    Sites of each element type are re-ordered by ascending fractional z
    (core.py:85-97, NumPy's default ``argsort``), which fixes the index
    order of every per-site array downstream.
    """

    def __init__(self, material_parameters):
        poscar = read_poscar(material_parameters.input_coord_file_location)
        self.lattice_matrix = poscar["lattice_matrix"]
        self.element_types = poscar["element_types"]
        self.n_elements_per_unit_cell = poscar["num_elements"]
        self.total_elements_per_unit_cell = poscar["total_elements"]
        coords = poscar["coordinates"]
        if poscar["coordinate_type"] == "Direct":
            frac = coords
        elif poscar["coordinate_type"] == "Cartesian":
            frac = np.dot(coords, np.linalg.inv(self.lattice_matrix))
        else:
            raise ValueError("unknown POSCAR coordinate type %r"
                             % poscar["coordinate_type"])
        self.lattice_matrix *= constants.ANG2BOHR
        self.num_element_types = len(self.element_types)
        self.element_type_index_list = np.repeat(
            np.arange(self.num_element_types), self.n_elements_per_unit_cell)
        p = material_parameters
        self.name = p.name
        self.species_types = p.species_types[:]
        self.num_species_types = len(self.species_types)
        self.species_charge_list = p.species_charge_list
        self.species_to_element_type_map = {
            k: v for k, v in p.species_to_element_type_map.items()}

        self.fractional_unit_cell_coords = np.zeros(frac.shape)
        self.unit_cell_class_list = []
        start = 0
        for et_index in range(self.num_element_types):
            et_frac = frac[self.element_type_index_list == et_index]
            order = et_frac[:, 2].argsort()
            end = start + self.n_elements_per_unit_cell[et_index]
            self.fractional_unit_cell_coords[start:end] = et_frac[order]
            et = self.element_types[et_index]
            self.unit_cell_class_list.extend(
                [p.class_list[et][i] - 1 for i in order])
            start = end
        self.cartesian_unit_cell_coords = np.dot(
            self.fractional_unit_cell_coords, self.lattice_matrix)
        self.charge_types = p.charge_types
        self.vn = p.vn / constants.SEC2AUTIME

        def _scale(table, factor, keep_none=False):
            out = {}
            for key, class_values in table.items():
                out[key] = [[(v * factor if v else None) if keep_none
                             else v * factor for v in values]
                            for values in class_values]
            return out

        self.lambda_values = _scale(p.lambda_values, constants.EV2HARTREE)
        self.v_ab = _scale(p.v_ab, constants.EV2HARTREE)
        self.neighbor_cutoff_dist = _scale(
            p.neighbor_cutoff_dist, constants.ANG2BOHR, keep_none=True)
        self.neighbor_cutoff_dist_tol = _scale(
            p.neighbor_cutoff_dist_tol, constants.ANG2BOHR, keep_none=True)
        self.num_unique_hopping_distances = {
            key: [len(v) for v in class_values]
            for key, class_values in self.neighbor_cutoff_dist.items()}
        self.element_type_delimiter = p.element_type_delimiter
        self.dielectric_constant = p.dielectric_constant
        self.num_classes = [len(set(p.class_list[et]))
                            for et in self.element_types]
        self.element_type_to_species_map = defaultdict(list)
        for et in self.element_types:
            for sp in self.species_types:
                if et in self.species_to_element_type_map[sp]:
                    self.element_type_to_species_map[et].append(sp)
        self.hop_element_types = {
            sp: [self.element_type_delimiter.join(c) for c in
                 itertools.product(self.species_to_element_type_map[sp],
                                   repeat=2)]
            for sp in self.species_types}

    def generate_sites(self, element_type_indices, cell_size):
        """Supercell sites, cell-major with the z cell index fastest
        (PyCD/core.py:154-241)."""
        cell_size = np.asarray(cell_size)
        assert all(s > 0 for s in cell_size), "cell size must be positive"
        element_type_indices = list(element_type_indices)
        extract = np.isin(self.element_type_index_list,
                          element_type_indices).nonzero()[0]
        uc_coords = self.cartesian_unit_cell_coords[extract]
        num_cells = int(cell_size.prod())
        n_per_cell = int(self.n_elements_per_unit_cell[
            element_type_indices].sum())
        uc_type = np.concatenate(
            [np.full(self.n_elements_per_unit_cell[e], e)
             for e in element_type_indices]).reshape(n_per_cell, 1)
        uc_elem = np.concatenate(
            [np.arange(self.n_elements_per_unit_cell[e])
             for e in element_type_indices]).reshape(n_per_cell, 1)
        gx, gy, gz = np.meshgrid(np.arange(cell_size[0]),
                                 np.arange(cell_size[1]),
                                 np.arange(cell_size[2]), indexing="ij")
        cells = np.column_stack((gx.ravel(), gy.ravel(), gz.ravel()))
        translations = np.dot(cells, self.lattice_matrix)
        coords = (uc_coords[np.newaxis, :, :]
                  + translations[:, np.newaxis, :]).reshape(-1, 3)
        quantum = np.zeros((num_cells * n_per_cell, 5), dtype=int)
        quantum[:, :3] = np.repeat(cells, n_per_cell, axis=0)
        quantum[:, 3] = np.tile(uc_type[:, 0], num_cells)
        quantum[:, 4] = np.tile(uc_elem[:, 0], num_cells)
        return ReturnValues(
            cell_coordinates=coords,
            quantum_index_list=quantum,
            system_element_index_list=np.arange(num_cells * n_per_cell))


def _ref_norm(v):
    return np.linalg.norm(v)


class Neighbors(object):
    """Supercell, minimum-image convention and hop-neighbour lists
    (PyCD/core.py:244-668)."""

    # pairs whose best and runner-up image distances, or whose distance and
    # a window edge, agree to this relative margin are re-evaluated with the
    # reference's per-vector arithmetic
    _TIE_RTOL = 1e-12

    def __init__(self, material, system_size, pbc):
        self.start_time = datetime.now()
        self.material = material
        self.system_size = np.asarray(system_size)
        self.n_dim = len(self.system_size)
        self.pbc = np.asarray(pbc)[:]
        self.num_cells = self.system_size.prod()
        self.num_system_elements = int(
            self.num_cells * self.material.total_elements_per_unit_cell)
        self.element_type_indices = range(self.material.num_element_types)
        self.bulk_sites = self.material.generate_sites(
            self.element_type_indices, self.system_size)
        rng = [range(-1, 2) if self.pbc[d] == 1 else [0] for d in range(3)]
        vecs = []
        for x in rng[0]:
            for y in rng[1]:
                for z in rng[2]:
                    vecs.append(np.dot(np.multiply(np.array([x, y, z]),
                                                   self.system_size),
                                       self.material.lattice_matrix))
        self.system_translational_vector_list = np.array(vecs)
        self.simulation_cell_matrix = (self.material.lattice_matrix
                                       * self.system_size[:, np.newaxis])
        self.simulation_cell_matrix_inv = np.linalg.inv(
            self.simulation_cell_matrix)
        self.pbc_mask = np.array(self.pbc, dtype=bool)
        deltas = []
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    if dx == 0 and dy == 0 and dz == 0:
                        continue
                    d = np.array([dx if self.pbc_mask[0] else 0,
                                  dy if self.pbc_mask[1] else 0,
                                  dz if self.pbc_mask[2] else 0])
                    if np.any(d != 0):
                        deltas.append(d)
        # image offsets in the reference's search order (core.py:324-341)
        self._image_deltas = np.array(deltas, dtype=np.float64).reshape(-1, 3)

    # -- minimum image -----------------------------------------------------
    def apply_minimum_image_convention(self, displacement_vector):
        """Single-vector minimum image, as PyCD/core.py:304-361."""
        return self.apply_minimum_image_convention_vectorized(
            np.asarray(displacement_vector, dtype=np.float64)[None, :])[0]

    def apply_minimum_image_convention_vectorized(self, displacement_vectors,
                                                  tie_check_below=None):
        """Minimum-image vectors for an (n, 3) array.

        Candidates are the rounded fractional image and its 26 neighbours in
        the reference's scan order; the first strictly shorter candidate
        wins.  Distances are compared vectorised, then every row whose
        decision is within rounding of a tie is redone with the per-vector
        norm the reference uses, so the chosen image is the reference's.
        ``tie_check_below``: only rows shorter than this are redone (callers
        that only keep short vectors, such as the hop-neighbour windows).
        """
        M = self.simulation_cell_matrix
        D = np.asarray(displacement_vectors, dtype=np.float64)
        frac = np.dot(D, self.simulation_cell_matrix_inv)
        base = np.zeros_like(frac)
        base[:, self.pbc_mask] = -np.round(frac[:, self.pbc_mask])
        best = np.dot(frac + base, M)
        best_d = np.sqrt(np.einsum("ij,ij->i", best, best))
        second_gap = np.full(len(D), np.inf)
        for delta in self._image_deltas:
            cand = np.dot(frac + (base + delta), M)
            cd = np.sqrt(np.einsum("ij,ij->i", cand, cand))
            gap = np.abs(cd - best_d)
            better = cd < best_d
            second_gap = np.minimum(second_gap, gap)
            best = np.where(better[:, None], cand, best)
            best_d = np.where(better, cd, best_d)
        close = second_gap <= self._TIE_RTOL * np.maximum(best_d, 1e-300)
        if tie_check_below is not None:
            close &= best_d <= tie_check_below
        for i in np.nonzero(close)[0]:
            best[i] = self._min_image_exact(D[i])
        return best

    def _min_image_exact(self, dv):
        M = self.simulation_cell_matrix
        frac = np.dot(dv, self.simulation_cell_matrix_inv)
        base = np.zeros(3)
        base[self.pbc_mask] = -np.round(frac[self.pbc_mask])
        best = np.dot(frac + base, M)
        best_d = _ref_norm(best)
        for delta in self._image_deltas:
            cand = np.dot(frac + (base + delta), M)
            cd = _ref_norm(cand)
            if cd < best_d:
                best_d, best = cd, cand
        return best

    def _max_hop(self):
        """Longest hop-window edge over all element pairs (bohr), with slack."""
        m = self.material
        edges = [d + t for key, cls in m.neighbor_cutoff_dist.items()
                 for ci, ds in enumerate(cls) for d, t in
                 zip(ds, m.neighbor_cutoff_dist_tol[key][ci]) if d is not None]
        return (max(edges) if edges else 0.0) * (1 + 1e-6)

    # -- index maps (PyCD/core.py:363-466) ---------------------------------
    def get_system_element_index(self, system_size, quantum_indices):
        q = np.asarray(quantum_indices)
        m = self.material
        idx = int(q[4] + m.n_elements_per_unit_cell[:q[3]].sum())
        n_dim = len(system_size)
        for k in range(n_dim):
            stride = m.total_elements_per_unit_cell
            if k:
                stride = stride * np.asarray(system_size)[-k:].prod()
            idx += int(stride * q[n_dim - 1 - k])
        return idx

    def get_quantum_indices(self, system_size, system_element_index):
        m = self.material
        q = np.zeros(5, dtype=int)
        uc = system_element_index % m.total_elements_per_unit_cell
        q[3] = np.where(m.n_elements_per_unit_cell.cumsum() >= uc + 1)[0][0]
        q[4] = uc - m.n_elements_per_unit_cell[:q[3]].sum()
        cells = (system_element_index - uc) // m.total_elements_per_unit_cell
        ss = np.asarray(system_size)
        for k in range(3):
            stride = int(ss[k + 1:].prod())
            q[k] = cells // stride
            cells -= q[k] * stride
        return q

    def get_coordinates(self, system_size, system_element_index):
        q = self.get_quantum_indices(system_size, system_element_index)
        m = self.material
        return (np.dot(q[:3], m.lattice_matrix)
                + m.cartesian_unit_cell_coords[
                    q[4] + m.n_elements_per_unit_cell[:q[3]].sum()])

    def compute_distance(self, system_size, i, j):
        d = (self.get_coordinates(system_size, j)
             - self.get_coordinates(system_size, i))
        return _ref_norm(self._min_image_exact(d))

    # -- hop neighbours (PyCD/core.py:485-569, 596-668) --------------------
    def hop_neighbor_sites(self, bulk_sites, center_site_indices,
                           neighbor_site_indices, cutoff_dist_limits,
                           cutoff_dist_key=None, _cache=None):
        """Neighbours of every centre site within the window
        ``lo < |d| <= hi``, in neighbour-scan order."""
        nb_coords = bulk_sites.cell_coordinates[neighbor_site_indices]
        nb_sei = bulk_sites.system_element_index_list[neighbor_site_indices]
        c_coords = bulk_sites.cell_coordinates[center_site_indices]
        lo, hi = cutoff_dist_limits
        n_c = len(c_coords)
        nbr_idx = np.empty(n_c, dtype=object)
        disp = np.empty(n_c, dtype=object)
        counts = np.zeros(n_c, dtype=int)
        chunk = max(1, int(4_000_000 // max(1, len(nb_coords))))
        for s in range(0, n_c, chunk):
            e = min(n_c, s + chunk)
            if _cache is not None and (s, e) in _cache:
                mi, dist = _cache[(s, e)]
            else:
                D = (nb_coords[None, :, :] - c_coords[s:e, None, :])
                mi = self.apply_minimum_image_convention_vectorized(
                    D.reshape(-1, 3), tie_check_below=self._max_hop()
                ).reshape(e - s, len(nb_coords), 3)
                dist = np.sqrt(np.einsum("ijk,ijk->ij", mi, mi))
                if _cache is not None:
                    _cache[(s, e)] = (mi, dist)
            sel = (lo < dist) & (dist <= hi)
            tol = self._TIE_RTOL * hi
            edge = (np.abs(dist - lo) <= tol) | (np.abs(dist - hi) <= tol)
            for r, c in zip(*np.nonzero(edge)):
                d = _ref_norm(mi[r, c])
                sel[r, c] = lo < d <= hi
            for r in range(e - s):
                cols = np.nonzero(sel[r])[0]
                nbr_idx[s + r] = nb_sei[cols]
                disp[s + r] = np.asarray([mi[r, c] for c in cols]) \
                    if len(cols) else np.asarray([])
                counts[s + r] = len(cols)
        return ReturnValues(neighbor_system_element_indices=nbr_idx,
                            displacement_vector_list=disp,
                            num_neighbors=counts)

    def get_pairwise_min_image_vector_data(self, dst_path=None):
        """All-pairs minimum-image vectors (N x N x 3, bohr); written to
        ``pairwise_min_image_vector_data.npy`` when ``dst_path`` is given
        (PyCD/core.py:571-594)."""
        coords = self.bulk_sites.cell_coordinates
        n = len(coords)
        out = np.zeros((n, n, 3))
        chunk = max(1, int(4_000_000 // max(1, n)))
        for s in range(0, n, chunk):
            e = min(n, s + chunk)
            D = coords[None, :, :] - coords[s:e, None, :]
            out[s:e] = self.apply_minimum_image_convention_vectorized(
                D.reshape(-1, 3)).reshape(e - s, n, 3)
        if dst_path is not None:
            np.save(Path(dst_path) / "pairwise_min_image_vector_data.npy", out)
            return None
        return out

    def _translated_neighbor_sites(self, idx, lo, hi):
        """Hop neighbours of every centre site in `idx` from those of the
        unit-cell centres, by supercell translation (fully periodic cells).

        Candidates come from translation invariance; each kept pair's vector
        is then computed with the same minimum-image arithmetic as the full
        scan and the window re-tested, so indices and vectors are the full
        scan's.  Returns None when a unit-cell distance lies within rounding
        of a window edge (the caller then uses the full scan)."""
        m = self.material
        tpc = int(m.total_elements_per_unit_cell)
        ss = self.system_size
        coords = self.bulk_sites.cell_coordinates
        n_idx = len(idx)
        per_cell = n_idx // int(self.num_cells)
        uc_idx = idx[:per_cell]
        D = coords[idx][None, :, :] - coords[uc_idx][:, None, :]
        mi = self.apply_minimum_image_convention_vectorized(
            D.reshape(-1, 3), tie_check_below=hi * (1 + 1e-6)
        ).reshape(per_cell, n_idx, 3)
        dist = np.sqrt(np.einsum("ijk,ijk->ij", mi, mi))
        tol = 1e-9 * hi
        if np.any((np.abs(dist - lo) <= tol) | (np.abs(dist - hi) <= tol)):
            return None
        sel = (lo < dist) & (dist <= hi)
        counts = sel.sum(axis=1)
        cells = self.bulk_sites.quantum_index_list[idx, :3]
        # neighbour j of unit-cell centre b, seen from a centre in cell c
        out_idx = np.empty(n_idx, dtype=object)
        out_vec = np.empty(n_idx, dtype=object)
        out_cnt = np.zeros(n_idx, dtype=int)
        centre_b = np.arange(n_idx) % per_cell
        all_pairs = []
        for b in range(per_cell):
            nbr = idx[np.nonzero(sel[b])[0]]
            nbr_cell = self.bulk_sites.quantum_index_list[nbr, :3]
            nbr_off = nbr - (((nbr_cell[:, 0] * ss[1] + nbr_cell[:, 1]) * ss[2]
                              + nbr_cell[:, 2]) * tpc)
            centres = np.nonzero(centre_b == b)[0]
            cc = cells[centres]
            shifted = (cc[:, None, :] + nbr_cell[None, :, :]) % ss
            flat = (((shifted[..., 0] * ss[1] + shifted[..., 1]) * ss[2]
                     + shifted[..., 2]) * tpc + nbr_off[None, :])
            flat.sort(axis=1)
            all_pairs.append((centres, flat))
        for centres, flat in all_pairs:
            ci = idx[centres]
            D = coords[flat] - coords[ci][:, None, :]
            v = self.apply_minimum_image_convention_vectorized(
                D.reshape(-1, 3), tie_check_below=hi * (1 + 1e-6)
            ).reshape(flat.shape + (3,))
            dd = np.sqrt(np.einsum("ijk,ijk->ij", v, v))
            if not np.all((lo < dd) & (dd <= hi)):
                return None
            for r, c in enumerate(centres):
                out_idx[c] = flat[r]
                out_vec[c] = v[r]
                out_cnt[c] = flat.shape[1]
        return ReturnValues(neighbor_system_element_indices=out_idx,
                            displacement_vector_list=out_vec,
                            num_neighbors=out_cnt)

    def generate_neighbor_list(self, dst_path, local_system_size=(3, 3, 3),
                               save=True, method="auto"):
        """Hop-neighbour dictionary keyed by 'A:B' element pair, then class,
        then hop-distance type; saved as ``hop_neighbor_list.npy``.

        ``method='scan'`` scans all centre/neighbour pairs like the
        reference; ``'auto'`` uses supercell translations for fully periodic
        cells (same result, O(N) instead of O(N^2)) and falls back to the
        scan wherever that cannot be confirmed."""
        assert all(s >= 3 for s in local_system_size), \
            "local system size must be >= 3 in every dimension"
        m = self.material
        hop_neighbor_list = {}
        sites = self.bulk_sites
        periodic = bool(np.all(self.pbc_mask))
        for key, class_lists in m.neighbor_cutoff_dist.items():
            center_type = key.split(m.element_type_delimiter)[0]
            ct = m.element_types.index(center_type)
            offsets = np.repeat(
                np.arange(0, m.total_elements_per_unit_cell * self.num_cells,
                          m.total_elements_per_unit_cell),
                m.n_elements_per_unit_cell[ct])
            idx = (np.tile(m.n_elements_per_unit_cell[:ct].sum()
                           + np.arange(m.n_elements_per_unit_cell[ct]),
                           self.num_cells) + offsets)
            cache = {}
            per_class = []
            for ci, dists in enumerate(class_lists):
                per_type = []
                for ti, dist in enumerate(dists):
                    tol = m.neighbor_cutoff_dist_tol[key][ci][ti]
                    lo, hi = dist - tol, dist + tol
                    fast = None
                    if method == "auto" and periodic:
                        fast = self._translated_neighbor_sites(idx, lo, hi)
                    per_type.append(fast if fast is not None else
                                    self.hop_neighbor_sites(
                                        sites, idx, idx, [lo, hi], key,
                                        _cache=cache))
                per_class.append(per_type)
            hop_neighbor_list[key] = per_class
        if save:
            Path(dst_path).mkdir(parents=True, exist_ok=True)
            np.save(Path(dst_path) / "hop_neighbor_list.npy",
                    hop_neighbor_list)
            generate_report(self.start_time, Path(dst_path), "neighbor_list", 1)
        return hop_neighbor_list
