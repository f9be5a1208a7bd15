"""Drop-in ``Material`` / ``Neighbors`` / ``System`` / ``Run`` for the PyCD
lattice-KMC hot path.

``System.get_precomputed_array`` (PyCD/core.py:1611-1679) builds the N x N
FP64 Ewald array on the GPU; ``Run.do_kmc_steps`` (PyCD/core.py:2647-2917)
runs every trajectory in the GPU KMC kernel and writes the reference's output
files.  Host code here only prepares tables, restores the per-trajectory
MT19937 streams (``random``, as PyCD/core.py:2566-2580, 2694-2695) and writes
files; there is no CPU compute path.
"""
import pickle
import random as rnd
from datetime import datetime
from pathlib import Path

import numpy as np

from . import constants
from . import _native as nat
from .ewald_params import EwaldParameterSearch
from .io import generate_report
from .lattice import Material, Neighbors, ReturnValues  # noqa: F401


def _numeric(v):
    return not isinstance(v, str) and bool(np.isreal(v))


class _Mt19937Stream(object):
    """The values ``random.random()`` would return from one CPython MT19937
    state, drawn in blocks: NumPy's MT19937 gives the same 32-bit outputs,
    combined as CPython's 53-bit ``random()`` ((a >> 5) 2^26 + (b >> 6)) / 2^53.
    ``state()`` is the CPython state after the values marked ``used``."""

    def __init__(self, state):
        self.bg = np.random.MT19937()
        self.bg.state = {"bit_generator": "MT19937",
                         "state": {"key": np.asarray(state[1][:624], np.uint32),
                                   "pos": int(state[1][624])}}
        self.gauss = state[2]
        self.block_start = self.bg.state
        self.consumed = 0  # values used since block_start

    def fill(self, out):
        """Write the next len(out) values into `out`; they become the block
        that ``used`` counts from."""
        self.block_start = self.bg.state
        self.consumed = 0
        raw = self.bg.random_raw(2 * len(out))
        a = (raw[0::2] >> np.uint64(5)).astype(np.float64)
        b = (raw[1::2] >> np.uint64(6)).astype(np.float64)
        out[:] = (a * 67108864.0 + b) / 9007199254740992.0

    def used(self, n):
        self.consumed += int(n)

    def state(self):
        bg = np.random.MT19937()
        bg.state = self.block_start
        if self.consumed:
            bg.random_raw(2 * self.consumed)
        st = bg.state["state"]
        return (3, tuple(int(x) for x in st["key"]) + (int(st["pos"]),), self.gauss)


class System(EwaldParameterSearch):
    """Ewald geometry and parameters (PyCD/core.py:671-797); the automatic
    parameter choices of PyCD/core.py:913-1592 come from EwaldParameterSearch."""

    def __init__(self, material_info, material_neighbors, hop_neighbor_list,
                 pairwise_min_image_vector_data, alpha, r_cut, k_cut,
                 precision_parameters=None, step_system_size_array=(),
                 step_hop_neighbor_master_list=()):
        self.start_time = datetime.now()
        self.material = material_info
        self.neighbors = material_neighbors
        self.hop_neighbor_list = hop_neighbor_list
        self.step_system_size_array = step_system_size_array
        self.step_hop_neighbor_master_list = step_hop_neighbor_master_list
        self.pbc = self.neighbors.pbc
        self.system_size = self.neighbors.system_size
        self.num_cells = self.system_size.prod()
        self.pairwise_min_image_vector_data = pairwise_min_image_vector_data
        # launch shape of the split-precision builds (None: the library's
        # default; autotune.tune_split sets a timed choice)
        self.split_launch = None
        # Ewald cell: np.multiply(system_size, lattice) scales COLUMNS
        # (core.py:709-710); it equals the supercell only when s_i = s_j
        # wherever lattice[i][j] != 0.  Kept as the reference has it.
        self.translational_matrix = np.multiply(self.system_size,
                                                self.material.lattice_matrix)
        T = self.translational_matrix
        self.system_volume = abs(np.dot(T[0], np.cross(T[1], T[2])))
        self.reciprocal_lattice_matrix = (
            2 * np.pi / self.system_volume
            * np.array([np.cross(T[1], T[2]), np.cross(T[2], T[0]),
                        np.cross(T[0], T[1])]))
        self.translational_vector_length = np.linalg.norm(T, axis=1)
        self.reciprocal_lattice_vector_length = np.linalg.norm(
            self.reciprocal_lattice_matrix, axis=1)
        self.system_class_index_list = np.tile(
            self.material.unit_cell_class_list, self.num_cells)
        m = self.material
        self.num_neighbors = np.zeros(m.num_species_types, int)
        for si, sp in enumerate(m.species_types):
            key = m.hop_element_types[sp][0]
            if key in m.neighbor_cutoff_dist and hop_neighbor_list is not None \
                    and key in hop_neighbor_list:
                for t in range(len(m.neighbor_cutoff_dist[key][0])):
                    self.num_neighbors[si] += \
                        hop_neighbor_list[key][0][t].num_neighbors[0]
        # alpha, r_cut, k_cut unit conversions (core.py:767-784); alpha is
        # used as eta^2 in bohr^-2 throughout
        self.alpha = alpha / constants.ANG2BOHR if np.isreal(alpha) else alpha
        self.r_cut = r_cut * constants.ANG2BOHR if np.isreal(r_cut) else r_cut
        if isinstance(k_cut, list):
            self.k_cut = k_cut
        elif np.isreal(k_cut):
            self.k_cut = k_cut / constants.ANG2BOHR
        else:
            self.k_cut = k_cut
        self.precision_parameters = precision_parameters
        if precision_parameters is not None:
            self._load_precision_parameters(precision_parameters)
        self.last_build_info = None

    def _user_specified(self):
        return (_numeric(self.alpha) and _numeric(self.r_cut)
                and (isinstance(self.k_cut, list) or _numeric(self.k_cut)))

    def _ewald_parameters(self):
        """Numeric alpha / r_cut / k_cut: user-specified, or a k_max list as
        core.py:1377-1382, or the result of the automatic selection
        (get_ewald_parameters, run once and kept)."""
        if not self._user_specified():
            chosen = getattr(self, "_chosen_parameters", None)
            if chosen is None:
                raise ValueError("automatic Ewald parameters are chosen by "
                                 "get_precomputed_array(dst_path, ...) first")
            return chosen
        if isinstance(self.k_cut, list):
            k_cut = 1.10 * max(np.asarray(self.k_cut)
                               * self.reciprocal_lattice_vector_length)
            choice = "user-specified (k_max)"
        else:
            k_cut, choice = self.k_cut, "user-specified"
        return float(self.alpha), float(self.r_cut), float(k_cut), choice

    def get_precomputed_array_device(self, precision="auto", pmiv="system",
                                     stream=None):
        """Build the array on the GPU and keep it there (CUDA float64)."""
        from .ewald import build_device_array
        alpha, r_cut, k_cut, _ = self._ewald_parameters()
        A, info = build_device_array(self, alpha, r_cut, k_cut, precision,
                                     pmiv, stream,
                                     split_launch=self.split_launch)
        self.last_build_info = info
        return A

    def get_precomputed_array(self, dst_path, compute_energy_contributions=0,
                              return_k_vector_data=0, precision="auto"):
        """(A, dst_path) with A the (N, N) float64 host array and the
        ``precomputed_array.log`` report of PyCD/core.py:1611-1679.

        User-specified alpha, r_cut and k_cut (or a k_max list) are built
        directly; any automatic choice ('optimal', 'converge',
        'simulation_cell') first runs get_ewald_parameters, whose energy scans
        run on the GPU, and may move dst_path as the reference does.  The
        report keeps the reference's lines (alpha on line 4, which
        material_run reads) and adds the k-vector count and build mode.
        ``return_k_vector_data`` also writes the per-k energy log
        (k_vector_data_report)."""
        import torch
        a2b = constants.ANG2BOHR
        if self._user_specified():
            alpha, r_cut, k_cut, kchoice = self._ewald_parameters()
            choice = {"alpha": "user-specified", "r_cut": "user-specified",
                      "k_cut": kchoice}
            lines = None
        else:
            if self.precision_parameters is None:
                raise ValueError("automatic Ewald parameters need precision_parameters")
            dst_path = Path(dst_path)
            params, lines, dst_path = self.get_ewald_parameters([], dst_path)
            alpha, r_cut, k_cut = (float(params["alpha"]), float(params["r_cut"]),
                                   float(params["k_cut"]))
            self._chosen_parameters = (alpha, r_cut, k_cut, "chosen")
        A_dev = self.get_precomputed_array_device(precision)
        torch.cuda.synchronize()
        A = A_dev.cpu().numpy()
        info = self.last_build_info
        n = self.neighbors.num_system_elements
        if lines is None:
            # timing lines from this build's own real / Fourier phases
            tau_r = info["real_ms"] / max(1, n * n)
            tau_f = info["fourier_ms"] / max(1, n * n * max(1, info["n_kvec"]))
            lines = [
                f"tau_ratio, (tau_r/tau_f): {tau_r / tau_f if tau_f else 0.0:.3e}\n",
                f"time_ratio, (time_r/time_f): "
                f"{info['real_ms'] / info['fourier_ms'] if info['fourier_ms'] else 0.0:.3e}\n\n",
                f"alpha: {alpha * a2b:.3e} / angstrom ({choice['alpha']})\n",
                f"r_cut: {r_cut / a2b:.3e} angstrom ({choice['r_cut']})\n",
                f"k_cut: {k_cut * a2b:.3e} / angstrom ({choice['k_cut']})\n"]
            q = self.base_charge_config_for_accuracy_analysis("full")
            einsum = float(np.einsum("ii", np.multiply(q.transpose(), q)))
            lines = self.compute_cutoff_errors(einsum, alpha, r_cut, k_cut,
                                               np.power(self.system_volume, 1 / 3), lines)
        k_max = info["k_max"]
        num_k_vectors = int(np.ceil(np.prod(2 * k_max + 1) * np.pi / 6 - 1))
        lines += [f"k_max: [{k_max[0]}, {k_max[1]}, {k_max[2]}]\n",
                  f"number of k-vectors: {num_k_vectors}\n\n"]
        if compute_energy_contributions:
            # core.py:1662-1673, each part's energy on the device
            ev = self._energy_evaluator("full")
            e_real = ev.real(alpha, r_cut)
            e_fourier = ev.fourier(alpha, k_cut)
            e_self = ev.self_term(alpha)
            eh = constants.EV2HARTREE
            lines += [f"Energy contribution from Real space: {e_real / eh} eV\n",
                      f"Energy contribution from Fourier-space: {e_fourier / eh} eV\n",
                      f"Energy contribution from self-interactions: {e_self / eh} eV\n",
                      f"Total system energy (neutral): "
                      f"{(e_real + e_fourier + e_self) / eh} eV\n\n"]
        lines += [f"k-vectors used: {info['n_kvec']}\n",
                  f"build: {info['mode']} on the GPU\n\n"]
        if dst_path is not None:
            Path(dst_path).mkdir(parents=True, exist_ok=True)
            if return_k_vector_data:
                self.k_vector_data_report(dst_path, alpha, k_cut)
            generate_report(self.start_time, Path(dst_path), "precomputed_array",
                            1, "".join(lines))
        return (A, dst_path)

    def k_vector_data_report(self, dst_path, alpha, k_cut):
        """The ``return_k_vector_data`` branch of get_precomputed_array
        (PyCD/core.py:1626-1653, pot_k_ewald_with_k_vector_data at
        core.py:880-911): the energy contribution of every half-space
        k-vector of the k_max box for the 'full' lattice charges (zero for
        those outside k_cut), sorted in decreasing order into
        ``k_vector_energy_contribution_within_user_specified_k_cut.log``.
        Each contribution is one device pass over the pairs per k-vector
        (``pycd_ewald_kvector_energies``).  Returns (k-vectors, contributions)
        in the reference's unsorted k order."""
        from .ewald import half_space_k_vectors, k_max_for
        kv, keep = half_space_k_vectors(self.reciprocal_lattice_matrix,
                                        k_max_for(self, k_cut), k_cut)
        contrib = np.zeros(len(kv))
        if keep.any():
            contrib[keep] = self._energy_evaluator("full").k_vectors(alpha, kv[keep])
        order = np.argsort(contrib)[::-1]
        eh = constants.EV2HARTREE
        lines = ["k-vectors sorted in the decreasing order of their energy contributions\n"]
        lines += [f"{k[0]:4d} {k[1]:4d} {k[2]:4d}: {e / eh:.3e} eV\n"
                  for k, e in zip(kv[order].tolist(), contrib[order])]
        generate_report(self.start_time, Path(dst_path),
                        "k_vector_energy_contribution_within_user_specified_k_cut", 0,
                        "".join(lines))
        print("Finished k-vector analysis")
        return kv, contrib


class Run(object):
    """KMC run (PyCD/core.py:1682-1933 set-up, 2647-2917 loop)."""

    # steps per kernel launch in the drop-in path; each launch consumes at
    # most this many pairs of host-generated MT19937 uniforms
    UNIFORM_BLOCK = 1 << 16

    def __init__(self, system, precomputed_array, temp, ion_charge_type,
                 species_charge_type, n_traj, t_final, time_interval,
                 species_count, initial_occupancy, relative_energies,
                 external_field, doping):
        self.start_time = datetime.now()
        self.system = system
        self.material = m = system.material
        self.neighbors = system.neighbors
        self.precomputed_array = precomputed_array
        self.temp = temp * constants.K2AUTEMP
        self.ion_charge_type = ion_charge_type
        self.species_charge_type = species_charge_type
        self.n_traj = int(n_traj)
        self.t_final = t_final * constants.SEC2AUTIME
        self.time_interval = time_interval * constants.SEC2AUTIME
        self.species_count = np.asarray(species_count)
        self.initial_occupancy = initial_occupancy
        self.system_size = system.system_size
        self.relative_energies = relative_energies
        # per-site relative energies (core.py:1716-1730)
        uc_rel = np.zeros(m.total_elements_per_unit_cell)
        start = 0
        for ei in range(m.num_element_types):
            end = start + m.n_elements_per_unit_cell[ei]
            if m.num_classes[ei] != 1:
                et = m.element_types[ei]
                uc_rel[start:end] += [
                    relative_energies["class_index"][et][ci] * constants.EV2HARTREE
                    for ci in m.unit_cell_class_list[start:end]]
            start = end
        self.undoped_system_relative_energies = np.tile(uc_rel, system.num_cells)
        self.system_relative_energies = np.copy(self.undoped_system_relative_energies)
        self.n_proc = int(np.dot(self.species_count, system.num_neighbors))
        self.head_start_n_elements_per_unit_cell_cum_sum = [
            m.n_elements_per_unit_cell[:e].sum()
            for e in self.neighbors.element_type_indices]
        # electric field (core.py:1748-1761)
        ef = external_field["electric"]
        self.electric_field_mag = ef["mag"]
        if ef["active"]:
            self.electric_field_active = 1
            fdir = np.asarray(ef["dir"])
            if ef["ld"] == 1:
                fdir = np.dot(fdir, m.lattice_matrix)
            self.electric_field = ef["mag"] * (fdir / np.linalg.norm(fdir))
        else:
            self.electric_field_active = 0
            self.electric_field = np.zeros(self.neighbors.n_dim)
        # doping (core.py:1763-1781)
        self.doping = doping
        self.doping_active = int(bool(np.any(doping["num_dopants"])))
        if self.doping_active:
            self.dopant_element_types, self.substitution_element_types = [], []
            self.dopant_species_types = []
            for mp in doping["doping_element_map"]:
                sub, dop = mp.split(m.element_type_delimiter)
                self.dopant_element_types.append(dop)
                self.substitution_element_types.append(sub)
                self.dopant_species_types.append(
                    m.element_type_to_species_map[sub][0])
        # one active carrier species: the reference's process bookkeeping
        # restarts its species index per type (core.py:1876-1878), so only
        # single-species runs are meaningful there
        active = [i for i, c in enumerate(self.species_count) if c]
        if len(active) > 1:
            raise NotImplementedError(
                "runs with more than one carrier species type are not "
                "supported (the reference's per-species process indices "
                "restart at 0 for each type)")
        self.active_species_index = active[0] if active else None
        self.total_species = int(self.species_count.sum())
        self.species_charge_list = [
            m.species_charge_list[species_charge_type][i]
            for i, c in enumerate(self.species_count) for _ in range(c)]
        self._build_site_tables()

    # -- per-(site, slot) process tables (core.py:1823-1927) ----------------
    def _build_site_tables(self):
        m, sysm = self.material, self.system
        N = self.neighbors.num_system_elements
        si = self.active_species_index
        if si is None:
            self.n_slots = 0
            return
        sp = m.species_types[si]
        key = m.hop_element_types[sp][0]
        et = m.species_to_element_type_map[sp][0]
        eti = m.element_types.index(et)
        S = int(sysm.num_neighbors[si])
        self.n_slots = S
        self.hop_element_type = key
        nbr = np.full((N, S), -1, np.int32)
        hop = np.zeros((N, S, 3))
        lam = np.zeros((N, S))
        vab = np.zeros((N, S))
        shift = np.zeros((N, S))
        tpc = m.total_elements_per_unit_cell
        per_cell = m.n_elements_per_unit_cell[eti]
        head = m.n_elements_per_unit_cell[:eti].sum()
        hl = sysm.hop_neighbor_list[key]
        if self._site_tables_vectorised(nbr, hop, lam, vab, shift, key, hl, tpc,
                                        per_cell, head, S):
            self.site_nbr, self.site_hop = nbr, hop
            self.site_lam, self.site_vab = lam, vab
            self.site_field_shift = shift if self.electric_field_active else None
            self.carrier_charge = float(
                m.species_charge_list[self.species_charge_type][si])
            return
        for cell in range(int(self.system.num_cells)):
            for e in range(per_cell):
                site = cell * tpc + head + e
                eei = cell * per_cell + e
                ci = sysm.system_class_index_list[site]
                s = 0
                for t, obj in enumerate(hl[ci][:len(m.neighbor_cutoff_dist[key][ci])]):
                    idx = obj.neighbor_system_element_indices[eei]
                    vecs = obj.displacement_vector_list[eei]
                    for j in range(len(idx)):
                        if s >= S:
                            raise ValueError("site %d has more hop neighbours "
                                             "than the %d processes per carrier"
                                             % (site, S))
                        nbr[site, s] = idx[j]
                        hop[site, s] = vecs[j]
                        lam[site, s] = m.lambda_values[key][ci][t]
                        vab[site, s] = m.v_ab[key][ci][t]
                        if self.electric_field_active:
                            shift[site, s] = 0.5 * np.dot(self.electric_field, vecs[j])
                        s += 1
                if s != S:
                    raise ValueError("site %d has %d hop neighbours, expected %d"
                                     % (site, s, S))
        self.site_nbr, self.site_hop = nbr, hop
        self.site_lam, self.site_vab = lam, vab
        self.site_field_shift = shift if self.electric_field_active else None
        self.carrier_charge = float(
            m.species_charge_list[self.species_charge_type][si])

    def _site_tables_vectorised(self, nbr, hop, lam, vab, shift, key, hl, tpc,
                                per_cell, head, S):
        """Fill the tables with array operations when every site of a class
        has the same neighbour count per hop type (the common case); returns
        False to fall back to the per-site loop."""
        m, sysm = self.material, self.system
        n_cells = int(self.system.num_cells)
        eei = np.arange(n_cells * per_cell)
        sites = (eei // per_cell) * tpc + head + (eei % per_cell)
        cls = np.asarray(sysm.system_class_index_list)[sites]
        for ci in np.unique(cls):
            sel = np.nonzero(cls == ci)[0]
            s0 = 0
            for t, obj in enumerate(hl[ci][:len(m.neighbor_cutoff_dist[key][ci])]):
                counts = np.asarray(obj.num_neighbors)[sel]
                if len(counts) == 0 or np.any(counts != counts[0]):
                    return False
                c = int(counts[0])
                if s0 + c > S:
                    return False
                idx = np.stack([np.asarray(obj.neighbor_system_element_indices[e])
                                for e in sel]).reshape(len(sel), c)
                vec = np.stack([np.asarray(obj.displacement_vector_list[e], np.float64)
                                .reshape(-1, 3) for e in sel]).reshape(len(sel), c, 3)
                nbr[sites[sel], s0:s0 + c] = idx
                hop[sites[sel], s0:s0 + c] = vec
                lam[sites[sel], s0:s0 + c] = m.lambda_values[key][ci][t]
                vab[sites[sel], s0:s0 + c] = m.v_ab[key][ci][t]
                if self.electric_field_active:
                    shift[sites[sel], s0:s0 + c] = 0.5 * np.einsum(
                        "k,ijk->ij", self.electric_field, vec)
                s0 += c
            if s0 != S:
                return False
        return True

    # -- charges (core.py:2530-2564) ----------------------------------------
    def base_charge_config(self):
        m = self.material
        uc = np.array([m.charge_types[self.ion_charge_type][m.element_types[e]]
                       for e in m.element_type_index_list])
        return np.tile(uc, self.system.num_cells)[:, np.newaxis]

    def fixed_charge_config(self, dopant_site_indices):
        """Lattice charges with dopant sites overwritten (no carriers)."""
        q = self.base_charge_config()
        if self.doping_active:
            for dop, sites in dopant_site_indices.items():
                q[sites] = self.doping["charge"][self.ion_charge_type][dop]
        return q

    def charge_config(self, occupancy, dopant_site_indices):
        q = self.fixed_charge_config(dopant_site_indices)
        for sti in range(self.material.num_species_types):
            s0 = self.species_count[:sti].sum()
            s1 = s0 + self.species_count[sti]
            q[list(occupancy[s0:s1])] += \
                self.material.species_charge_list[self.species_charge_type][sti]
        return q

    # -- initial occupancy (core.py:2478-2528), MT19937 semantics -----------
    def generate_initial_occupancy(self, dopant_site_indices):
        m = self.material
        occupancy = []
        for sti, num in enumerate(self.species_count):
            sp = m.species_types[sti]
            if self.doping_active:
                for mi, dsp in enumerate(self.dopant_species_types):
                    nd = self.doping["num_dopants"][mi]
                    if (self.doping["site_charge_initiation"][mi] == "yes"
                            and dsp == sp and nd and num):
                        de = self.dopant_element_types[mi]
                        occupancy.extend(rnd.sample(dopant_site_indices[de], num)[:])
                        num -= len(dopant_site_indices[de][:num])
            if sp in self.initial_occupancy:
                occupancy.extend([i for i in self.initial_occupancy[sp]])
                num -= len(self.initial_occupancy[sp])
            if num:
                sites = []
                for el in m.species_to_element_type_map[sp]:
                    ei = m.element_types.index(el)
                    offs = np.repeat(np.arange(0, m.total_elements_per_unit_cell
                                               * self.system.num_cells,
                                               m.total_elements_per_unit_cell),
                                     m.n_elements_per_unit_cell[ei])
                    idx = (np.tile(m.n_elements_per_unit_cell[:ei].sum()
                                   + np.arange(m.n_elements_per_unit_cell[ei]),
                                   self.system.num_cells) + offs)
                    sites.extend(list(idx))
                    sites = [i for i in sites if i not in occupancy]
                occupancy.extend(rnd.sample(sites, num)[:])
        return occupancy

    # -- per-trajectory seeds (core.py:2566-2580) ---------------------------
    def preproduction(self, dst_path, random_seed):
        dst_path = Path(dst_path)
        rnd.seed(random_seed)
        seeds = [rnd.random() for _ in range(self.n_traj)]
        for ti in range(self.n_traj):
            d = dst_path / f"traj{ti + 1}"
            d.mkdir(parents=True, exist_ok=True)
            rnd.seed(seeds[ti])
            with open(d / "initial_rnd_state.dump", "wb") as fh:
                pickle.dump(rnd.getstate(), fh)
        if self.doping_active:
            for ti in range(self.n_traj):
                d = dst_path / f"traj{ti + 1}"
                if not (d / "site_indices.npy").exists() and \
                        not (dst_path / "site_indices.npy").exists():
                    raise NotImplementedError(
                        "dopant placement is not part of this package; write "
                        "site_indices.npy (see pycd_gb300.doping) first")
        return None

    def _load_doping(self, traj_dir):
        """Dopant sites and per-site energy shifts from site_indices.npy
        (core.py:2723-2764)."""
        self.system_relative_energies = np.copy(self.undoped_system_relative_energies)
        if not self.doping_active:
            return {}
        pairwise = ("pairwise" in self.doping["insertion_type"] and
                    self.doping["num_dopants"][
                        self.doping["insertion_type"].index("pairwise")] != 0)
        path = (traj_dir.parent if pairwise else traj_dir) / "site_indices.npy"
        data = np.load(path)
        sites, types, shells = data[:, 0], data[:, 1], data[:, 3]
        dopant_site_indices = {}
        for ai in np.where(shells == 0)[0]:
            de = self.dopant_element_types[types[ai]]
            dopant_site_indices.setdefault(de, []).append(int(sites[ai]))
        for i in range(len(types)):
            de = self.dopant_element_types[types[i]]
            mi = self.dopant_element_types.index(de)
            sub = self.substitution_element_types[mi]
            if shells[i] < len(self.relative_energies["doping"][sub][mi]):
                self.system_relative_energies[sites[i]] += (
                    self.relative_energies["doping"][sub][mi][shells[i]]
                    * constants.EV2HARTREE)
        return dopant_site_indices

    def device_tables(self, A_device=None, dopant_site_indices=None):
        """KmcTables for the current doping (A may already be on the GPU)."""
        from .kmc import KmcTables
        A = self.precomputed_array if A_device is None else A_device
        q_fixed = self.fixed_charge_config(dopant_site_indices or {})[:, 0]
        num_path = int(self.t_final / self.time_interval) + 1
        return KmcTables(
            A, self.site_nbr, self.site_hop, self.site_lam, self.site_vab,
            self.system_relative_energies, q_fixed, self.carrier_charge,
            self.total_species, self.material.vn, self.temp, self.time_interval,
            num_path, field_shift=self.site_field_shift)

    # -- the KMC loop -------------------------------------------------------
    # device memory for one group of trajectories advanced together (path
    # grids, per-step logs, uniforms); larger runs go in several groups
    GROUP_BYTES = 2 << 30

    def _group_size(self, num_path, outputs):
        per = (8 * num_path * 3 * self.total_species * (1 + outputs)
               + 28 * self.UNIFORM_BLOCK + 4096)
        return max(1, int(self.GROUP_BYTES // per))

    def do_kmc_steps(self, dst_path, output_data, random_seed, compute_mode):
        """Run every trajectory on the GPU and write the reference's files
        (core.py:2863-2906) with the same 'ab' append semantics.

        The reference runs its trajectories one after another
        (core.py:2668); here all n_traj trajectories of the call advance
        together in one batch, each on its own MT19937 stream restored from
        its initial_rnd_state.dump (core.py:2694-2695) and drawn in blocks of
        UNIFORM_BLOCK steps.  A trajectory's events, times and files are the
        same as when it runs alone.  A trajectory that stops on a zero or
        non-finite k_total raises NativeError after the files of the
        trajectories before it are written, where the reference raises its
        IndexError."""
        import torch
        from .kmc import KmcBatch, KmcEngine
        nat.require_device()
        dst_path = Path(dst_path)
        if compute_mode != "parallel":
            self.preproduction(dst_path, random_seed)
        num_path = int(self.t_final / self.time_interval) + 1
        ue = output_data["unwrapped_traj"]
        if not ue["write"]:
            raise ValueError("output_data['unwrapped_traj']['write'] must be 1")
        every_step = bool(ue.get("write_every_step", 0))
        want = lambda k: k in output_data and output_data[k]["write"]
        system_charge = np.dot(self.species_count,
                               self.material.species_charge_list[self.species_charge_type])
        ewald_neut = -(np.pi * system_charge ** 2
                       / (2 * self.system.system_volume * self.system.alpha))
        A_dev = torch.as_tensor(np.ascontiguousarray(self.precomputed_array,
                                                     np.float64)).cuda()
        drift = np.zeros((self.n_traj, self.total_species, 3)) \
            if self.electric_field_active else None
        self.last_run_steps = []
        # per-trajectory set-up in the reference's order: MT state, doping,
        # initial occupancy (which may draw from the stream), energy
        trajs = []
        shared_tables = None
        for ti in range(self.n_traj):
            traj_dir = (dst_path / f"traj{ti + 1}") if compute_mode != "parallel" \
                else dst_path
            traj_dir.mkdir(parents=True, exist_ok=True)
            with open(traj_dir / "initial_rnd_state.dump", "rb") as fh:
                rnd.setstate(pickle.load(fh))
            dopants = self._load_doping(traj_dir)
            occ = self.generate_initial_occupancy(dopants)
            q = self.charge_config(occ, dopants)
            qq = np.multiply(q.transpose(), q)
            energy0 = ewald_neut + np.sum(np.multiply(qq, self.precomputed_array))
            if self.doping_active:
                tables = self.device_tables(A_dev, dopants)
            else:
                if shared_tables is None:
                    shared_tables = self.device_tables(A_dev, dopants)
                tables = shared_tables
            trajs.append({"dir": traj_dir, "occ": list(occ), "energy0": energy0,
                          "tables": tables, "stream": _Mt19937Stream(rnd.getstate()),
                          "occupancy_list": [list(occ)] if self.doping_active else None})
        outputs = int(bool(want("energy"))) + int(bool(want("delg_0")))
        g = self._group_size(num_path, outputs)
        failure = None
        for g0 in range(0, self.n_traj, g):
            group = trajs[g0:g0 + g]
            results = self._advance_group(group, num_path, want)
            for off, (tr, res) in enumerate(zip(group, results)):
                ti = g0 + off
                if res["error"] is not None:
                    failure = (ti, res["error"])
                    break
                step_proc = res["step_proc"]
                self.last_run_steps.append(step_proc)
                occ = tr["occ"]
                if self.doping_active:
                    tr["occupancy_list"].extend(self._replay_occupancy(occ, step_proc)[1:])
                unwrapped = (self._every_step_rows(occ, step_proc) if every_step
                             else res["unwrapped"])
                if drift is not None:
                    drift[ti] = res["drift"]
                arrays = {"unwrapped_traj": unwrapped, "time": res["time"],
                          "wrapped_traj": np.zeros((num_path, self.total_species * 3)),
                          "potential": np.zeros((num_path, self.total_species))}
                if want("energy"):
                    arrays["energy"] = res["energy"]
                if want("delg_0"):
                    arrays["delg_0"] = res["delg_0"]
                for kind, attrs in output_data.items():
                    if attrs.get("write") and kind in arrays:
                        with open(tr["dir"] / attrs["file_name"], "ab") as fh:
                            np.save(fh, arrays[kind])
                self._write_hdf5(tr["dir"], output_data, unwrapped, res["time"], every_step)
                if self.doping_active:
                    np.save(tr["dir"] / "occupancy.npy",
                            np.asarray(tr["occupancy_list"], dtype=int))
            if failure is not None:
                break
        # the module-level stream ends where the last trajectory's ended
        last = trajs[failure[0] if failure else -1]["stream"]
        rnd.setstate(last.state())
        if failure is not None:
            ti, (status, steps) = failure
            raise nat.NativeError(
                nat.ERR_STALLED if status == nat.TRAJ_STALLED else nat.ERR_BAD_INDEX,
                "trajectory %d stopped with status %d after %d steps "
                "(k_total zero/not finite, or no event selected)" % (ti + 1, status, steps))
        prefix = ""
        if self.electric_field_active:
            prefix = self._drift_mobility_report(drift, dst_path)
        generate_report(self.start_time, dst_path, "Run", 1, prefix)
        return None

    def _write_hdf5(self, traj_dir, output_data, unwrapped, time_data, every_step):
        """The optional HDF5 trajectory file of one trajectory
        (PyCD/core.py:2677-2691, 2882-2902; layout in hdf5_io).  It is written
        when output_data['hdf5_output']['enabled'] is true, the unwrapped rows
        are written and h5py can be imported; without h5py it is left out
        silently, as the reference does.  Failures print the reference's
        warnings and the run goes on.

        /time holds each frame's simulation time.  Per-step rows
        (write_every_step): row k is appended at the end of step k + 1
        (core.py:2832-2845), so its time is time_data[k + 1].  Grid rows: row
        r is the state at r * time_interval.  The reference passes its whole
        time list (steps + 1 values) for the frames, which h5py refuses in
        both cases (its /time stays zero-filled, with a warning), or, when
        the time output is off, the frame indices 0, 1, ... as times; its
        coordinates are the ones written here."""
        cfg = output_data.get("hdf5_output")
        if not (cfg and cfg.get("enabled", False)
                and output_data.get("unwrapped_traj", {}).get("write", False)):
            return
        try:
            from .hdf5_io import HDF5TrajectoryWriter
        except ImportError:
            return
        try:
            writer = HDF5TrajectoryWriter(Path(traj_dir) / cfg["file_name"],
                                          self.total_species, len(self.species_count))
        except Exception as e:
            print(f"Warning: Could not initialize HDF5 writer: {e}")
            return
        try:
            n = len(unwrapped)
            t = np.asarray(time_data, dtype=np.float64)
            times = (t[1:] if every_step and len(t) == n + 1
                     else np.arange(n) * self.time_interval)
            writer.write_frames(unwrapped, times)
        except Exception as e:
            print(f"Warning: Failed to write HDF5 trajectory data: {e}")
        try:
            writer.close()
        except Exception as e:
            print(f"Warning: Failed to close HDF5 writer: {e}")

    def _advance_group(self, group, num_path, want):
        """Advance the trajectories of `group` together to the end of their
        time grids.  Launches run in lockstep: each advances every running
        trajectory by UNIFORM_BLOCK steps on the next UNIFORM_BLOCK pairs of
        its own uniforms, so a running trajectory's step count is always
        launch * UNIFORM_BLOCK and one log offset serves all of them."""
        import torch
        from .kmc import KmcBatch, KmcEngine
        B = self.UNIFORM_BLOCK
        T = len(group)
        tables, sys_index = [], []
        for tr in group:
            for i, t in enumerate(tables):
                if t is tr["tables"]:
                    sys_index.append(i)
                    break
            else:
                sys_index.append(len(tables))
                tables.append(tr["tables"])
        batch = KmcBatch(np.asarray([tr["occ"] for tr in group]),
                         sys_index=sys_index if len(tables) > 1 else None,
                         energy0=[tr["energy0"] for tr in group],
                         unwrapped_rows=num_path, step_capacity=B,
                         energy_grid_rows=num_path if want("energy") else None,
                         delg0_grid_rows=num_path if want("delg_0") else None,
                         drift=self.electric_field_active)
        engine = KmcEngine(tables)
        host_u = torch.empty((T, 2 * B), dtype=torch.float64, pin_memory=True)
        ubuf = torch.empty((T, 2 * B), dtype=torch.float64, device="cuda")
        times = [[] for _ in range(T)]
        procs = [[] for _ in range(T)]
        running = np.ones(T, bool)
        error = [None] * T
        hu = host_u.numpy()
        launch = 0
        while running.any():
            for t in np.nonzero(running)[0]:
                group[t]["stream"].fill(hu[t])
            ubuf.copy_(host_u, non_blocking=True)
            batch.u_cursor.zero_()
            batch.step_offset = launch * B
            engine.advance(batch, B, engine.rng_struct(ubuf))
            torch.cuda.synchronize()
            steps = batch.step.cpu().numpy()
            status = batch.status.cpu().numpy()
            st_time = batch.step_time.cpu().numpy()
            st_proc = batch.step_proc.cpu().numpy()
            for t in np.nonzero(running)[0]:
                n_done = int(steps[t]) - launch * B
                times[t].append(st_time[t, :n_done].copy())
                procs[t].append(st_proc[t, :n_done].copy())
                group[t]["stream"].used(2 * n_done)
                if status[t] == nat.TRAJ_RUNNING:
                    continue
                running[t] = False
                if status[t] != nat.TRAJ_DONE:
                    error[t] = (int(status[t]), int(steps[t]))
            launch += 1
        unw = batch.unwrapped[:, :, :3 * self.total_species].cpu().numpy()
        eg = batch.energy_grid.cpu().numpy() if want("energy") else None
        dg = batch.delg0_grid.cpu().numpy() if want("delg_0") else None
        dr = batch.drift[:, :self.total_species].cpu().numpy() \
            if self.electric_field_active else None
        out = []
        for t in range(T):
            out.append({"error": error[t],
                        "step_proc": (np.concatenate(procs[t]) if procs[t]
                                      else np.zeros(0, np.int32)),
                        "time": np.concatenate([[0.0]] + times[t]),
                        "unwrapped": unw[t],
                        "energy": None if eg is None else eg[t],
                        "delg_0": None if dg is None else dg[t],
                        "drift": None if dr is None else dr[t]})
        return out

    def _replay_occupancy(self, occ0, step_proc):
        occ = list(occ0)
        out = [list(occ)]
        S = self.n_slots
        for p in step_proc:
            c, s = divmod(int(p), S)
            occ[c] = int(self.site_nbr[occ[c], s])
            out.append(list(occ))
        return out

    def _every_step_rows(self, occ0, step_proc):
        """write_every_step rows: row 0 is zero and the first hop is not
        recorded, as core.py:2832-2843 does."""
        S = self.n_slots
        occ = list(occ0)
        rows = np.zeros((max(1, len(step_proc)), 3 * self.total_species))
        for i, p in enumerate(step_proc):
            c, s = divmod(int(p), S)
            h = self.site_hop[occ[c], s]
            occ[c] = int(self.site_nbr[occ[c], s])
            if i > 0:
                rows[i] = rows[i - 1]
                rows[i, 3 * c:3 * c + 3] += h
        return rows

    def _drift_mobility_report(self, drift_velocity_array, dst_path):
        mob_au = (np.dot(drift_velocity_array, self.electric_field)
                  / self.electric_field_mag ** 2)
        mob = mob_au * (constants.BOHR2CM ** 2 * constants.SEC2AUTIME
                        * constants.V2AUPOT)
        with open(Path(dst_path) / "drift_mobility.dat", "wb") as fh:
            np.savetxt(fh, mob)
        lines = []
        start = 0
        for si, num in enumerate(self.species_count):
            end = start + num
            if num:
                sp = self.material.species_types[si]
                avg = np.mean(mob[:, start:end], axis=1)
                lines.append(f"Estimated value of {sp} drift mobility is: "
                             f"{np.mean(avg):4.3e} cm2/V.s.\n")
                lines.append(f"Standard error of mean in {sp} drift mobility is: "
                             f"{np.std(avg) / np.sqrt(self.n_traj):4.3e} cm2/V.s.\n")
            start = end
        return "".join(lines)
