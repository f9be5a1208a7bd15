"""Ewald parameter selection (PyCD/core.py:913-1592) with every energy
evaluated on the GPU.

The reference chooses alpha, r_cut and k_cut by scanning energies: the
real-space and Fourier-space energies sum_ij q_i q_j A_part[i, j] of the
lattice charges at tens of cutoffs, and the contribution of single
k-vectors.  Each of those is one NumPy array build of O(N^2) (real space) or
O(N^2 K) (Fourier space).  Here every energy is one device build of the part
alone (``PycdEwaldDesc.parts``) followed by q . (A q) on the device, so a scan
takes milliseconds per point.  The decisions around the energies (fsolve on
the cutoff-error models, convergence checks, step-change analysis, the
printed progress and the report lines) are the reference's, restated on the
host.  Figures are not drawn.

The methods keep the reference's names; where the reference passes
``charge_list_prod`` (the N x N matrix q q^T) they take an ``EwaldEnergy``
evaluator for the same charges.  ``System`` mixes this class in.
"""
from pathlib import Path

import numpy as np
from scipy.optimize import fsolve

from . import _native as nat
from . import constants
from .io import generate_report


def _num_k_vectors(k_max):
    """Upper estimate of the half-space k count (core.py:1600)."""
    return np.ceil(np.prod(2 * np.asarray(k_max) + 1) * np.pi / 6 - 1).astype(int)


class EwaldEnergy(object):
    """sum_ij q_i q_j A_part[i, j] for one charge vector, each part built on
    the current GPU (FP64; the reference's own formula for any pmiv)."""

    def __init__(self, system, charge_list):
        import torch
        from .ewald import choose_mode
        self.system = system
        self.n = int(system.neighbors.num_system_elements)
        dev = torch.device("cuda", torch.cuda.current_device())
        nat.require_device()
        self.q = torch.as_tensor(np.asarray(charge_list, np.float64).ravel()).to(dev)
        self.A = torch.empty((self.n, self.n), dtype=torch.float64, device=dev)
        self.phi = torch.empty(self.n, dtype=torch.float64, device=dev)
        self.e = torch.empty(1, dtype=torch.float64, device=dev)
        pmiv = system.pairwise_min_image_vector_data
        mode = choose_mode(system, pmiv, "auto")
        self.mode = mode if mode in ("fp64", "fp64_direct") else "fp64"
        self.builds = 0
        self._kcache = {}

    def _energy(self, alpha, r_cut, k_cut, parts, kvecs=None):
        from .ewald import build_device_array
        _, info = build_device_array(self.system, alpha, r_cut, k_cut, self.mode,
                                     out=self.A, parts=parts, kvecs=kvecs)
        nat.check(nat.lib().pycd_potential_gemv(
            self.A.data_ptr(), self.n, self.q.data_ptr(), self.phi.data_ptr(),
            self.e.data_ptr(), nat.stream_handle()))
        self.builds += 1
        self.last_info = info
        return float(self.e.item())

    def real(self, alpha, r_cut):
        """Energy of get_precomputed_array_real(alpha, r_cut) (core.py:1594-1596)."""
        return self._energy(alpha, r_cut, 0.0, nat.EWALD_PART_REAL)

    # systems up to this many sites take Fourier energies from cached per-k
    # contributions (one pass over the N^2 pairs per new k) instead of a build
    PER_K_MAX_SITES = 1024

    def fourier(self, alpha, k_cut):
        """Energy of get_precomputed_array_fourier(alpha, k_cut)[0] (core.py:1598-1602).

        Small systems: (2 / eps) times the sum of the per-k contributions of
        the k list, each contribution computed once per alpha and cached, so a
        k_cut scan costs one pass per distinct k.  Identical k lists give
        identical sums.  Larger systems: one device build of the part."""
        if self.n > self.PER_K_MAX_SITES:
            return self._energy(alpha, 0.0, k_cut, nat.EWALD_PART_FOURIER)
        from .ewald import effective_k_vectors, k_max_for
        kv = effective_k_vectors(self.system.reciprocal_lattice_matrix,
                                 k_max_for(self.system, k_cut), k_cut)
        cache = self._kcache.setdefault(float(alpha), {})
        keys = [tuple(r) for r in kv.tolist()]
        new = [k for k in dict.fromkeys(keys) if k not in cache]
        if new:
            for k, e in zip(new, self.k_vectors(alpha, np.array(new, np.int32))):
                cache[k] = float(e)
        total = 0.0
        for k in keys:
            total += cache[k]
        return 2.0 * total / self.system.material.dielectric_constant

    def self_term(self, alpha):
        """Energy of the self-interaction diagonal (core.py:1656)."""
        return self._energy(alpha, 0.0, 0.0, nat.EWALD_PART_SELF)

    def k_vectors(self, alpha, k_vectors):
        """get_k_vector_energy_contribution (core.py:1171-1184) of every row
        of the (K, 3) integer array, in one device pass over the pairs per k."""
        import torch
        from .ewald import make_desc
        kv = np.ascontiguousarray(np.asarray(k_vectors, np.int32).reshape(-1, 3))
        if len(kv) == 0:
            return np.zeros(0)
        pmiv = self.system.pairwise_min_image_vector_data
        desc, keep, _ = make_desc(self.system, alpha, 0.0, 0.0, pmiv, kvecs=kv)
        out = torch.empty(len(kv), dtype=torch.float64, device=self.q.device)
        nat.check(nat.lib().pycd_ewald_kvector_energies(
            nat.C.byref(desc), self.q.data_ptr(), out.data_ptr(), nat.stream_handle()))
        self.builds += 1
        return out.cpu().numpy()

    def k_vector(self, alpha, k_vector):
        """get_k_vector_energy_contribution (core.py:1171-1184): the sum over
        pairs of (2 pi/V) e^{-k^2/4 alpha} cos(k . d_ij) / k^2, i.e. the
        one-vector Fourier energy without the factor 2 and the 1/eps."""
        e = self._energy(alpha, 0.0, 0.0, nat.EWALD_PART_FOURIER,
                         kvecs=np.asarray(k_vector, np.int32).reshape(1, 3))
        return e * self.system.material.dielectric_constant / 2


class _Deferred(object):
    """Builds its target on first attribute access."""

    def __init__(self, make):
        self._make, self._obj = make, None

    def __getattr__(self, name):
        if self._obj is None:
            self._obj = self._make()
        return getattr(self._obj, name)


class EwaldParameterSearch(object):
    """The reference's Ewald parameter search, mixed into ``System``."""

    def _load_precision_parameters(self, precision_parameters):
        """core.py:785-797."""
        p = precision_parameters
        self.lower_bound_real = p['lower_bound_real']
        self.lower_bound_rcut = p['lower_bound_rcut']
        self.upper_bound_rcut = p['upper_bound_rcut']
        self.lower_bound_kcut = p['lower_bound_kcut']
        self.upper_bound_kcut = p['upper_bound_kcut']
        self.threshold_fraction = p['threshold_fraction']
        self.num_data_points_low = int(p['num_data_points_low'])
        self.num_data_points_high = int(p['num_data_points_high'])
        self.precise_r_cut = p['precise_r_cut']
        self.err_tol = p['err_tol'] * constants.EV2HARTREE
        self.step_increase_tol = p['step_increase_tol'] * constants.EV2HARTREE
        self.step_change_data_points = p['step_change_data_points']

    def _k_cut_given(self):
        """k_cut numeric or a k_max list.  The reference writes
        np.isreal(k_cut) or isinstance(k_cut, list), which raises for a list
        (the truth value of an array); the list is tested first here."""
        return isinstance(self.k_cut, list) or bool(np.isreal(self.k_cut))

    # -- timing ------------------------------------------------------------
    def benchmark_ewald(self, num_repeats, benchmark_parameters):
        """Seconds per real-space pair and per (entry, k) of the device builds
        (core.py:913-939, which times the NumPy builds)."""
        from .ewald import effective_k_vectors
        k_max = benchmark_parameters['k_max']
        alpha = benchmark_parameters['alpha']
        r_cut = benchmark_parameters['r_cut']
        k_cut = benchmark_parameters['k_cut']
        ev = self._energy_evaluator()
        kv = effective_k_vectors(self.reciprocal_lattice_matrix, k_max, k_cut)
        time_r = time_f = 0.0
        for _ in range(num_repeats):
            ev._energy(alpha, r_cut, 0.0, nat.EWALD_PART_REAL)
            time_r += ev.last_info["real_ms"] / 1e3
            ev._energy(alpha, 0.0, k_cut, nat.EWALD_PART_FOURIER, kvecs=kv)
            time_f += ev.last_info["fourier_ms"] / 1e3
        num_neighbor_pairs = self._num_pairs_within(r_cut)
        tau_r = time_r / num_repeats / num_neighbor_pairs
        num_k_vectors = _num_k_vectors(k_max)
        tau_f = (time_f / num_repeats / self.neighbors.num_system_elements ** 2
                 / num_k_vectors)
        return (tau_r / tau_f, time_r / time_f)

    def _num_pairs_within(self, r_cut):
        """Pairs with |pmiv_ij| < r_cut, the diagonal included (core.py:807-811)."""
        pmiv = self.pairwise_min_image_vector_data
        if pmiv is None:
            pmiv = self.neighbors.get_pairwise_min_image_vector_data()
        return int((np.linalg.norm(pmiv, axis=2) < r_cut).sum())

    def _energy_evaluator(self, ion_charge_type='full'):
        """EwaldEnergy of the lattice charges, created on first use (branches
        that only solve the cutoff-error models never touch the GPU)."""
        key = ion_charge_type
        cache = getattr(self, "_ewald_energy_cache", None)
        if cache is None or cache[0] != key:
            q = self.base_charge_config_for_accuracy_analysis(ion_charge_type)
            self._ewald_energy_cache = (key, _Deferred(lambda: EwaldEnergy(self, q)))
        return self._ewald_energy_cache[1]

    # -- cutoff-error models (host) -----------------------------------------
    def base_charge_config_for_accuracy_analysis(self, ion_charge_type):
        """Lattice charges of every site (core.py:941-948), shape (N, 1)."""
        m = self.material
        unit = np.array([m.charge_types[ion_charge_type][m.element_types[e]]
                         for e in m.element_type_index_list])
        return np.tile(unit, self.num_cells)[:, np.newaxis]

    def _real_cutoff_error(self, einsum, alpha, r_cut):
        return (einsum * np.sqrt(r_cut / (2 * self.system_volume))
                * (np.exp(-(alpha * r_cut) ** 2) / (alpha * r_cut) ** 2))

    def _fourier_cutoff_error(self, einsum, length, alpha, n_cut):
        x = np.pi * n_cut / (alpha * length)
        return einsum * np.sqrt(n_cut) / (alpha * length ** 2) * (np.exp(-x ** 2) / x ** 2)

    def minimize_real_space_cutoff_error(self, charge_list_einsum, real_space_parameters,
                                         x_real_initial_guess):
        """core.py:950-961."""
        p = real_space_parameters
        if 'alpha' in p:
            alpha = p['alpha']
            f = lambda r_cut: self._real_cutoff_error(charge_list_einsum, alpha, r_cut) - self.err_tol
            p['r_cut'] = fsolve(f, x_real_initial_guess / alpha)[0]
        else:
            r_cut = p['r_cut']
            f = lambda alpha: self._real_cutoff_error(charge_list_einsum, alpha, r_cut) - self.err_tol
            p['alpha'] = fsolve(f, x_real_initial_guess / r_cut)[0]
        return p

    def minimize_fourier_space_cutoff_error(self, charge_list_einsum, volume_derived_length,
                                            fourier_space_parameters, x_fourier_initial_guess):
        """core.py:963-975."""
        p, L = fourier_space_parameters, volume_derived_length
        if 'alpha' in p:
            alpha = p['alpha']
            f = lambda n_cut: self._fourier_cutoff_error(charge_list_einsum, L, alpha, n_cut) - self.err_tol
            n_cut0 = x_fourier_initial_guess * L * alpha / np.pi
            p['k_cut'] = 2 * np.pi / L * fsolve(f, n_cut0)[0]
        else:
            n_cut = p['k_cut'] * L / (2 * np.pi)
            f = lambda alpha: self._fourier_cutoff_error(charge_list_einsum, L, alpha, n_cut) - self.err_tol
            alpha0 = np.pi * n_cut / (x_fourier_initial_guess * L)
            p['alpha'] = fsolve(f, alpha0)[0]
        return p

    def compute_cutoff_errors(self, charge_list_einsum, alpha, r_cut, k_cut,
                              volume_derived_length, prefix_list):
        """core.py:977-984."""
        real_err = self._real_cutoff_error(charge_list_einsum, alpha, r_cut)
        n_cut = k_cut * volume_derived_length / (2 * np.pi)
        fourier_err = self._fourier_cutoff_error(charge_list_einsum, volume_derived_length,
                                                 alpha, n_cut)
        prefix_list.append(f'Real-space cutoff error: {real_err:.3e}\n')
        prefix_list.append(f'Fourier-space cutoff error: {fourier_err:.3e}\n\n')
        return prefix_list

    # -- energy scans (device) ------------------------------------------------
    def convergence_check_with_r_cut(self, ev, alpha, r_cut_max, lower_bound, upper_bound):
        """core.py:986-998."""
        lower = ev.real(alpha, lower_bound * r_cut_max)
        upper = ev.real(alpha, upper_bound * r_cut_max)
        return 1 if abs(lower - upper) < self.err_tol else 0

    def get_energy_profile_with_r_cut(self, ev, alpha, r_cut_max, lower_bound, upper_bound,
                                      num_data_points):
        """core.py:1000-1010."""
        r_cut_data = np.linspace(lower_bound * r_cut_max, upper_bound * r_cut_max,
                                 num_data_points)
        energy = np.array([ev.real(alpha, r) for r in r_cut_data])
        return (r_cut_data, energy)

    def convergence_check_with_k_cut(self, ev, alpha, k_cut_lower, k_cut_upper):
        """core.py:1012-1024."""
        lower = ev.fourier(alpha, k_cut_lower)
        upper = ev.fourier(alpha, k_cut_upper)
        return 1 if abs(lower - upper) < self.err_tol else 0

    def get_energy_profile_with_k_cut(self, ev, alpha, k_cut_lower, k_cut_upper,
                                      num_data_points):
        """core.py:1026-1034."""
        k_cut_data = np.linspace(k_cut_lower, k_cut_upper, num_data_points)
        energy = np.array([ev.fourier(alpha, k) for k in k_cut_data])
        return (k_cut_data, energy)

    def check_for_k_cut_step_energy_convergence(self, step_energy_k_cut_data, energy_changes,
                                                k_cut_lower, k_cut_upper):
        """core.py:1036-1045."""
        sel = energy_changes[(step_energy_k_cut_data >= k_cut_lower)
                             & (step_energy_k_cut_data <= k_cut_upper)]
        return 1 if (sel.sum() < self.err_tol and abs(sel).max() < self.err_tol) else 0

    def get_convergence_rcut(self, ev, alpha, r_cut_max, lower_bound, upper_bound):
        """core.py:1047-1058."""
        r_cut_data, energy = self.get_energy_profile_with_r_cut(
            ev, alpha, r_cut_max, lower_bound, upper_bound, self.num_data_points_low)
        off = np.where(np.abs(energy - energy[-1]) > self.err_tol)[0]
        return r_cut_data[0] if len(off) == 0 else r_cut_data[off.max() + 1]

    def get_simulation_cell_real_space_parameters(self, ev, charge_list_einsum,
                                                  real_space_parameters,
                                                  x_real_initial_guess, dst_path):
        """core.py:1060-1126 (figures not drawn)."""
        a2b = constants.ANG2BOHR
        r_cut_max = min(self.translational_vector_length) / 2
        real_space_parameters['r_cut'] = 0.75 * r_cut_max
        real_space_parameters = self.minimize_real_space_cutoff_error(
            charge_list_einsum, real_space_parameters, x_real_initial_guess)
        alpha = real_space_parameters['alpha']
        up = 10
        print('Attempting to find best alpha towards converging real-space energy '
              'within the simulation cell:\n')
        print(f'Starting with an estimate for alpha={alpha * a2b:.3e} / angstrom')
        while not self.convergence_check_with_r_cut(ev, alpha, r_cut_max, self.threshold_fraction,
                                                    self.upper_bound_rcut):
            alpha = (1 + up / 100) * alpha
            print(f'Couldn\'t find real-space energy convergence within simulation cell. '
                  f'Re-attempting with {up} % increased alpha={alpha * a2b:.3e} / angstrom')
        print(f'Preliminary convergence in real-space energy achieved at '
              f'alpha={alpha * a2b:.3e} / angstrom\n')
        alpha_conv = alpha
        r_cut_conv = self.get_convergence_rcut(ev, alpha_conv, r_cut_max, self.lower_bound_real,
                                               self.upper_bound_rcut)
        print(f'alpha={alpha_conv * a2b:.3e} / angstrom; r_cut={r_cut_conv / r_cut_max:.3f} max L/2')
        down = 5
        print(f'Attempting to achieve convergence above {self.threshold_fraction * 100:.1f} '
              f'% of max L/2:')
        while r_cut_conv / r_cut_max < self.threshold_fraction:
            alpha_new = (1 - down / 100) * alpha_conv
            r_cut_new = self.get_convergence_rcut(ev, alpha_new, r_cut_max,
                                                  self.lower_bound_real, self.upper_bound_rcut)
            if r_cut_new / r_cut_max < self.upper_bound_rcut:
                r_cut_conv, alpha_conv = r_cut_new, alpha_new
                print(f'alpha={alpha_conv * a2b:.3e} / angstrom; '
                      f'r_cut={r_cut_conv / r_cut_max:.3f} max L/2')
            else:
                break
        real_space_parameters['r_cut'] = r_cut_conv
        real_space_parameters['alpha'] = alpha_conv
        print(f'Convergence in real-space energy achieved at alpha={alpha_conv * a2b:.3e} / '
              f'angstrom with r_cut={r_cut_conv / r_cut_max:.3f} max L/2\n')
        return real_space_parameters

    def get_step_change_analysis_with_k_cut(self, k_cut_data, fourier_space_energy_data):
        """Upward steps of the Fourier energy between neighbouring k_cut
        points (core.py:1128-1137)."""
        i0 = np.where(np.diff(fourier_space_energy_data) > self.step_increase_tol)[0]
        i1 = i0 + 1
        return (k_cut_data[i0], k_cut_data[i1],
                fourier_space_energy_data[i1] - fourier_space_energy_data[i0])

    def get_new_k_vectors(self, k_cut0, k_cut1):
        """Integer k with k_cut0^2 <= k^2 < k_cut1^2 (core.py:1152-1169)."""
        k_max = np.ceil(k_cut1 / self.reciprocal_lattice_vector_length).astype(int)
        grid = np.mgrid[-k_max[0]:k_max[0] + 1, -k_max[1]:k_max[1] + 1,
                        -k_max[2]:k_max[2] + 1].reshape(3, -1).T
        k = np.dot(grid, self.reciprocal_lattice_matrix)
        k2 = np.sum(k * k, axis=1)
        return grid[(k2 >= k_cut0 ** 2) & (k2 < k_cut1 ** 2)].tolist()

    def get_k_vector_based_energy_contribution(self, ev, alpha, k_cut0_of_step_change,
                                               k_cut1_of_step_change, prefix_list):
        """core.py:1186-1213."""
        new = []
        for k0, k1 in zip(k_cut0_of_step_change, k_cut1_of_step_change):
            new.extend(self.get_new_k_vectors(k0, k1))
        new = np.asarray(new)
        print(f'Identified a total of {len(new)} k-vectors contributing towards energy changes')
        contrib = ev.k_vectors(alpha, new)
        order = np.argsort(contrib)[::-1]
        prefix_list.append('k-vectors sorted in the decreasing order of their energy '
                           'contributions\n')
        for k, e in zip(new[order], contrib[order]):
            prefix_list.append(f'{k[0]:4d} {k[1]:4d} {k[2]:4d}: '
                               f'{e / constants.EV2HARTREE:.3e} eV\n')
        return prefix_list

    def _k_range_report(self, k_cut_lower, k_cut_upper):
        lo = np.ceil(k_cut_lower / self.reciprocal_lattice_vector_length).astype(int)
        hi = np.ceil(k_cut_upper / self.reciprocal_lattice_vector_length).astype(int)
        print(f'k_max vary from [{",".join(str(e) for e in lo)}] to '
              f'[{",".join(str(e) for e in hi)}]')
        print(f'Maximum number of k-vectors vary from {_num_k_vectors(lo)} to '
              f'{_num_k_vectors(hi)}')

    def get_precise_step_change_data(self, ev, alpha, k_cut_lower, k_cut_upper, dst_path,
                                     sub_prefix_list):
        """core.py:1215-1286 (figures not drawn)."""
        self._k_range_report(k_cut_lower, k_cut_upper)
        k_cut_data, energy = self.get_energy_profile_with_k_cut(
            ev, alpha, k_cut_lower, k_cut_upper, self.num_data_points_high)
        print('Generated energy profile\n')
        converged = energy[-1]
        print('Estimating the step energy changes in Fourier-space energy within this '
              'k_cut range:')
        k0_est, k1_est = self.get_step_change_analysis_with_k_cut(k_cut_data, energy)[:-1]
        k0s, k1s, changes = [], [], []
        print(f'Identified {len(k0_est)} preliminary step changes\n')
        max_divergent_k_cut = 0
        print('Analyzing each step energy change in detail:')
        for i in range(len(k0_est)):
            print(f'Analyzing step-change {i + 1}')
            lower, upper = k0_est[i], k1_est[i]
            self._k_range_report(lower, upper)
            step_k, step_e = self.get_energy_profile_with_k_cut(
                ev, alpha, lower, upper, self.step_change_data_points)
            divergent = step_k[abs(step_e - converged) > self.err_tol]
            if len(divergent) != 0:
                max_divergent_k_cut = max(divergent)
            a, b, c = self.get_step_change_analysis_with_k_cut(step_k, step_e)
            k0s.extend(a.tolist())
            k1s.extend(b.tolist())
            changes.extend(c.tolist())
        k0s, k1s, changes = np.asarray(k0s), np.asarray(k1s), np.asarray(changes)
        sub_prefix_list.append(f'Number of step changes in Fourier-space energy with '
                               f'varying k_cut: {len(changes)}\n')
        print(f'Identified a total of {len(changes)} step changes\n')
        return (k_cut_data, k0s, k1s, changes, max_divergent_k_cut, sub_prefix_list)

    def get_k_cut_choices(self, k_cut_data, k_cut0_of_step_change, k_cut1_of_step_change,
                          energy_changes, max_divergent_k_cut, k_cut_estimate,
                          sub_prefix_list):
        """core.py:1288-1318."""
        a2b = constants.ANG2BOHR
        b_len = self.reciprocal_lattice_vector_length
        gentle = k_cut_data[k_cut_data > max_divergent_k_cut][0] if max_divergent_k_cut > 0 else 0
        sub_prefix_list.append(f'k_cut (gentle): {gentle * a2b:.3e} / angstrom\n')
        k_max_g = np.ceil(gentle / b_len).astype(int)
        print(f'k_cut (gentle): {gentle * a2b:.3e} / angstrom; k_max: '
              f'[{",".join(str(e) for e in k_max_g)}]; num_k-vectors: {_num_k_vectors(k_max_g)}')
        stringent = k_cut1_of_step_change[-1]
        sub_prefix_list.append(f'k_cut (stringent): {stringent * a2b:.3e} / angstrom\n')
        k_max_s = np.ceil(stringent / b_len).astype(int)
        print(f'k_cut (stringent): {stringent * a2b:.3e} / angstrom; k_max: '
              f'[{",".join(str(e) for e in k_max_s)}]; num_k-vectors: '
              f'{_num_k_vectors(k_max_s)}\n')
        factor = stringent / k_cut_estimate
        sub_prefix_list.append(f'Factor of increase in the value of converged k_cut from '
                               f'estimation: {factor:.3e}\n')
        print('Analyzing convergence in step energy change:')
        ok = self.check_for_k_cut_step_energy_convergence(
            k_cut0_of_step_change, energy_changes, self.threshold_fraction * stringent, stringent)
        word = 'NOT ' if not ok else ''
        sub_prefix_list.append(f'Step energy changes have {word}converged\n')
        print(f'Step energy changes have {word}converged\n')
        return (stringent, sub_prefix_list)

    def get_optimized_r_cut(self, ev, alpha, choice_parameters, dst_path, prefix_list):
        """core.py:1320-1355; the unsupported-alpha exit writes the report and
        raises SystemExit as the reference's exit() does."""
        r_cut_max = min(self.translational_vector_length) / 2
        r_data, energy = self.get_energy_profile_with_r_cut(
            ev, alpha, r_cut_max, self.lower_bound_rcut, self.upper_bound_rcut,
            self.num_data_points_high)
        if self.convergence_check_with_r_cut(ev, alpha, r_cut_max, self.threshold_fraction,
                                             self.upper_bound_rcut):
            conv = energy[-1]
            if self.precise_r_cut:
                lower = r_data[abs(energy - conv) > self.err_tol][-1] / r_cut_max
                upper = r_data[abs(energy - conv) < self.err_tol][0] / r_cut_max
                r_local, e_local = self.get_energy_profile_with_r_cut(
                    ev, alpha, r_cut_max, lower, upper, self.num_data_points_high)
                return r_local[abs(e_local - conv) < self.err_tol][0]
            return r_data[abs(energy - conv) < self.err_tol][0]
        a = alpha * constants.ANG2BOHR
        msg = (f'This code doesn\'t support user-specified alpha={a:.3e} as r_cut is over '
               f'L/2. Please re-run at a suitable alpha value.')
        print(msg)
        prefix_list.append(f'alpha: {a:.3e} / angstrom ({choice_parameters["r_cut"]})\n')
        prefix_list.append(msg + '\n\n')
        generate_report(self.start_time, dst_path, 'precomputed_array', 1, ''.join(prefix_list))
        raise SystemExit

    def get_cutoff_parameters(self, tau_ratio, dst_path, prefix_list):
        """The choice of alpha, r_cut and k_cut (core.py:1357-1557)."""
        a2b = constants.ANG2BOHR
        real, fourier = {}, {}
        if np.isreal(self.alpha):
            alpha_choice = 'user-specified'
            alpha = real['alpha'] = self.alpha
            fourier['alpha'] = self.alpha
        else:
            alpha_choice = 'optimal'
        if np.isreal(self.r_cut):
            r_cut_choice = 'user-specified'
            r_cut = real['r_cut'] = self.r_cut
        elif self.r_cut == 'simulation_cell':
            r_cut_choice = 'simulation_cell'
            k_cut_choice = 'imported'
        else:
            r_cut_choice = 'optimal'
        unit_cell = np.array_equal(self.system_size, np.ones(self.neighbors.n_dim, int))
        if self.r_cut != 'simulation_cell':
            if isinstance(self.k_cut, list):
                k_cut = 1.10 * max(np.asarray(self.k_cut) * self.reciprocal_lattice_vector_length)
                print(f'At the user-specified k_max=[{",".join(str(e) for e in self.k_cut)}], '
                      f'k_cut={k_cut * a2b:.3e} / angstrom')
                print(f'Maximum number of k-vectors: {_num_k_vectors(self.k_cut)}')
                k_cut_choice = 'user-specified (k_max)'
            elif np.isreal(self.k_cut):
                k_cut_choice = 'user-specified'
                k_cut = fourier['k_cut'] = self.k_cut
            elif self.k_cut == 'converge' and unit_cell:
                k_cut_choice = 'converge'
            else:
                k_cut_choice = 'optimal'
        choice = {'alpha': alpha_choice, 'r_cut': r_cut_choice, 'k_cut': k_cut_choice}
        ev = self._energy_evaluator('full')
        charge_list = self.base_charge_config_for_accuracy_analysis('full')
        einsum = float(np.einsum('ii', np.multiply(charge_list.transpose(), charge_list)))
        xr = xf = 0.5
        vdl = np.power(self.system_volume, 1 / 3)
        if self.r_cut == 'simulation_cell':
            real = self.get_simulation_cell_real_space_parameters(ev, einsum, real, xr, dst_path)
            alpha, r_cut = real['alpha'], real['r_cut']
            ones = np.ones(self.neighbors.n_dim, int)
            dst_path = Path(dst_path)
            conv_dir = (dst_path.resolve().parents[1]
                        / ('SystemSize[' + ','.join(str(e) for e in ones) + ']')
                        / dst_path.parts[-1] / f'alpha={alpha * a2b:.3e}')
            if not conv_dir.exists():
                msg = (f'Please re-run after converging k_cut at alpha={alpha * a2b:.3e} for '
                       f'system size [{",".join(str(e) for e in ones)}]')
                print(msg)
                prefix_list.append(f'alpha: {alpha * a2b:.3e} / angstrom ({choice["r_cut"]})\n')
                prefix_list.append(f'r_cut: {r_cut / a2b:.3e} angstrom ({choice["r_cut"]})\n')
                n_max = np.round(r_cut / self.translational_vector_length).astype(int)
                prefix_list.append(f'n_max: [{n_max[0]}, {n_max[1]}, {n_max[2]}]\n')
                prefix_list.append(msg + '\n\n')
                generate_report(self.start_time, dst_path, 'precomputed_array', 1,
                                ''.join(prefix_list))
                raise SystemExit
            with open(conv_dir / 'k_cut_convergence.log') as fh:
                for i, line in enumerate(fh):
                    if i == 3:  # the stringent k_cut
                        k_cut = float(line[19:28]) / a2b
            fourier = self.minimize_fourier_space_cutoff_error(einsum, vdl, {'alpha': alpha}, xf)
        elif self.k_cut == 'converge' and unit_cell:
            sub01 = []
            print(f'Attempting to converge k_cut for user-specified alpha={alpha * a2b:.3e} '
                  f'/ angstrom:\n')
            out_dir = Path(dst_path) / f'alpha={alpha * a2b:.3e}'
            out_dir.mkdir(parents=True, exist_ok=True)
            fourier = self.minimize_fourier_space_cutoff_error(einsum, vdl, fourier, xf)
            k_cut_estimate = fourier['k_cut']
            print(f'Starting with an estimate for k_cut={k_cut_estimate * a2b:.3e} / angstrom')
            print(f'Exploring convergence in Fourier-space energy between '
                  f'{int(self.lower_bound_kcut)}x and {int(self.upper_bound_kcut)}x of '
                  f'estimated k_cut')
            k_cut_upper = self.upper_bound_kcut * k_cut_estimate
            k_cut_threshold = self.threshold_fraction * k_cut_upper
            while not self.convergence_check_with_k_cut(ev, alpha, k_cut_threshold, k_cut_upper):
                k_cut_upper = (1 + 10 / 100) * k_cut_upper
                print('Could not find convergence in given k_cut range. Re-attempting with '
                      f'upper bound increased by {10:.3f} %')
            sub01.append(f'Preliminary convergence in Fourier-space energy achieved at k_cut: '
                         f'{k_cut_upper * a2b:.3e} / angstrom\n')
            print(f'Preliminary convergence in absolute value of Fourier-space energy achieved '
                  f'within k_cut={k_cut_upper * a2b:.3e} / angstrom\n')
            print('Attempting to identify precise k_cut:')
            dst_path = out_dir
            k_cut_lower = self.lower_bound_kcut * k_cut_estimate
            k_cut_upper = self.upper_bound_kcut * k_cut_estimate
            print(f'Generating energy profile between {int(self.lower_bound_kcut)}x and '
                  f'{int(self.upper_bound_kcut)}x of estimated k_cut')
            (k_data, k0s, k1s, changes, max_div, sub01) = self.get_precise_step_change_data(
                ev, alpha, k_cut_lower, k_cut_upper, out_dir, sub01)
            k_cut, sub01 = self.get_k_cut_choices(k_data, k0s, k1s, changes, max_div,
                                                  k_cut_estimate, sub01)
            print('Analyzing energy contributions of individual k-vectors:')
            sub02 = self.get_k_vector_based_energy_contribution(ev, alpha, k0s, k1s, [])
            generate_report(self.start_time, dst_path, 'k_vector_energy_contribution', 0,
                            ''.join(sub02))
            print('Finished k-vector analysis')
            generate_report(self.start_time, out_dir, 'k_cut_convergence', 0, ''.join(sub01))
        elif not (np.isreal(self.alpha) and np.isreal(self.r_cut)
                  and (self._k_cut_given())):
            if np.isreal(self.alpha) & np.isreal(self.r_cut):
                fourier = self.minimize_fourier_space_cutoff_error(einsum, vdl, fourier, xf)
                k_cut = fourier['k_cut']
            elif np.isreal(self.alpha) & self._k_cut_given():
                r_cut = self.get_optimized_r_cut(ev, alpha, choice, dst_path, prefix_list)
            elif np.isreal(self.r_cut) and self._k_cut_given():
                real = self.minimize_real_space_cutoff_error(einsum, real, xr)
                alpha = real['alpha']
            elif np.isreal(self.alpha):
                r_cut = self.get_optimized_r_cut(ev, alpha, choice, dst_path, prefix_list)
                print(f'Convergence in real-space energy achieved at alpha={alpha * a2b:.3e} / '
                      f'angstrom with r_cut:{r_cut / a2b:.3e}\n')
                fourier = self.minimize_fourier_space_cutoff_error(einsum, vdl, fourier, xf)
                k_cut = fourier['k_cut']
            elif np.isreal(self.r_cut):
                real = self.minimize_real_space_cutoff_error(einsum, real, xr)
                alpha = fourier['alpha'] = real['alpha']
                fourier = self.minimize_fourier_space_cutoff_error(einsum, vdl, fourier, xf)
                k_cut = fourier['k_cut']
            elif self._k_cut_given():
                fourier = self.minimize_fourier_space_cutoff_error(einsum, vdl, fourier, xf)
                alpha = real['alpha'] = fourier['alpha']
                r_cut = self.get_optimized_r_cut(ev, alpha, choice, dst_path, prefix_list)
            else:
                # alpha balancing the measured real / Fourier costs (core.py:1543-1545)
                alpha = (tau_ratio * np.pi ** 3 / (self.system_volume) ** 2) ** (1 / 6)
                real['alpha'] = fourier['alpha'] = alpha
                r_cut = self.get_optimized_r_cut(ev, alpha, choice, dst_path, prefix_list)
                fourier = self.minimize_fourier_space_cutoff_error(einsum, vdl, fourier, xf)
                k_cut = fourier['k_cut']
        return (alpha, r_cut, k_cut, choice, einsum, vdl, prefix_list, dst_path)

    def get_ewald_parameters(self, prefix_list, dst_path):
        """Benchmark, choose and report alpha, r_cut, k_cut (core.py:1559-1592)."""
        a2b = constants.ANG2BOHR
        bench = {'n_max': np.zeros(self.pbc.shape, int), 'k_max': np.ones(self.pbc.shape, int),
                 'alpha': 0.5, 'r_cut': min(self.translational_vector_length) / 2.1,
                 'k_cut': max(self.reciprocal_lattice_vector_length)}
        tau_ratio, time_ratio = self.benchmark_ewald(1, bench)
        prefix_list.append(f'tau_ratio, (tau_r/tau_f): {tau_ratio:.3e}\n')
        prefix_list.append(f'time_ratio, (time_r/time_f): {time_ratio:.3e}\n\n')
        (alpha, r_cut, k_cut, choice, einsum, vdl, prefix_list, dst_path) = \
            self.get_cutoff_parameters(tau_ratio, dst_path, prefix_list)
        prefix_list.append(f'alpha: {alpha * a2b:.3e} / angstrom ({choice["alpha"]})\n')
        prefix_list.append(f'r_cut: {r_cut / a2b:.3e} angstrom ({choice["r_cut"]})\n')
        prefix_list.append(f'k_cut: {k_cut * a2b:.3e} / angstrom ({choice["k_cut"]})\n')
        prefix_list = self.compute_cutoff_errors(einsum, alpha, r_cut, k_cut, vdl, prefix_list)
        return ({'alpha': alpha, 'r_cut': r_cut, 'k_cut': k_cut}, prefix_list, dst_path)
