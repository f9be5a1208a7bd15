"""Mean squared displacement analysis: PyCD's ``Analysis`` (core.py:2920-3081)
with the squared displacements and their averages on the GPU.

``Analysis(...).compute_msd(dst_path, output_data)`` reads the trajectories
``traj{i}/unwrapped_traj.npy`` that ``Run.do_kmc_steps`` wrote, as the
reference does, and returns the same ``ReturnValues(msd_data, sem_data,
species_types, file_name)``, writing ``MSD_Data_<file_name>.npy`` and the
``MSD_Analysis_<file_name>.log`` report.  ``msd_device`` runs the same
analysis on rows that are already in device memory, such as the unwrapped
rows of a batched KMC run, without a round trip through files.

Every array reduction runs in libpycd_gb300 (``pycd_msd_compute``); the
host computes only the unit factors and formats the report.  Plotting
(``generate_msd_plot``) is not provided.
"""
import ctypes as C
from datetime import datetime
from pathlib import Path

import numpy as np

from . import _native as nat
from . import constants
from .io import generate_report
from .lattice import ReturnValues


def msd_device(rows, species_count, n_rows, n_lags, trim_length, dist_conversion,
               time_interval, time_conversion, n_species=None, stream=None):
    """MSD analysis of unwrapped rows in device memory.

    ``rows``: CUDA float64 tensor of shape (n_traj, >= n_rows, >= 3 * n_species)
    (extra rows and trailing columns are skipped through the strides), in
    bohr, carriers grouped by species type in the order of ``species_count``.
    ``time_interval`` is in atomic units.  Returns a dict of device tensors:
    sd (n_traj, n_lags, n_species), species_avg (n_traj, n_lags, n_types),
    msd_data (n_lags, n_types + 1), sem_data (n_lags, n_types), slopes
    (n_traj, n_types), slope_stats (2, n_types: mean and standard error),
    plus ``types``: indices of the species types present."""
    import torch
    if rows.dtype != torch.float64 or not rows.is_cuda or rows.dim() != 3:
        raise ValueError("rows must be a 3-d float64 CUDA tensor")
    if rows.stride(2) != 1:
        raise ValueError("rows must have unit stride in its last dimension")
    counts = [int(c) for c in species_count]
    types = [i for i, c in enumerate(counts) if c != 0]
    S = int(sum(counts)) if n_species is None else int(n_species)
    if S != sum(counts):
        raise ValueError("n_species must equal sum(species_count)")
    if len(types) > nat.MSD_MAX_TYPES:
        raise ValueError("at most %d species types" % nat.MSD_MAX_TYPES)
    T = rows.shape[0]
    if rows.shape[1] < n_rows or rows.shape[2] < 3 * S:
        raise ValueError("rows hold %s, need (n_traj, >= %d, >= %d)"
                         % (tuple(rows.shape), n_rows, 3 * S))
    d = nat.MsdDesc()
    d.d_rows = rows.data_ptr()
    d.n_traj, d.n_rows = T, int(n_rows)
    d.traj_stride, d.row_stride = rows.stride(0), rows.stride(1)
    d.n_species, d.n_types = S, len(types)
    for j, k in enumerate(types):
        d.type_count[j] = counts[k]
    d.n_lags, d.trim_length = int(n_lags), int(trim_length)
    d.dist_conversion = float(dist_conversion)
    d.time_interval = float(time_interval)
    d.time_conversion = float(time_conversion)
    K, L = len(types), int(n_lags)
    f64 = dict(dtype=torch.float64, device=rows.device)
    out = {"sd": torch.empty((T, L, S), **f64),
           "species_avg": torch.empty((T, L, K), **f64),
           "msd_data": torch.empty((L, K + 1), **f64),
           "sem_data": torch.empty((L, K), **f64),
           "slopes": torch.empty((T, K), **f64),
           "slope_stats": torch.empty((2, K), **f64)}
    fit = L - 2 * int(trim_length) >= 2
    nat.check(nat.lib().pycd_msd_compute(
        C.byref(d), out["sd"].data_ptr(), out["species_avg"].data_ptr(),
        out["msd_data"].data_ptr(), out["sem_data"].data_ptr(),
        out["slopes"].data_ptr() if fit else None,
        out["slope_stats"].data_ptr() if fit else None, nat.stream_handle(stream)))
    if not fit:
        del out["slopes"], out["slope_stats"]
    out["types"] = types
    return out


class Analysis(object):
    """Post-simulation analysis (PyCD/core.py:2920-2972): the same
    constructor, unit handling and step counts as the reference."""

    def __init__(self, material_info, n_dim, species_count, n_traj, t_final,
                 time_interval, msd_t_final, trim_length, temp, repr_time='ns',
                 repr_dist='Angstrom'):
        self.start_time = datetime.now()
        self.material = material_info
        self.n_dim = n_dim
        self.species_count = np.asarray(species_count)
        self.total_species = self.species_count.sum()
        self.n_traj = int(n_traj)
        self.t_final = t_final * constants.SEC2AUTIME
        self.time_interval = time_interval * constants.SEC2AUTIME
        self.trim_length = trim_length
        self.temp = temp
        self.num_path_steps_per_traj = int(self.t_final / self.time_interval) + 1
        self.repr_time = repr_time
        self.repr_dist = repr_dist
        # unknown unit names leave the conversion unset, as in the reference
        time_conv = {'ns': constants.AUTIME2NS, 'ps': constants.AUTIME2PS,
                     'fs': constants.AUTIME2FS, 's': 1E+00 / constants.SEC2AUTIME}
        dist_conv = {'m': constants.BOHR, 'um': constants.BOHR2UM,
                     'angstrom': 1E+00 / constants.ANG2BOHR}
        if repr_time in time_conv:
            self.time_conversion = time_conv[repr_time]
        if repr_dist in dist_conv:
            self.dist_conversion = dist_conv[repr_dist]
        self.kBT = constants.KB * self.temp / constants.EV2J  # eV
        self.msd_t_final = msd_t_final / self.time_conversion
        self.num_msd_steps_per_traj = int(self.msd_t_final / self.time_interval) + 1

    @property
    def file_name(self):
        """Output name stem (core.py:3035-3040)."""
        return (('%1.2E' % (self.msd_t_final * self.time_conversion))
                + str(self.repr_time) + '_trim=' + str(self.trim_length))

    def _load_rows(self, dst_path, output_data):
        """Trajectory files stacked and cut as core.py:2981-2990 does."""
        name = output_data['unwrapped_traj']['file_name']
        parts = [np.load(Path(dst_path) / f'traj{i + 1}' / name)
                 for i in range(self.n_traj)]
        rows = np.vstack(parts)[:self.n_traj * self.num_path_steps_per_traj + 1]
        return rows.reshape((self.n_traj, self.num_path_steps_per_traj,
                             int(self.total_species) * 3))

    def compute_msd_device(self, rows, stream=None):
        """The analysis of ``compute_msd`` on device rows (see msd_device)."""
        return msd_device(rows, self.species_count, self.num_path_steps_per_traj,
                          self.num_msd_steps_per_traj, self.trim_length,
                          self.dist_conversion, self.time_interval,
                          self.time_conversion, stream=stream)

    def diffusivity(self, slope):
        """D / kBT in cm2/Vs from an MSD slope (core.py:3061-3072)."""
        return (slope * constants.ANG2CM ** 2 * constants.SEC2NS
                / (2 * self.n_dim) / self.kBT)

    def compute_msd(self, dst_path, output_data):
        """MSD table, SEM table, report and data file (core.py:2974-3081)."""
        import torch
        assert dst_path, 'Please provide the destination path where MSD ' \
                         'output files needs to be saved'
        dst_path = Path(dst_path)
        nat.require_device()
        host = torch.from_numpy(np.ascontiguousarray(
            self._load_rows(dst_path, output_data), dtype=np.float64))
        res = self.compute_msd_device(host.cuda())
        msd_data = res["msd_data"].cpu().numpy()
        sem_data = res["sem_data"].cpu().numpy()
        stats = res["slope_stats"].cpu().numpy() if "slope_stats" in res else None
        if stats is None:
            raise ValueError("the slope fit needs at least 2 lags between the "
                             "trim lengths")
        species_types = [self.material.species_types[i] for i in res["types"]]
        file_name = self.file_name
        np.save(dst_path / ''.join(['MSD_Data_', file_name, '.npy']), msd_data)
        lines = []
        for j, species_type in enumerate(species_types):
            species_diff = self.diffusivity(stats[0, j])
            lines.append(f'Estimated value of {species_type} diffusivity is: '
                         f'{species_diff:.3e} cm2/Vs\n')
            species_diff_sem = self.diffusivity(stats[1, j])
            lines.append(f'Standard error of mean in {species_type} diffusivity '
                         f'is: {species_diff_sem:.3e} cm2/Vs\n')
        report_file_name = ''.join(['MSD_Analysis', ('_' if file_name else ''),
                                    file_name])
        generate_report(self.start_time, dst_path, report_file_name, 1, ''.join(lines))
        return ReturnValues(msd_data=msd_data, sem_data=sem_data,
                            species_types=species_types, file_name=file_name)
