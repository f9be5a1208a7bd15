"""ORACLE (test infrastructure only) - CPU restatement of PyCD's mean squared
displacement analysis, Analysis.compute_msd.  Never imported by the product
package; used by tests/ as the checker.

Pinned: ``compute_msd`` reproduces the reference's own output on the shipped
examples/Hematite trajectory with the example's MSD parameters and on a
synthetic three-species-type case (tests/golden/msd.*, written by
tests/golden/make_golden.py from the reference's Analysis.compute_msd).

It follows, in NumPy:
  unit setup           PyCD/core.py:2922-2972
  squared displacement PyCD/core.py:2983-3005 (mean over all row pairs at a lag)
  species averages     PyCD/core.py:3006-3024
  MSD / SEM tables     PyCD/core.py:3026-3034
  file name            PyCD/core.py:3035-3040
  slopes, diffusivity  PyCD/core.py:3053-3073 (linregress on the trimmed range)
"""
import numpy as np
from scipy.stats import linregress

# unit constants in the reference's order of evaluation (PyCD/constants.py)
_PI = 3.14159265358979323846
_KE = 1 / (4 * _PI * 8.854187817E-12)
_BOHR = 1.054571800E-34 ** 2 / (9.10938356E-31 * 1.6021766208E-19 ** 2 * _KE)
_HARTREE = 1.054571800E-34 ** 2 / (9.10938356E-31 * _BOHR ** 2)
_AUTIME = 1.054571800E-34 / _HARTREE
_SEC2AUTIME = 1 / _AUTIME
_SEC2NS = 1.00E+09
_AUTIME2NS = _SEC2NS / _SEC2AUTIME
_AUTIME2PS = 1.00E+12 / _SEC2AUTIME
_AUTIME2FS = 1.00E+15 / _SEC2AUTIME
_ANG2BOHR = 1E-10 / _BOHR
_ANG2CM = 1.00e-08
_KB = 1.38064852E-23
_EV2J = 1.6021766208E-19

TIME_CONVERSION = {"ns": _AUTIME2NS, "ps": _AUTIME2PS, "fs": _AUTIME2FS,
                   "s": 1E+00 / _SEC2AUTIME}
DIST_CONVERSION = {"m": _BOHR, "um": 1.00E-04 / _ANG2BOHR,
                   "angstrom": 1E+00 / _ANG2BOHR}


def squared_displacements(positions, n_lags):
    """positions: (R, S, 3) of one trajectory -> (n_lags, S) mean squared
    displacement over every pair of rows `lag` apart (row 0 = 0)."""
    R = positions.shape[0]
    sd = np.zeros((n_lags, positions.shape[1]))
    for lag in range(1, n_lags):
        d = positions[lag:] - positions[:R - lag]
        sd[lag] = np.mean(np.einsum("ijk,ijk->ij", d, d), axis=0)
    return sd


def compute_msd(rows, species_types, species_count, n_dim, t_final, time_interval,
                msd_t_final, trim_length, temp, repr_time="ns", repr_dist="angstrom"):
    """rows: (n_traj, >= R, 3 * sum(species_count)) unwrapped trajectory rows
    in bohr.  Returns a dict with msd_data, sem_data, species_avg, slopes,
    diffusivity, diffusivity_sem, species_types, file_name, report_prefix."""
    rows = np.asarray(rows, dtype=np.float64)
    n_traj = rows.shape[0]
    species_count = np.asarray(species_count)
    total = int(species_count.sum())
    tc = TIME_CONVERSION[repr_time]
    dc = DIST_CONVERSION[repr_dist]
    t_final_au = t_final * _SEC2AUTIME
    dt_au = time_interval * _SEC2AUTIME
    R = int(t_final_au / dt_au) + 1
    msd_t_final_au = msd_t_final / tc
    L = int(msd_t_final_au / dt_au) + 1
    kBT = _KB * temp / _EV2J
    pos = rows[:, :R].reshape(n_traj, R, total, 3) * dc
    sd = np.stack([squared_displacements(pos[t], L) for t in range(n_traj)])
    present = [i for i, c in enumerate(species_count) if c != 0]
    bounds = np.concatenate([[0], np.cumsum(species_count)])
    species_avg = np.stack([sd[:, :, bounds[i]:bounds[i + 1]].mean(axis=2)
                            for i in present], axis=2)
    msd_data = np.zeros((L, len(present) + 1))
    msd_data[:, 0] = np.arange(L) * dt_au * tc
    msd_data[:, 1:] = species_avg.mean(axis=0)
    sem_data = species_avg.std(axis=0) / np.sqrt(n_traj)
    file_name = ("%1.2E" % (msd_t_final_au * tc)) + str(repr_time) + "_trim=" + str(trim_length)
    names = [species_types[i] for i in present]
    lo, hi = trim_length, L - trim_length
    slopes = np.zeros((n_traj, len(present)))
    lines, diff, diff_sem = [], [], []
    for s, name in enumerate(names):
        for t in range(n_traj):
            slopes[t, s] = linregress(msd_data[lo:hi, 0], species_avg[t, lo:hi, s])[0]
        factor = _ANG2CM ** 2 * _SEC2NS / (2 * n_dim) / kBT
        d = np.mean(slopes[:, s]) * factor
        d_sem = np.std(slopes[:, s]) / np.sqrt(n_traj) * factor
        diff.append(d)
        diff_sem.append(d_sem)
        lines.append(f"Estimated value of {name} diffusivity is: {d:.3e} cm2/Vs\n")
        lines.append(f"Standard error of mean in {name} diffusivity is: {d_sem:.3e} cm2/Vs\n")
    return {"msd_data": msd_data, "sem_data": sem_data, "species_avg": species_avg,
            "sd": sd, "slopes": slopes, "diffusivity": np.array(diff),
            "diffusivity_sem": np.array(diff_sem), "species_types": names,
            "file_name": file_name, "report_prefix": "".join(lines),
            "n_rows": R, "n_lags": L}
