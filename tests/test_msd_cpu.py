"""CPU: the MSD oracle against the reference's own Analysis.compute_msd
output (pins the oracle), and the host side of pycd_gb300.analysis."""
import types

import numpy as np
import pytest

import golden_io as gio
from oracle import msd_oracle as mo
from pycd_gb300.analysis import Analysis


def _case(name):
    cfg, arr = gio.load("msd")
    c = cfg[name]
    pre = "hem" if name == "hematite" else "syn"
    rows = arr[pre + "_rows"]
    if rows.ndim == 2:
        rows = rows[None]
    return c, rows, arr[pre + "_msd"], arr[pre + "_sem"]


def _analysis(c):
    mat = types.SimpleNamespace(species_types=c["species_types"],
                                num_species_types=len(c["species_types"]))
    return Analysis(mat, c["n_dim"], c["species_count"], c["n_traj"], c["t_final"],
                    c["time_interval"], c["msd_t_final"], c["trim_length"], c["temp"],
                    c["repr_time"], c["repr_dist"])


@pytest.mark.parametrize("name", ["hematite", "synthetic"])
def test_oracle_msd_reproduces_reference(name):
    c, rows, msd, sem = _case(name)
    o = mo.compute_msd(rows, c["species_types"], c["species_count"], c["n_dim"],
                       c["t_final"], c["time_interval"], c["msd_t_final"],
                       c["trim_length"], c["temp"], c["repr_time"], c["repr_dist"])
    assert np.array_equal(o["msd_data"], msd)
    assert np.array_equal(o["sem_data"], sem)
    assert o["file_name"] == c["file_name"]
    assert o["report_prefix"] == c["report_prefix"]
    assert o["species_types"] == c["out_species"]


@pytest.mark.parametrize("name", ["hematite", "synthetic"])
def test_analysis_host_setup_matches_reference(name):
    """Step counts, unit factors and the file name are host arithmetic in
    the reference's order; they must agree with the reference's outputs."""
    c, rows, msd, sem = _case(name)
    an = _analysis(c)
    assert an.num_msd_steps_per_traj == msd.shape[0]
    assert an.num_path_steps_per_traj == rows.shape[1]
    assert an.file_name == c["file_name"]
    # the time column is (lag * dt) * time_conversion
    lags = np.arange(an.num_msd_steps_per_traj)
    assert np.array_equal(lags * an.time_interval * an.time_conversion, msd[:, 0])


def test_analysis_unknown_distance_unit_fails_like_reference():
    c, _, _, _ = _case("hematite")
    c = dict(c, repr_dist="Angstrom")  # the reference's default spelling
    an = _analysis(c)
    with pytest.raises(AttributeError):
        an.dist_conversion


def test_analysis_reads_trajectory_files_as_reference(tmp_path):
    c, rows, _, _ = _case("synthetic")
    for i, r in enumerate(rows):
        (tmp_path / f"traj{i + 1}").mkdir()
        np.save(tmp_path / f"traj{i + 1}" / "unwrapped_traj.npy", r)
    an = _analysis(c)
    got = an._load_rows(tmp_path, {"unwrapped_traj": {"file_name": "unwrapped_traj.npy"}})
    assert np.array_equal(got, rows)
