"""HDF5 trajectory output (PyCD/hdf5_io.py, PyCD/core.py:2677-2691 and
2882-2902) against the reference's own writer, recorded through the h5py
stand-in tests/fake_h5py.py (tests/golden/hdf5.*); the cases of the
reference's PyCD/tests/test_hdf5_io.py; and Run's gate for the output."""
import importlib
import sys
import tempfile
import types
from pathlib import Path

import numpy as np
import pytest

import fake_h5py
import golden_io as gio
from pycd_gb300 import constants
from pycd_gb300.core import Run


@pytest.fixture
def h5(monkeypatch):
    """pycd_gb300.hdf5_io imported over the stand-in."""
    monkeypatch.setitem(sys.modules, "h5py", fake_h5py)
    monkeypatch.delitem(sys.modules, "pycd_gb300.hdf5_io", raising=False)
    mod = importlib.import_module("pycd_gb300.hdf5_io")
    yield mod
    sys.modules.pop("pycd_gb300.hdf5_io", None)


def _fixture():
    ref, arr = gio.load("hdf5")
    arrays = {k.replace("|", "/"): v for k, v in arr.items()}
    return ref, arrays


def _same_file(path, ref_records, ref_arrays, prefix, check_time=True):
    got = fake_h5py.load(path)
    assert sorted(got) == sorted(ref_records)
    for key, want in ref_records.items():
        g = got[key]
        if want.get("group"):
            assert g.get("group") and g["attrs"] == want["attrs"]
            continue
        d = g["data"]
        assert d.dtype.str == want["dtype"] and list(d.shape) == want["shape"], key
        assert [None if m is None else int(m) for m in g["maxshape"]] == want["maxshape"]
        assert g["chunks"] == want["chunks"] and g["compression"] == want["compression"]
        assert g["attrs"] == want["attrs"]
        if key == "/time" and not check_time:
            continue
        assert np.array_equal(d, ref_arrays[prefix + key]), key


def test_writer_frames_match_reference(h5, tmp_path):
    """write_frame, then write_frames of (frames, 3 n_atoms) rows: the same
    datasets, types, creation arguments, attributes and values as the
    reference's writer."""
    ref, arrays = _fixture()
    coords = arrays["frames_in_coords"]
    with h5.HDF5TrajectoryWriter(tmp_path / "frames.h5", 3, 1) as w:
        w.write_frame(coords[0].ravel(), 0.5)
        w.write_frames(coords[1:].reshape(3, 9), np.array([1.5, 2.5, 4.0]))
    _same_file(tmp_path / "frames.h5", ref["records"]["frames"], arrays, "frames")


def test_save_trajectory_matches_reference(h5, tmp_path):
    """save_trajectory_hdf5 of a 2-D array with times and n_atoms, and of a
    1-D array alone (one frame, time 0)."""
    ref, arrays = _fixture()
    h5.save_trajectory_hdf5(tmp_path / "s2.h5", arrays["save2d_in_coords"],
                            np.arange(4, dtype=float), n_atoms=2)
    _same_file(tmp_path / "s2.h5", ref["records"]["save2d"], arrays, "save2d")
    h5.save_trajectory_hdf5(tmp_path / "s1.h5", arrays["save1d_in_coords"])
    _same_file(tmp_path / "s1.h5", ref["records"]["save1d"], arrays, "save1d")


def test_writer_layout_units_and_topology(h5, tmp_path):
    """The checks of the reference's test_hdf5_trajectory_writer and
    test_hdf5_single_frame."""
    n_atoms, n_frames = 3, 5
    coords = np.random.default_rng(1).random((n_frames, n_atoms, 3)) * 10.0
    path = tmp_path / "t.h5"
    with h5.HDF5TrajectoryWriter(path, n_atoms, 1) as w:
        w.write_frames(coords, np.arange(n_frames, dtype=float))
    assert path.exists()
    with fake_h5py.File(path, "r") as f:
        for name in ("coordinates", "time", "topology", "topology/atoms",
                     "topology/atoms/name", "topology/atoms/element", "topology/atoms/index"):
            assert name in f
        assert f["coordinates"].shape == (n_frames, n_atoms, 3)
        assert f["time"].shape == (n_frames,)
        assert f["coordinates"].attrs["units"] == "nanometers"
        assert f["time"].attrs["units"] == "picoseconds"
        assert len(f["topology/atoms/name"]) == n_atoms
        assert f["topology/atoms/name"][2] == b"ATOM2"
        assert np.array_equal(f["time"][:], np.arange(n_frames) * constants.AUTIME2PS)
    one = tmp_path / "one.h5"
    with h5.HDF5TrajectoryWriter(one, 2, 1) as w:
        w.write_frame(np.array([[1.0, 2.0, 3.0], [4.0, 5.0, 6.0]]), 0.0)
    with fake_h5py.File(one, "r") as f:
        assert f["coordinates"].shape == (1, 2, 3) and f["time"].shape == (1,)


def test_hdf5_and_npy_agree(h5, tmp_path):
    """The reference's test_hdf5_cross_format_consistency: the file's
    coordinates, taken back to bohr, equal the rows within float32 (1e-6)."""
    rows = np.random.default_rng(2).random((3, 6)) * 10.0
    h5.save_trajectory_hdf5(tmp_path / "c.h5", rows, np.arange(3, dtype=float), n_atoms=2)
    with fake_h5py.File(tmp_path / "c.h5", "r") as f:
        back = f["coordinates"][:].reshape(3, 6) / (0.1 / constants.ANG2BOHR)
    np.testing.assert_allclose(rows, back, rtol=1e-6)


def test_writer_errors(h5, tmp_path):
    """A path that cannot be created raises (the reference's
    test_hdf5_error_handling).  A time list that is not one per frame is
    refused before anything is written (the reference writes the
    coordinates first)."""
    with pytest.raises(Exception):
        with h5.HDF5TrajectoryWriter(tmp_path / "no" / "such" / "dir.h5", 2, 1):
            pass
    path = tmp_path / "m.h5"
    with h5.HDF5TrajectoryWriter(path, 1, 1) as w:
        with pytest.raises(ValueError):
            w.write_frames(np.zeros((4, 3)), np.zeros(5))
    with fake_h5py.File(path, "r") as f:
        assert f["coordinates"].shape == (0, 1, 3) and f["time"].shape == (0,)


def test_writer_append_continues(h5, tmp_path):
    path = tmp_path / "a.h5"
    rows = np.arange(12, dtype=float).reshape(4, 3)
    with h5.HDF5TrajectoryWriter(path, 1, 1) as w:
        w.write_frames(rows[:2], np.array([0.0, 1.0]))
    with h5.HDF5TrajectoryWriter(path, 1, 1, append=True) as w:
        w.write_frames(rows[2:], np.array([2.0, 3.0]))
    with fake_h5py.File(path, "r") as f:
        assert f["coordinates"].shape == (4, 1, 3)
        assert np.array_equal(f["coordinates"][:].reshape(4, 3),
                              (rows / constants.ANG2BOHR * 0.1).astype(np.float32))
        assert np.array_equal(f["time"][:], np.arange(4.0) * constants.AUTIME2PS)


def _run_like(n_species=1, dt=3.5):
    return types.SimpleNamespace(total_species=n_species,
                                 species_count=np.array([n_species, 0]),
                                 time_interval=dt)


OUT = {"time": {"file_name": "time_data.npy", "write": 1},
       "unwrapped_traj": {"file_name": "unwrapped_traj.npy", "write": 1,
                          "write_every_step": 0},
       "hdf5_output": {"enabled": True, "file_name": "trajectory.h5"}}


def test_run_hdf5_gate_and_frame_times(h5, tmp_path, capsys):
    """Run._write_hdf5: written only when enabled with the unwrapped rows
    written; grid rows get r * time_interval, per-step rows time_data[k + 1];
    a failing write prints the reference's warning and returns."""
    rows = np.random.default_rng(3).random((5, 3))
    steps_t = np.cumsum(np.r_[0.0, np.random.default_rng(4).random(5)])
    run = _run_like()
    Run._write_hdf5(run, tmp_path, OUT, rows, steps_t, False)
    with fake_h5py.File(tmp_path / "trajectory.h5", "r") as f:
        assert np.array_equal(f["time"][:], np.arange(5) * 3.5 * constants.AUTIME2PS)
        assert np.array_equal(f["coordinates"][:].reshape(5, 3),
                              (rows / constants.ANG2BOHR * 0.1).astype(np.float32))
    d2 = tmp_path / "every"
    d2.mkdir()
    Run._write_hdf5(run, d2, OUT, rows, steps_t, True)
    with fake_h5py.File(d2 / "trajectory.h5", "r") as f:
        assert np.array_equal(f["time"][:], steps_t[1:] * constants.AUTIME2PS)
    for out in ({**OUT, "hdf5_output": {"enabled": False, "file_name": "x.h5"}},
                {**OUT, "unwrapped_traj": {"file_name": "u.npy", "write": 0}},
                {k: v for k, v in OUT.items() if k != "hdf5_output"}):
        d = Path(tempfile.mkdtemp(dir=tmp_path))
        Run._write_hdf5(run, d, out, rows, steps_t, False)
        assert not any(d.iterdir())
    d3 = tmp_path / "bad"
    d3.mkdir()
    Run._write_hdf5(run, d3, OUT, np.zeros((5, 5)), steps_t, False)
    assert "Warning: Failed to write HDF5 trajectory data" in capsys.readouterr().out


def test_run_hdf5_without_h5py_is_skipped(monkeypatch, tmp_path):
    """Without h5py the output is left out silently (PyCD/core.py:29-32)."""
    monkeypatch.setitem(sys.modules, "h5py", None)  # import h5py raises ImportError
    monkeypatch.delitem(sys.modules, "pycd_gb300.hdf5_io", raising=False)
    Run._write_hdf5(_run_like(), tmp_path, OUT, np.zeros((3, 3)), np.zeros(4), False)
    assert not any(tmp_path.iterdir())
    with pytest.raises(ImportError):
        importlib.import_module("pycd_gb300.hdf5_io")


def test_with_real_h5py(tmp_path):
    """With h5py installed: the same file through the real library."""
    real = pytest.importorskip("h5py")
    if real is fake_h5py:
        pytest.skip("stand-in in place")
    from pycd_gb300 import hdf5_io
    rows = np.random.default_rng(5).random((4, 6))
    hdf5_io.save_trajectory_hdf5(tmp_path / "r.h5", rows, np.arange(4.0), n_atoms=2)
    with real.File(tmp_path / "r.h5", "r") as f:
        assert f["coordinates"].shape == (4, 2, 3) and f["time"].shape == (4,)
        assert np.array_equal(f["coordinates"][:].reshape(4, 6),
                              (rows / constants.ANG2BOHR * 0.1).astype(np.float32))
