"""HDF5 trajectory file of Run.do_kmc_steps' optional ``hdf5_output``
(PyCD/hdf5_io.py:19-226, used at PyCD/core.py:2677-2691 and 2882-2902), in
the MDTraj layout the reference writes:

  /coordinates                float32 (frames, n_atoms, 3), nanometres
  /time                       float64 (frames,), picoseconds
  /topology/atoms/name        'ATOM<i>' as S10
  /topology/atoms/element     'C' as S2
  /topology/atoms/index       int32

``coordinates`` and ``time`` grow along frames (chunked, gzip) and carry a
``units`` attribute.  Coordinates are given in bohr and times in atomic
units, converted as the reference converts them: x / ANG2BOHR * 0.1 and
t * AUTIME2PS.

This module needs h5py: importing it raises ImportError without h5py, and
Run.do_kmc_steps then leaves the HDF5 output out, as the reference does
(PyCD/core.py:29-32).

Two differences from the reference's writer, both where it fails:
* ``append=True`` on an existing file continues its datasets (the
  reference's writer opens the file but never binds them, so its next write
  raises AttributeError);
* ``write_frames`` checks that there is one time per frame before writing
  (the reference writes the coordinates, then h5py refuses the time values
  and /time stays zero-filled).
"""
from pathlib import Path

import h5py
import numpy as np

from . import constants


def _nm(coords_bohr):
    return coords_bohr / constants.ANG2BOHR * 0.1


def _ps(time_au):
    return time_au * constants.AUTIME2PS


class HDF5TrajectoryWriter(object):
    """Frames of one trajectory in the layout above (PyCD/hdf5_io.py:19-184)."""

    def __init__(self, filename, n_atoms, n_species, append=False):
        self.filename = Path(filename)
        self.n_atoms = int(n_atoms)
        self.n_species = int(n_species)
        self.append = append
        reopen = bool(append) and self.filename.exists()
        self.h5file = h5py.File(self.filename, "a" if reopen else "w")
        if reopen:
            self.coords_dset = self.h5file["coordinates"]
            self.time_dset = self.h5file["time"]
            self._frame_count = int(self.coords_dset.shape[0])
        else:
            self._write_topology()
            self._create_frame_datasets()
            self._frame_count = 0

    def _write_topology(self):
        if "topology" in self.h5file:
            del self.h5file["topology"]
        atoms = self.h5file.create_group("topology").create_group("atoms")
        n = self.n_atoms
        atoms.create_dataset("name", data=np.array(["ATOM%d" % i for i in range(n)],
                                                   dtype="S10"))
        atoms.create_dataset("element", data=np.array(["C"] * n, dtype="S2"))
        atoms.create_dataset("index", data=np.arange(n, dtype=np.int32))

    def _create_frame_datasets(self):
        n = self.n_atoms
        self.coords_dset = self.h5file.create_dataset(
            "coordinates", shape=(0, n, 3), maxshape=(None, n, 3), dtype=np.float32,
            chunks=True, compression="gzip")
        self.coords_dset.attrs["units"] = "nanometers"
        self.time_dset = self.h5file.create_dataset(
            "time", shape=(0,), maxshape=(None,), dtype=np.float64, chunks=True,
            compression="gzip")
        self.time_dset.attrs["units"] = "picoseconds"

    def _grow(self, n_frames):
        start = self._frame_count
        end = start + n_frames
        self.coords_dset.resize((end, self.n_atoms, 3))
        self.time_dset.resize((end,))
        self._frame_count = end
        return start, end

    def write_frame(self, coordinates, time_value):
        """One frame: coordinates (n_atoms, 3) or (3 n_atoms,) in bohr, its
        time in atomic units."""
        coords = np.asarray(coordinates)
        if coords.ndim == 1:
            coords = coords.reshape(-1, 3)
        start, _ = self._grow(1)
        self.coords_dset[start] = _nm(coords)
        self.time_dset[start] = _ps(time_value)

    def write_frames(self, coordinates_array, time_array):
        """Frames: coordinates (frames, n_atoms, 3) or (frames, 3 n_atoms)
        in bohr and one time per frame in atomic units."""
        coords = np.asarray(coordinates_array)
        times = np.asarray(time_array)
        if coords.ndim == 2 and coords.shape[1] == 3 * self.n_atoms:
            coords = coords.reshape(coords.shape[0], self.n_atoms, 3)
        n = coords.shape[0]
        if times.shape != (n,):
            raise ValueError("write_frames: %d frames but time values of shape %s"
                             % (n, times.shape))
        start, end = self._grow(n)
        self.coords_dset[start:end] = _nm(coords)
        self.time_dset[start:end] = _ps(times)

    def close(self):
        if getattr(self, "h5file", None):
            self.h5file.close()

    def __enter__(self):
        return self

    def __exit__(self, exc_type, exc_val, exc_tb):
        self.close()


def save_trajectory_hdf5(filename, coordinates, time_data=None, n_atoms=None):
    """Write coordinates (bohr) and times (atomic units; 0, 1, ... when not
    given) as one file (PyCD/hdf5_io.py:187-226).  A 1-D array is one frame
    of n / 3 atoms; a 2-D array (frames, 3 n_atoms) or (frames, n_atoms);
    a 3-D array (frames, n_atoms, 3)."""
    coords = np.asarray(coordinates)
    if n_atoms is None:
        if coords.ndim == 1:
            n_atoms = len(coords) // 3
        elif coords.ndim == 2:
            n_atoms = coords.shape[1] // 3 if coords.shape[1] % 3 == 0 else coords.shape[1]
        elif coords.ndim == 3:
            n_atoms = coords.shape[1]
        else:
            raise ValueError("Cannot infer n_atoms from coordinate shape")
    if time_data is None:
        time_data = (np.array([0.0]) if coords.ndim == 1
                     else np.arange(coords.shape[0], dtype=float))
    with HDF5TrajectoryWriter(filename, n_atoms, 1) as writer:
        if coords.ndim == 1:
            writer.write_frame(coords, time_data[0])
        else:
            writer.write_frames(coords, time_data)
