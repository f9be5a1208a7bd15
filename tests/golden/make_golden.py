"""Generate the golden fixtures under tests/golden/ from the reference PyCD.

Run where a checkout of the reference exists, with $PYCD_REFERENCE naming
its root directory (the one holding PyCD/ and examples/):

    PYCD_REFERENCE=<reference checkout> python tests/golden/make_golden.py [parts]

The reference is imported with test-only shims (stub matplotlib / yaml
modules, ``np.in1d = np.isin``, a ragged-list ``asarray`` for multi-element
POSCARs) and driven through its own classes.  Every fixture written here was
produced by the reference's code or ships with it:

  hematite.json/.npz, bvo.json/.npz
      examples/{Hematite,BVO}: shipped precomputed_array.npy and pmiv (the
      array is rebuilt by the reference's pot_r_ewald/pot_k_ewald and checked
      against the shipped one), the shipped hop-neighbour list, the shipped
      initial MT19937 state, and the shipped unwrapped_traj.npy /
      time_data.npy (re-run here through do_kmc_steps and checked).
  corundum324.json/.npz
      the 324-site corundum lattice (3x3x3 cells of the 12-site Fe sublattice
      of examples/Hematite): the reference's own hop-neighbour list, pmiv
      digest and Ewald array rows, and its event stream for 1e5 steps driven
      by injected uniforms np.random.default_rng(0).random(2e5).
  corundum3600.json/.npz
      the 3,600-site lattice (10x10x3 cells) with 4 electrons and 4 fixed +1
      dopants: digests of the reference's own hop-neighbour list and pmiv,
      rows of its own FP64 Ewald array (the carrier and dopant sites), and
      its event stream for a 2,000-step prefix of two trajectories run on
      that array.
  ewald_params.json/.npz
      get_ewald_parameters of the reference on the Hematite example lattice:
      automatic r_cut, automatic r_cut and k_cut, automatic alpha (2x2x1,
      shipped pmiv) and the 'converge' k_cut scan of the unit cell (its pmiv
      from the reference): the choices, the report lines after the timing
      lines, and the k_cut convergence / k-vector contribution logs.
  kvector_data.json
      get_precomputed_array(dst, 0, 1) of the reference on the Hematite
      example (2x2x1, shipped pmiv, its own alpha / r_cut / k_cut): the
      k_vector_energy_contribution_within_user_specified_k_cut.log it writes
      (every half-space k-vector of the k_max box, sorted by decreasing
      energy contribution, zero outside k_cut) and the k_max / k-vector
      count lines of precomputed_array.log.
  hdf5.json/.npz
      the reference's HDF5TrajectoryWriter (PyCD/hdf5_io.py) and its use in
      do_kmc_steps, run against the h5py stand-in tests/fake_h5py.py (h5py is
      not installed here): write_frame + write_frames and
      save_trajectory_hdf5 of 2-D and 1-D arrays on seeded coordinates, and
      the file do_kmc_steps writes for examples/Hematite's first ~2,000
      steps with hdf5_output enabled, per step (write_every_step = 1) and
      on the time grid (its coordinates, its warning and its /time).
  msd.json/.npz
      Analysis.compute_msd of the reference on the shipped Hematite
      trajectory (examples/Hematite/traj1, with the example's MSD parameters)
      and on three synthetic random-walk trajectories with three species
      types, one of them empty: MSD table, SEM table and report lines.
"""
import hashlib
import json
import os
import pickle
import shutil
import sys
import tempfile
import time
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
sys.path[:0] = [str(HERE.parent), str(REPO)]
from golden_io import hop_digest, hop_to_arrays  # noqa: E402  (same canonical form as the tests)
REF = Path(os.environ["PYCD_REFERENCE"]) if os.environ.get("PYCD_REFERENCE") else None


# ---------------------------------------------------------------- shims
def install_shims():
    for name in ("matplotlib", "matplotlib.pyplot", "matplotlib.offsetbox", "yaml"):
        sys.modules.setdefault(name, types.ModuleType(name))
    sys.modules["matplotlib"].pyplot = sys.modules["matplotlib.pyplot"]
    sys.modules["matplotlib.pyplot"].switch_backend = lambda *a, **k: None
    sys.modules["matplotlib.offsetbox"].AnchoredText = object
    if not hasattr(np, "in1d"):
        np.in1d = np.isin
    sys.path.insert(0, str(REF))
    import PyCD.core as core

    class _NumpyProxy:
        def __getattr__(self, name):
            return getattr(np, name)

        @staticmethod
        def asarray(x, *a, **k):
            try:
                return np.asarray(x, *a, **k)
            except ValueError:
                out = np.empty(len(x), dtype=object)
                for i, row in enumerate(x):
                    out[i] = np.asarray(row)
                return out

    core.np = _NumpyProxy()
    return core


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


# ---------------------------------------------------------------- configs
PRECISION = dict(lower_bound_real=0.75, lower_bound_rcut=0.0, upper_bound_rcut=0.9999,
                 lower_bound_kcut=0.0, upper_bound_kcut=10.0, threshold_fraction=0.9,
                 precise_r_cut=0, err_tol=2.585e-3, step_increase_tol=2.585e-10,
                 num_data_points_low=10.0, num_data_points_high=50.0,
                 step_change_data_points=10.0)

HEMATITE = dict(
    name="Fe2O3", species_types=["electron", "hole"],
    species_charge_list={"full": [-1, 1], "partial": [-0.5, 0.5]},
    species_to_element_type_map={"electron": ["Fe"], "hole": ["O"]},
    charge_types={"full": {"Fe": 3.0, "O": -2.0},
                  "partial": {"Fe": 1.6349, "O": -1.0899}},
    neighbor_cutoff_dist={"Fe:Fe": [[2.971, 2.901]]},
    neighbor_cutoff_dist_tol={"Fe:Fe": [[0.0020, 0.0020]]},
    vn=1.85e13, lambda_values={"Fe:Fe": [[1.74533, 1.88683]]},
    v_ab={"Fe:Fe": [[0.184, 0.028]]},
    class_list={"Fe": [1] * 12, "O": [1] * 18}, element_type_delimiter=":",
    dielectric_constant=9.355, alpha=2.667e-01, r_cut=4.618e+00, k_cut=6.998e+00,
    precision_parameters=PRECISION)

BVO = dict(
    name="BVO", species_types=["electron", "hole"],
    species_charge_list={"full": [-1, 1], "partial": [-0.5, 0.5]},
    species_to_element_type_map={"electron": ["V"], "hole": ["O"]},
    charge_types={"full": {"Bi": 3.0, "O": -2.0, "V": 5.0},
                  "partial": {"Bi": 2.0311, "O": -1.0352, "V": 2.1098}},
    neighbor_cutoff_dist={
        "V:V": [[3.8474, 3.9447, 5.0935, 5.1956]],
        "O:O": [[2.7450, 2.8541, 2.8600, 2.9573, 2.9723, 3.0033, 3.0076, 3.0205,
                 3.0473, 3.6123, 3.6845],
                [2.7962, 2.8541, 2.8600, 2.9123, 2.9707, 2.9678, 3.0076, 3.0205,
                 2.9958, 3.6123, 3.6845]]},
    neighbor_cutoff_dist_tol={
        "V:V": [[0.0020] * 4],
        "O:O": [[0.0020, 0.0020, 0.0020, 0.0020, 0.0010, 0.0020, 0.0020, 0.0020,
                 0.0020, 0.0020, 0.0020]] * 2},
    vn=1.00e13,
    lambda_values={"V:V": [[1.4768, 1.4964, 1.4652, 1.4932]],
                   "O:O": [[1.4668, 0.7552, 0.7552, 1.6419, 0.9952, 1.5667, 1.4887,
                            1.4887, 2.3456, 1.4863, 1.4863]] * 2},
    v_ab={"V:V": [[0.0] * 4], "O:O": [[0.0] * 11] * 2},
    class_list={"O": [2, 1] * 8, "V": [1] * 4, "Bi": [1] * 4},
    element_type_delimiter=":", dielectric_constant=38.299,
    alpha=2.051e-01, r_cut=4.669e+00, k_cut=5.298e+00,
    precision_parameters=dict(PRECISION, upper_bound_kcut=100.0,
                              step_increase_tol=2.585e-07))

RUN_COMMON = dict(
    temp=300, ion_charge_type="full", species_charge_type="full",
    species_count=[1, 0], time_interval=1.0e-08,
    initial_occupancy={"electron": [], "hole": []},
    relative_energies={"class_index": {"O": [0.0, 0.0406]},
                       "doping": {"V": [[0.6596, -0.0168, -0.0154],
                                        [0.0791, -0.0024, -0.0188]]}},
    external_field={"electric": {"active": 0, "dir": [1, 0, 0], "ld": 0, "mag": 0.0001}},
    doping={"num_dopants": [0, 0], "doping_element_map": ["V:W", "V:Mo"],
            "insertion_type": ["random", "random"], "charge": {"full": {"Mo": 5, "W": 5}},
            "site_charge_initiation": ["no", "no"], "min_shell_separation": [4, 4],
            "max_attempts": 100},
    output_data={
        "delg_0": {"file_name": "delG0_traj.npy", "write": 0},
        "energy": {"file_name": "energy_traj.npy", "write": 0},
        "potential": {"file_name": "potential_traj.npy", "write": 0},
        "time": {"file_name": "time_data.npy", "write": 1},
        "unwrapped_traj": {"file_name": "unwrapped_traj.npy", "write": 1,
                           "write_every_step": 0},
        "wrapped_traj": {"file_name": "wrapped_traj.npy", "write": 0}},
    random_seed=2)

# synthetic corundum (Fe sublattice of hematite, R-centred 12c sites)
CORUNDUM_LATTICE = [[5.038, 0.0, 0.0], [-2.519, 4.363036, 0.0], [0.0, 0.0, 13.772]]


def corundum_frac(z=0.3553):
    base = [(0, 0, z), (0, 0, -z), (0, 0, 0.5 + z), (0, 0, 0.5 - z)]
    cent = [(0, 0, 0), (2 / 3, 1 / 3, 1 / 3), (1 / 3, 2 / 3, 2 / 3)]
    out = []
    for c in cent:
        for b in base:
            out.append([(b[i] + c[i]) % 1.0 for i in range(3)])
    return np.array(out)


CORUNDUM = dict(
    name="corundum", species_types=["electron"],
    species_charge_list={"full": [-1]},
    species_to_element_type_map={"electron": ["Fe"]},
    charge_types={"full": {"Fe": 0.0}},
    neighbor_cutoff_dist={"Fe:Fe": [[2.90, 2.97]]},
    neighbor_cutoff_dist_tol={"Fe:Fe": [[0.01, 0.01]]},
    vn=1.85e13, lambda_values={"Fe:Fe": [[0.9, 0.9]]}, v_ab={"Fe:Fe": [[0.2, 0.2]]},
    class_list={"Fe": [1] * 12}, element_type_delimiter=":",
    dielectric_constant=12.0, alpha=0.25, r_cut=6.4, k_cut=1.6,
    precision_parameters=PRECISION)


def poscar_text(comment, lattice, types_, counts, frac):
    out = [comment, "1.0"]
    for row in lattice:
        out.append("  ".join(f"{v:20.10f}" for v in row))
    out.append("   ".join(types_))
    out.append("   ".join(str(c) for c in counts))
    out.append("Direct")
    for row in frac:
        out.append("  ".join(f"{v:18.12f}" for v in row))
    return "\n".join(out) + "\n"


# ---------------------------------------------------------------- helpers
def material_objects(core, params, poscar, system_size, pbc, tmp):
    p = dict(params)
    p.pop("precision_parameters", None)
    path = Path(tmp) / "POSCAR"
    path.write_text(poscar)
    p["input_coord_file_location"] = path
    mat = core.Material(core.ReturnValues(**p))
    nb = core.Neighbors(mat, np.asarray(system_size), np.asarray(pbc))
    return mat, nb


def make_system(core, mat, nb, hop, pmiv, params):
    return core.System(mat, nb, hop, pmiv, params["alpha"], params["r_cut"],
                       params["k_cut"], params["precision_parameters"], [], [])


def ref_array(system, mat, nb):
    Ar = system.get_precomputed_array_real(system.alpha, system.r_cut)
    Af, _, _ = system.get_precomputed_array_fourier(system.alpha, system.k_cut)
    As = -np.eye(nb.num_system_elements) * np.sqrt(system.alpha / np.pi) \
        / mat.dielectric_constant
    return Ar + Af + As


# ---------------------------------------------------------------- examples
def example(core, name, params, t_final):
    ex = REF / "examples" / name
    poscar = (ex / "InputFiles" / "POSCAR").read_text()
    tmp = tempfile.mkdtemp()
    mat, nb = material_objects(core, params, poscar, [2, 2, 1], [1, 1, 1], tmp)
    hop = np.load(ex / "InputFiles" / "hop_neighbor_list.npy", allow_pickle=True)[()]
    pmiv = np.load(ex / "InputFiles" / "pairwise_min_image_vector_data.npy")
    A_shipped = np.load(ex / "InputFiles" / "precomputed_array.npy")
    system = make_system(core, mat, nb, hop, pmiv, params)
    A = ref_array(system, mat, nb)
    err = float(np.abs(A - A_shipped).max())
    print(f"{name}: reference rebuild vs shipped array max |dA| = {err:.3e} Ha")
    assert err < 1e-15
    run_p = dict(RUN_COMMON, t_final=t_final)
    run = core.Run(system, A_shipped, run_p["temp"], run_p["ion_charge_type"],
                   run_p["species_charge_type"], 1, t_final, run_p["time_interval"],
                   np.asarray(run_p["species_count"]), run_p["initial_occupancy"],
                   run_p["relative_energies"], run_p["external_field"], run_p["doping"])
    d = Path(tempfile.mkdtemp())
    shutil.copy(ex / "traj1" / "initial_rnd_state.dump", d / "initial_rnd_state.dump")
    t0 = time.time()
    run.do_kmc_steps(d, run_p["output_data"], run_p["random_seed"], "parallel")
    dt = time.time() - t0
    u_ship = np.load(ex / "traj1" / "unwrapped_traj.npy")
    t_ship = np.load(ex / "traj1" / "time_data.npy")
    u_ref = np.load(d / "unwrapped_traj.npy")
    t_ref = np.load(d / "time_data.npy")
    assert np.array_equal(u_ref, u_ship)
    rel = float(np.abs(t_ref[1:] / t_ship[1:] - 1).max())
    print(f"{name}: re-run {len(t_ref) - 1} steps in {dt:.1f} s, unwrapped "
          f"bit-identical, time max rel {rel:.2e}")
    with open(ex / "traj1" / "initial_rnd_state.dump", "rb") as fh:
        state = pickle.load(fh)
    meta, arrs = hop_to_arrays(hop)
    stride_u = 1 if len(u_ship) <= 20001 else 10
    stride_t = 1 if len(t_ship) <= 40001 else 16
    cfg = {"name": name, "params": params, "poscar": poscar, "system_size": [2, 2, 1],
           "pbc": [1, 1, 1], "run": run_p, "hop_meta": meta,
           "rnd_state": [state[0], list(state[1]), state[2]],
           "n_steps": int(len(t_ship) - 1), "unwrapped_stride": stride_u,
           "time_stride": stride_t, "unwrapped_sha256": sha(u_ship),
           "reference_seconds": dt,
           "array_rebuild_max_abs_ha": err}
    np.savez_compressed(HERE / f"{name.lower()}.npz", A=A_shipped, pmiv=pmiv,
                        unwrapped=u_ship[::stride_u], time=t_ship[::stride_t],
                        time_last=t_ship[-1:], **arrs)
    (HERE / f"{name.lower()}.json").write_text(json.dumps(cfg, indent=1))


def every_step(core):
    """examples/Hematite for its first ~2,000 steps with write_every_step = 1:
    the reference's per-step unwrapped rows (core.py:2832-2846) and times,
    from the shipped traj1 random state."""
    import copy
    name, params, t_final = "Hematite", HEMATITE, 6e-7
    ex = REF / "examples" / name
    poscar = (ex / "InputFiles" / "POSCAR").read_text()
    tmp = tempfile.mkdtemp()
    mat, nb = material_objects(core, params, poscar, [2, 2, 1], [1, 1, 1], tmp)
    hop = np.load(ex / "InputFiles" / "hop_neighbor_list.npy", allow_pickle=True)[()]
    pmiv = np.load(ex / "InputFiles" / "pairwise_min_image_vector_data.npy")
    A_shipped = np.load(ex / "InputFiles" / "precomputed_array.npy")
    system = make_system(core, mat, nb, hop, pmiv, params)
    run_p = copy.deepcopy(dict(RUN_COMMON, t_final=t_final))
    run_p["output_data"]["unwrapped_traj"]["write_every_step"] = 1
    run = core.Run(system, A_shipped, run_p["temp"], run_p["ion_charge_type"],
                   run_p["species_charge_type"], 1, t_final, run_p["time_interval"],
                   np.asarray(run_p["species_count"]), run_p["initial_occupancy"],
                   run_p["relative_energies"], run_p["external_field"], run_p["doping"])
    d = Path(tempfile.mkdtemp())
    shutil.copy(ex / "traj1" / "initial_rnd_state.dump", d / "initial_rnd_state.dump")
    run.do_kmc_steps(d, run_p["output_data"], run_p["random_seed"], "parallel")
    u = np.load(d / "unwrapped_traj.npy")
    t = np.load(d / "time_data.npy")
    print(f"{name} every step: {len(t) - 1} steps, {len(u)} rows")
    np.savez_compressed(HERE / "hematite_every_step.npz", unwrapped=u, time=t)
    cfg = {"t_final": t_final, "n_steps": int(len(t) - 1), "rows": int(len(u)),
           "output_data": run_p["output_data"], "unwrapped_sha256": sha(u)}
    (HERE / "hematite_every_step.json").write_text(json.dumps(cfg, indent=1))


def hematite_outputs(core):
    """examples/Hematite for its first ~2,000 steps with the energy and dG0
    path grids written (core.py:2806-2808, 2848-2861, 2863-2906), from the
    shipped traj1 random state."""
    import copy
    name, params, t_final = "Hematite", HEMATITE, 6e-7
    ex = REF / "examples" / name
    poscar = (ex / "InputFiles" / "POSCAR").read_text()
    tmp = tempfile.mkdtemp()
    mat, nb = material_objects(core, params, poscar, [2, 2, 1], [1, 1, 1], tmp)
    hop = np.load(ex / "InputFiles" / "hop_neighbor_list.npy", allow_pickle=True)[()]
    pmiv = np.load(ex / "InputFiles" / "pairwise_min_image_vector_data.npy")
    A_shipped = np.load(ex / "InputFiles" / "precomputed_array.npy")
    system = make_system(core, mat, nb, hop, pmiv, params)
    run_p = copy.deepcopy(dict(RUN_COMMON, t_final=t_final))
    run_p["output_data"]["energy"]["write"] = 1
    run_p["output_data"]["delg_0"]["write"] = 1
    run = core.Run(system, A_shipped, run_p["temp"], run_p["ion_charge_type"],
                   run_p["species_charge_type"], 1, t_final, run_p["time_interval"],
                   np.asarray(run_p["species_count"]), run_p["initial_occupancy"],
                   run_p["relative_energies"], run_p["external_field"], run_p["doping"])
    d = Path(tempfile.mkdtemp())
    shutil.copy(ex / "traj1" / "initial_rnd_state.dump", d / "initial_rnd_state.dump")
    run.do_kmc_steps(d, run_p["output_data"], run_p["random_seed"], "parallel")
    out = {k: np.load(d / run_p["output_data"][k]["file_name"])
           for k in ("unwrapped_traj", "time", "energy", "delg_0")}
    print(f"{name} outputs: {len(out['time']) - 1} steps, energy rows {len(out['energy'])}")
    np.savez_compressed(HERE / "hematite_outputs.npz", **out)
    cfg = {"t_final": t_final, "n_steps": int(len(out["time"]) - 1),
           "output_data": run_p["output_data"]}
    (HERE / "hematite_outputs.json").write_text(json.dumps(cfg, indent=1))


BVO_DOPING = {"num_dopants": [2, 0], "doping_element_map": ["V:W", "V:Mo"],
              "insertion_type": ["manual", "manual"],
              "charge": {"full": {"W": 6.0, "Mo": 6.0}},
              "site_charge_initiation": ["yes", "no"], "min_shell_separation": [0, 0],
              "max_attempts": 1}


def bvo_doped(core):
    """examples/BVO with two W dopants (charge 6 on V sites) from a manual
    site_indices.npy with shell-indexed site energies (shells 0, 1, 2), the
    electron starting on a dopant site (site_charge_initiation 'yes', drawn
    by rnd.sample from the shipped traj1 random state).  The reference's
    do_kmc_steps: unwrapped rows, times, occupancy list and its doped site
    energies (core.py:2723-2772, 2478-2528)."""
    import copy
    name, params, t_final = "BVO", BVO, 4e-5
    ex = REF / "examples" / name
    poscar = (ex / "InputFiles" / "POSCAR").read_text()
    tmp = tempfile.mkdtemp()
    mat, nb = material_objects(core, params, poscar, [2, 2, 1], [1, 1, 1], tmp)
    hop = np.load(ex / "InputFiles" / "hop_neighbor_list.npy", allow_pickle=True)[()]
    pmiv = np.load(ex / "InputFiles" / "pairwise_min_image_vector_data.npy")
    A_shipped = np.load(ex / "InputFiles" / "precomputed_array.npy")
    system = make_system(core, mat, nb, hop, pmiv, params)
    # V sites: the hop neighbours of the V:V list; two dopants and a few shells
    v_sites = sorted({int(i) for obj in hop["V:V"][0]
                      for row in obj.neighbor_system_element_indices for i in row})
    d1, d2 = v_sites[1], v_sites[6]
    near = [i for i in v_sites if i not in (d1, d2)]
    site_indices = np.array([[d1, 0, 0, 0], [d2, 0, 0, 0],
                             [near[0], 0, 0, 1], [near[2], 0, 0, 1],
                             [near[4], 0, 0, 2], [near[7], 0, 0, 2]], dtype=int)
    run_p = copy.deepcopy(dict(RUN_COMMON, t_final=t_final, doping=BVO_DOPING))
    run = core.Run(system, A_shipped, run_p["temp"], run_p["ion_charge_type"],
                   run_p["species_charge_type"], 1, t_final, run_p["time_interval"],
                   np.asarray(run_p["species_count"]), run_p["initial_occupancy"],
                   run_p["relative_energies"], run_p["external_field"], run_p["doping"])
    d = Path(tempfile.mkdtemp())
    shutil.copy(ex / "traj1" / "initial_rnd_state.dump", d / "initial_rnd_state.dump")
    np.save(d / "site_indices.npy", site_indices)
    run.do_kmc_steps(d, run_p["output_data"], run_p["random_seed"], "parallel")
    u = np.load(d / "unwrapped_traj.npy")
    t = np.load(d / "time_data.npy")
    occ = np.load(d / "occupancy.npy")
    print(f"{name} doped: {len(t) - 1} steps, first site {occ[0].tolist()}, "
          f"dopants {d1}, {d2}")
    np.savez_compressed(HERE / "bvo_doped.npz", unwrapped=u, time=t, occupancy=occ,
                        site_indices=site_indices,
                        system_relative_energies=np.asarray(run.system_relative_energies))
    cfg = {"t_final": t_final, "n_steps": int(len(t) - 1), "doping": run_p["doping"],
           "output_data": run_p["output_data"], "unwrapped_sha256": sha(u)}
    (HERE / "bvo_doped.json").write_text(json.dumps(cfg, indent=1))


# ---------------------------------------------------------------- injected run
class Injected:
    """random-module stand-in: random() pops injected uniforms, sample()
    delegates (only used when no initial occupancy is given)."""

    def __init__(self, u):
        self.u, self.i = u, 0

    def random(self):
        if self.i >= len(self.u):
            raise StopIteration
        v = self.u[self.i]
        self.i += 1
        return float(v)

    def sample(self, *a):
        raise RuntimeError("sample() not expected")


def injected_run(core, run, A, occ, uniforms, n_steps_expected):
    """Run do_kmc_steps' loop with injected uniforms; returns (proc, time)
    reconstructed from the recorded rates with the reference's expressions."""
    rec_rates = []
    orig_rates = core.Run.get_process_rates

    def rates(self, attrs, q):
        r = orig_rates(self, attrs, q)
        rec_rates.append(r[0].copy())
        return r

    saved_rnd = core.rnd
    core.rnd = Injected(uniforms)
    core.Run.get_process_rates = rates
    d = Path(tempfile.mkdtemp())
    pickle.dump(saved_rnd.getstate(), open(d / "initial_rnd_state.dump", "wb"))
    core.rnd.setstate = lambda s: None
    try:
        run.initial_occupancy = {"electron": list(occ)}
        out = {k: dict(v) for k, v in RUN_COMMON["output_data"].items()}
        run.do_kmc_steps(d, out, 0, "parallel")
    except StopIteration:
        pass
    finally:
        core.rnd = saved_rnd
        core.Run.get_process_rates = orig_rates
    # rates recorded for the step that ran out of uniforms are dropped
    n = min(len(rec_rates), len(uniforms) // 2)
    procs, times = [], [0.0]
    t = 0
    for i in range(n):
        k = rec_rates[i]
        k_total = sum(k)
        cum = (k / k_total).cumsum()
        procs.append(int(np.where(cum > uniforms[2 * i])[0][0]))
        t -= np.log(uniforms[2 * i + 1]) / k_total
        times.append(t)
    assert n == n_steps_expected, (n, n_steps_expected)
    return np.asarray(procs, np.uint8), np.asarray(times)


def corundum324(core):
    frac = corundum_frac()
    poscar = poscar_text("corundum Fe sublattice", CORUNDUM_LATTICE, ["Fe"], [12], frac)
    tmp = tempfile.mkdtemp()
    mat, nb = material_objects(core, CORUNDUM, poscar, [3, 3, 3], [1, 1, 1], tmp)
    t0 = time.time()
    nb.generate_neighbor_list(Path(tmp), np.array([3, 3, 3]))
    hop = np.load(Path(tmp) / "hop_neighbor_list.npy", allow_pickle=True)[()]
    nb.get_pairwise_min_image_vector_data(Path(tmp))
    pmiv = np.load(Path(tmp) / "pairwise_min_image_vector_data.npy")
    print(f"corundum324: reference neighbour list + pmiv in {time.time() - t0:.1f} s")
    system = make_system(core, mat, nb, hop, pmiv, CORUNDUM)
    t0 = time.time()
    A = ref_array(system, mat, nb)
    t_ewald = time.time() - t0
    site = int(np.random.default_rng(0).integers(324))
    U = np.random.default_rng(0).random(200000)
    run = core.Run(system, A, 300, "full", "full", 1, 1e-6, 1e-9, np.array([1]),
                   {"electron": [site]}, {"class_index": {}, "doping": {}},
                   RUN_COMMON["external_field"], {"num_dopants": [0]})
    t0 = time.time()
    procs, times = injected_run(core, run, A, [site], U, 100000)
    t_kmc = time.time() - t0
    print(f"corundum324: Ewald {t_ewald:.2f} s, 1e5 KMC steps {t_kmc:.1f} s")
    meta, arrs = hop_to_arrays(hop)
    rows = np.array([0, 1, 161, 323])
    cfg = {"name": "corundum324", "params": CORUNDUM, "poscar": poscar,
           "system_size": [3, 3, 3], "pbc": [1, 1, 1], "hop_meta": meta,
           "carrier_site": site, "uniform_seed": 0, "n_steps": 100000,
           "t_final": 1e-6, "time_interval": 1e-9, "A_sha256": sha(A),
           "pmiv_sha256": sha(pmiv), "A_rows": rows.tolist(),
           "reference_ewald_seconds": t_ewald, "reference_kmc_seconds": t_kmc}
    np.savez_compressed(HERE / "corundum324.npz", A_rows=A[rows], A_diag=np.diag(A),
                        proc=procs, time=times[::8], time_last=times[-1:], **arrs)
    (HERE / "corundum324.json").write_text(json.dumps(cfg, indent=1))
    return mat


def corundum3600(core):
    sys.path.insert(0, str(REPO))
    from oracle import ewald_oracle as eo
    frac = corundum_frac()
    poscar = poscar_text("corundum Fe sublattice", CORUNDUM_LATTICE, ["Fe"], [12], frac)
    tmp = tempfile.mkdtemp()
    params = dict(CORUNDUM)
    mat, nb = material_objects(core, params, poscar, [10, 10, 3], [1, 1, 1], tmp)
    t0 = time.time()
    nb.generate_neighbor_list(Path(tmp), np.array([3, 3, 3]))
    hop = np.load(Path(tmp) / "hop_neighbor_list.npy", allow_pickle=True)[()]
    nb.get_pairwise_min_image_vector_data(Path(tmp))
    pmiv = np.load(Path(tmp) / "pairwise_min_image_vector_data.npy")
    t_nbr = time.time() - t0
    print(f"corundum3600: reference neighbour list + pmiv in {t_nbr:.1f} s")
    system = make_system(core, mat, nb, hop, pmiv, params)
    t0 = time.time()
    A = ref_array(system, mat, nb)
    t_ewald = time.time() - t0
    print(f"corundum3600: reference Ewald array in {t_ewald:.1f} s")
    rng = np.random.default_rng(3600)
    sites = rng.choice(3600, size=8, replace=False)
    carriers, dopants = sites[:4].tolist(), sites[4:].tolist()
    rows = np.array(carriers + dopants)
    # the oracle's translation-class evaluation against the reference's rows
    from pycd_gb300 import constants as K
    orc = eo.class_array(mat.cartesian_unit_cell_coords, mat.lattice_matrix, [10, 10, 3],
                         params["alpha"] / K.ANG2BOHR, params["r_cut"] * K.ANG2BOHR,
                         params["k_cut"] / K.ANG2BOHR, params["dielectric_constant"],
                         rows=rows)
    orc_err = float(np.abs(orc - A[rows]).max())
    print(f"corundum3600: oracle rows vs reference rows {orc_err:.3e} Ha")
    # dopants: lattice charge 0 overwritten by +1 (charge_config, core.py:2550-2554)
    doping = {"num_dopants": [4], "doping_element_map": ["Fe:D"],
              "insertion_type": ["manual"], "charge": {"full": {"D": 1.0}},
              "site_charge_initiation": ["no"], "min_shell_separation": [0],
              "max_attempts": 1}
    relE = {"class_index": {}, "doping": {"Fe": [[0.0]]}}
    procs_all, times_all = [], []
    for traj in range(2):
        # carriers trapped on +1 dopants have residence times of ~1e14 s, so
        # the time grid spans 1e30 s to keep the run going for 2,000 steps
        run = core.Run(system, A, 300, "full", "full", 1, 1e30, 1e27, np.array([4]),
                       {"electron": carriers}, relE, RUN_COMMON["external_field"], doping)
        U = np.random.default_rng(1000 + traj).random(4000)
        d = Path(tempfile.mkdtemp())
        # site_indices.npy: [site, dopant type, unused, shell]
        si = np.array([[s, 0, 0, 0] for s in dopants])
        rec = []
        orig = core.Run.get_process_rates

        def rates(self, attrs, q):
            r = orig(self, attrs, q)
            rec.append(r[0].copy())
            return r

        saved = core.rnd
        core.rnd = Injected(U)
        core.rnd.setstate = lambda s: None
        core.Run.get_process_rates = rates
        pickle.dump(saved.getstate(), open(d / "initial_rnd_state.dump", "wb"))
        np.save(d / "site_indices.npy", si)
        t0 = time.time()
        try:
            out = {k: dict(v) for k, v in RUN_COMMON["output_data"].items()}
            run.do_kmc_steps(d, out, 0, "parallel")
        except StopIteration:
            pass
        finally:
            core.rnd = saved
            core.Run.get_process_rates = orig
        print(f"corundum3600 traj {traj}: 2000 steps in {time.time() - t0:.1f} s")
        procs, times, t = [], [0.0], 0
        for i in range(2000):
            k = rec[i]
            kt = sum(k)
            procs.append(int(np.where((k / kt).cumsum() > U[2 * i])[0][0]))
            t -= np.log(U[2 * i + 1]) / kt
            times.append(t)
        procs_all.append(procs)
        times_all.append(times)
    cfg = {"name": "corundum3600", "params": params, "poscar": poscar,
           "system_size": [10, 10, 3], "pbc": [1, 1, 1], "carriers": carriers,
           "dopants": dopants, "dopant_charge": 1.0, "uniform_seeds": [1000, 1001],
           "n_steps": 2000, "t_final": 1e30, "time_interval": 1e27,
           "hop_sha256": hop_digest(hop), "pmiv_sha256": sha(pmiv),
           "A_diag": float(A[0, 0]), "A_diag_ptp": float(np.ptp(np.diag(A))),
           "oracle_rows_max_abs_ha": orc_err,
           "reference_neighbor_seconds": t_nbr, "reference_ewald_seconds": t_ewald}
    np.savez_compressed(HERE / "corundum3600.npz", proc=np.asarray(procs_all, np.uint8),
                        time=np.asarray(times_all), A_rows=A[rows])
    (HERE / "corundum3600.json").write_text(json.dumps(cfg, indent=1))


def _ref_msd(core, rows_per_traj, species_types, species_count, params):
    """Run the reference's Analysis.compute_msd on trajectory files written
    the way do_kmc_steps writes them (traj{i}/unwrapped_traj.npy)."""
    mat = types.SimpleNamespace(num_species_types=len(species_types),
                                species_types=list(species_types))
    with tempfile.TemporaryDirectory() as d:
        d = Path(d)
        for i, rows in enumerate(rows_per_traj):
            (d / f"traj{i + 1}").mkdir()
            np.save(d / f"traj{i + 1}" / "unwrapped_traj.npy", rows)
        an = core.Analysis(mat, params["n_dim"], np.asarray(species_count),
                           len(rows_per_traj), params["t_final"], params["time_interval"],
                           params["msd_t_final"], params["trim_length"], params["temp"],
                           params["repr_time"], params["repr_dist"])
        out = an.compute_msd(d, {"unwrapped_traj": {"file_name": "unwrapped_traj.npy"}})
        msd_file = d / ("MSD_Data_" + out.file_name + ".npy")
        saved = np.load(msd_file)
        report = (d / ("MSD_Analysis_" + out.file_name + ".log")).read_text()
    assert np.array_equal(saved, out.msd_data)
    prefix = report[:report.index("Time elapsed")]
    return out, prefix


def msd(core):
    """MSD fixtures: the shipped Hematite trajectory with the example's own
    MSD parameters (examples/Hematite/simulation_parameters.yml), and a
    synthetic 3-trajectory case with three species types, one of them empty."""
    hem_params = {"n_dim": 3, "t_final": 1e-4, "time_interval": 1e-8,
                  "msd_t_final": 5000.0, "trim_length": 50, "temp": 300,
                  "repr_time": "ns", "repr_dist": "angstrom"}
    hem_rows = np.load(REF / "examples" / "Hematite" / "traj1" / "unwrapped_traj.npy")
    hem, hem_prefix = _ref_msd(core, [hem_rows], ["electron", "hole"], [1, 0], hem_params)
    # synthetic: 2 electrons + 0 holes + 1 "ion" per trajectory, random walks
    # of bohr-sized hops, 301 rows per trajectory
    syn_params = {"n_dim": 3, "t_final": 3e-6, "time_interval": 1e-8,
                  "msd_t_final": 1000.0, "trim_length": 10, "temp": 450,
                  "repr_time": "ns", "repr_dist": "angstrom"}
    rng = np.random.default_rng(11)
    syn_rows = []
    for t in range(3):
        steps = rng.normal(0.0, 5.5, size=(301, 9))
        steps[0] = 0.0
        syn_rows.append(np.cumsum(steps, axis=0))
    syn, syn_prefix = _ref_msd(core, syn_rows, ["electron", "hole", "ion"], [2, 0, 1],
                               syn_params)
    np.savez_compressed(HERE / "msd.npz", hem_rows=hem_rows, hem_msd=hem.msd_data,
                        hem_sem=hem.sem_data, syn_rows=np.stack(syn_rows),
                        syn_msd=syn.msd_data, syn_sem=syn.sem_data)
    cfg = {"hematite": dict(hem_params, species_types=["electron", "hole"],
                            species_count=[1, 0], n_traj=1, file_name=hem.file_name,
                            out_species=hem.species_types, report_prefix=hem_prefix),
           "synthetic": dict(syn_params, species_types=["electron", "hole", "ion"],
                             species_count=[2, 0, 1], n_traj=3, file_name=syn.file_name,
                             out_species=syn.species_types, report_prefix=syn_prefix,
                             rows_seed=11)}
    (HERE / "msd.json").write_text(json.dumps(cfg, indent=1))
    print("msd:", hem.file_name, hem_prefix.strip().replace("\n", " | "))
    print("msd:", syn.file_name, syn_prefix.strip().replace("\n", " | "))


class _Anything(object):
    """Stand-in for the matplotlib objects the parameter search draws on."""

    def __getattr__(self, name):
        return _Anything()

    def __call__(self, *a, **k):
        return _Anything()


def _ref_ewald_parameters(core, mat, nb, hop, pmiv, params, tmp):
    """Run the reference's get_ewald_parameters; return the choice, the
    report lines after the two timing lines, and the files it wrote."""
    core.plt = _Anything()
    ticker = types.ModuleType("matplotlib.ticker")
    ticker.FormatStrFormatter = _Anything()
    sys.modules["matplotlib.ticker"] = ticker
    sys.modules["matplotlib"].ticker = ticker
    system = make_system(core, mat, nb, hop, pmiv, params)
    dst = Path(tmp) / "InputFiles"
    dst.mkdir(parents=True, exist_ok=True)
    out = {"exit": False}
    try:
        ewald, prefix, dst2 = system.get_ewald_parameters([], dst)
        out.update(alpha=float(ewald["alpha"]), r_cut=float(ewald["r_cut"]),
                   k_cut=float(ewald["k_cut"]), lines=prefix[2:],
                   dst_suffix=str(Path(dst2).relative_to(dst)))
    except SystemExit:
        out["exit"] = True
        out["report"] = (dst / "precomputed_array.log").read_text().split("Time elapsed")[0]
    files = {}
    for f in sorted(dst.rglob("*.log")):
        files[str(f.relative_to(dst))] = f.read_text().split("Time elapsed")[0]
    out["files"] = files
    return out


def ewald_params(core):
    """Ewald parameter selection fixtures: the reference's own
    get_ewald_parameters (core.py:1559-1592) on the Hematite example lattice,
    one case per scan kind.  Timing-dependent output (the tau/time ratios and
    the all-automatic alpha) is not recorded."""
    ex = REF / "examples" / "Hematite"
    poscar = (ex / "InputFiles" / "POSCAR").read_text()
    hop = np.load(ex / "InputFiles" / "hop_neighbor_list.npy", allow_pickle=True)[()]
    pmiv221 = np.load(ex / "InputFiles" / "pairwise_min_image_vector_data.npy")
    cases = {
        "rcut_optimal": ([2, 2, 1], dict(alpha=0.6, r_cut="optimal", k_cut=6.998)),
        "rcut_kcut_optimal": ([2, 2, 1], dict(alpha=0.6, r_cut="optimal", k_cut="optimal")),
        "alpha_optimal": ([2, 2, 1], dict(alpha="optimal", r_cut=4.0, k_cut=6.998)),
        "kcut_converge": ([1, 1, 1], dict(alpha=0.6, r_cut=2.0, k_cut="converge")),
    }
    cfg, arrays = {}, {}
    for name, (size, over) in cases.items():
        tmp = tempfile.mkdtemp()
        # step_change_data_points reaches np.linspace uncast (core.py:797,
        # 1029): an int, as YAML would load it
        params = dict(HEMATITE, precision_parameters=dict(PRECISION, step_change_data_points=10),
                      **over)
        mat, nb = material_objects(core, params, poscar, size, [1, 1, 1], tmp)
        if size == [2, 2, 1]:
            pmiv = pmiv221
        else:
            nb.get_pairwise_min_image_vector_data(Path(tmp))
            pmiv = np.load(Path(tmp) / "pairwise_min_image_vector_data.npy")
            arrays[name + "|pmiv"] = pmiv
        t0 = time.time()
        res = _ref_ewald_parameters(core, mat, nb, hop, pmiv, params, tmp)
        res["system_size"], res["params"] = size, over
        res["reference_seconds"] = time.time() - t0
        cfg[name] = res
        print(f"ewald_params {name}: {res.get('alpha')}, {res.get('r_cut')}, "
              f"{res.get('k_cut')} exit={res['exit']} ({res['reference_seconds']:.1f} s)")
    cfg["poscar"] = poscar
    cfg["base_params"] = HEMATITE
    np.savez_compressed(HERE / "ewald_params.npz", **arrays)
    (HERE / "ewald_params.json").write_text(json.dumps(cfg, indent=1))


def kvector_data(core):
    """get_precomputed_array(dst, compute_energy_contributions=0,
    return_k_vector_data=1) of the reference (core.py:1611-1679) on the
    Hematite example: the sorted per-k energy contributions it logs and the
    array it returns (checked against the shipped one)."""
    name, params = "Hematite", HEMATITE
    ex = REF / "examples" / name
    poscar = (ex / "InputFiles" / "POSCAR").read_text()
    tmp = tempfile.mkdtemp()
    mat, nb = material_objects(core, params, poscar, [2, 2, 1], [1, 1, 1], tmp)
    hop = np.load(ex / "InputFiles" / "hop_neighbor_list.npy", allow_pickle=True)[()]
    pmiv = np.load(ex / "InputFiles" / "pairwise_min_image_vector_data.npy")
    A_shipped = np.load(ex / "InputFiles" / "precomputed_array.npy")
    system = make_system(core, mat, nb, hop, pmiv, params)
    dst = Path(tmp) / "InputFiles"
    dst.mkdir(parents=True, exist_ok=True)
    t0 = time.time()
    A, _ = system.get_precomputed_array(dst, 0, 1)
    dt = time.time() - t0
    err = float(np.abs(A - A_shipped).max())
    print(f"kvector_data: {dt:.1f} s, array vs shipped max |dA| = {err:.3e} Ha")
    assert err < 1e-15
    log = (dst / "k_vector_energy_contribution_within_user_specified_k_cut.log").read_text()
    report = (dst / "precomputed_array.log").read_text().split("Time elapsed")[0]
    tail = [l + "\n" for l in report.splitlines()
            if l.startswith(("k_max:", "number of k-vectors:"))]
    cfg = {"system_size": [2, 2, 1],
           "params": {k: params[k] for k in ("alpha", "r_cut", "k_cut")},
           "kvector_log": log, "report_lines": tail, "reference_seconds": dt,
           "array_vs_shipped_max_abs_ha": err}
    (HERE / "kvector_data.json").write_text(json.dumps(cfg, indent=1))


def _h5_record(path, prefix, out_json, out_arrays):
    """Flatten a stand-in HDF5 file into the fixture: structure and
    attributes into out_json[prefix], dataset values into out_arrays."""
    import fake_h5py
    rec = {}
    for key, v in sorted(fake_h5py.load(path).items()):
        if v.get("group"):
            rec[key] = {"group": True, "attrs": v["attrs"]}
            continue
        d = v["data"]
        rec[key] = {"dtype": d.dtype.str, "shape": list(d.shape),
                    "maxshape": [None if m is None else int(m) for m in v["maxshape"]],
                    "chunks": v["chunks"],
                    "compression": v["compression"], "attrs": v["attrs"]}
        out_arrays[prefix + key] = d
    out_json[prefix] = rec


def hdf5(core):
    """HDF5 output of the reference against the h5py stand-in (installed in
    main() before PyCD.core is imported, so that its HDF5_AVAILABLE holds)."""
    import contextlib
    import copy
    import io as _io
    from PyCD import hdf5_io
    rng = np.random.default_rng(7)
    rec, arrays = {}, {}
    tmp = Path(tempfile.mkdtemp())
    coords = rng.random((4, 3, 3)) * 10.0
    with hdf5_io.HDF5TrajectoryWriter(tmp / "frames.h5", 3, 1) as w:
        w.write_frame(coords[0].ravel(), 0.5)
        w.write_frames(coords[1:].reshape(3, 9), np.array([1.5, 2.5, 4.0]))
    _h5_record(tmp / "frames.h5", "frames", rec, arrays)
    arrays["frames_in_coords"] = coords
    c2 = rng.random((4, 6)) * 5.0
    hdf5_io.save_trajectory_hdf5(tmp / "save2d.h5", c2, np.arange(4, dtype=float), n_atoms=2)
    _h5_record(tmp / "save2d.h5", "save2d", rec, arrays)
    arrays["save2d_in_coords"] = c2
    c1 = rng.random(6)
    hdf5_io.save_trajectory_hdf5(tmp / "save1d.h5", c1)
    _h5_record(tmp / "save1d.h5", "save1d", rec, arrays)
    arrays["save1d_in_coords"] = c1
    # do_kmc_steps with hdf5_output ('write': 0 keeps the reference's output
    # loop, which reads every entry's 'write' (core.py:2864-2866), from
    # raising KeyError on the hdf5_output entry)
    name, params, t_final = "Hematite", HEMATITE, 6e-7
    ex = REF / "examples" / name
    poscar = (ex / "InputFiles" / "POSCAR").read_text()
    mat, nb = material_objects(core, params, poscar, [2, 2, 1], [1, 1, 1], tempfile.mkdtemp())
    hop = np.load(ex / "InputFiles" / "hop_neighbor_list.npy", allow_pickle=True)[()]
    pmiv = np.load(ex / "InputFiles" / "pairwise_min_image_vector_data.npy")
    A_shipped = np.load(ex / "InputFiles" / "precomputed_array.npy")
    system = make_system(core, mat, nb, hop, pmiv, params)
    runs = {}
    for label, every in (("run_every_step", 1), ("run_grid", 0)):
        run_p = copy.deepcopy(dict(RUN_COMMON, t_final=t_final))
        run_p["output_data"]["unwrapped_traj"]["write_every_step"] = every
        run_p["output_data"]["hdf5_output"] = {"enabled": True, "file_name": "trajectory.h5",
                                               "write": 0}
        run = core.Run(system, A_shipped, run_p["temp"], run_p["ion_charge_type"],
                       run_p["species_charge_type"], 1, t_final, run_p["time_interval"],
                       np.asarray(run_p["species_count"]), run_p["initial_occupancy"],
                       run_p["relative_energies"], run_p["external_field"], run_p["doping"])
        d = Path(tempfile.mkdtemp())
        shutil.copy(ex / "traj1" / "initial_rnd_state.dump", d / "initial_rnd_state.dump")
        out = _io.StringIO()
        with contextlib.redirect_stdout(out):
            run.do_kmc_steps(d, run_p["output_data"], run_p["random_seed"], "parallel")
        _h5_record(d / "trajectory.h5", label, rec, arrays)
        u = np.load(d / "unwrapped_traj.npy")
        t = np.load(d / "time_data.npy")
        runs[label] = {"output_data": run_p["output_data"], "rows": int(len(u)),
                       "n_steps": int(len(t) - 1),
                       "warnings": [l for l in out.getvalue().splitlines()
                                    if l.startswith("Warning")]}
        print(f"hdf5 {label}: {len(u)} rows, {len(t) - 1} steps, "
              f"warnings {runs[label]['warnings']}")
    cfg = {"t_final": t_final, "records": rec, "runs": runs}
    np.savez_compressed(HERE / "hdf5.npz", **{k.replace("/", "|"): v for k, v in arrays.items()})
    (HERE / "hdf5.json").write_text(json.dumps(cfg, indent=1))


def main(parts):
    if REF is None:
        raise SystemExit("set PYCD_REFERENCE to the root of a reference checkout")
    if "hdf5" in parts:
        import fake_h5py
        sys.modules["h5py"] = fake_h5py  # before PyCD.core reads HDF5_AVAILABLE
    core = install_shims()
    if "hdf5" in parts:
        hdf5(core)
    if "kvector_data" in parts:
        kvector_data(core)
    if "ewald_params" in parts:
        ewald_params(core)
    if "msd" in parts:
        msd(core)
    if "hematite" in parts:
        example(core, "Hematite", HEMATITE, 1e-4)
    if "every_step" in parts:
        every_step(core)
    if "hematite_outputs" in parts:
        hematite_outputs(core)
    if "bvo" in parts:
        example(core, "BVO", BVO, 1e-3)
    if "bvo_doped" in parts:
        bvo_doped(core)
    if "corundum324" in parts:
        corundum324(core)
    if "corundum3600" in parts:
        corundum3600(core)


if __name__ == "__main__":
    main(sys.argv[1:] or ["hematite", "every_step", "hematite_outputs", "bvo", "bvo_doped",
                          "corundum324", "corundum3600", "msd", "ewald_params", "kvector_data",
                          "hdf5"])
