"""GPU: the MSD analysis (pycd_msd_compute through pycd_gb300.analysis)
against the reference's own outputs and against the oracle on rows of a
batched KMC run read in place from device memory."""
import types

import numpy as np
import pytest

import golden_io as gio
from oracle import msd_oracle as mo
from pycd_gb300 import _native as nat
from pycd_gb300 import constants as K
from pycd_gb300 import workloads as wl
from pycd_gb300.analysis import Analysis, msd_device
from pycd_gb300.batch import BatchedKmc

pytestmark = pytest.mark.gpu

# FP64 sums in a different order from NumPy's: relative to the largest value
RTOL = 1e-12


def _close(a, b, rtol=RTOL):
    a, b = np.asarray(a), np.asarray(b)
    scale = max(np.abs(b[np.isfinite(b)]).max(initial=0.0), 1e-300)
    assert a.shape == b.shape
    assert np.array_equal(np.isnan(a), np.isnan(b))
    ok = np.isfinite(b)
    assert np.abs(a[ok] - b[ok]).max(initial=0.0) <= rtol * scale


@pytest.mark.parametrize("name", ["hematite", "synthetic"])
def test_compute_msd_matches_reference(cuda_ready, tmp_path, name):
    cfg, arr = gio.load("msd")
    c = cfg[name]
    pre = "hem" if name == "hematite" else "syn"
    rows = arr[pre + "_rows"]
    rows = rows[None] if rows.ndim == 2 else rows
    for i, r in enumerate(rows):
        (tmp_path / f"traj{i + 1}").mkdir()
        np.save(tmp_path / f"traj{i + 1}" / "unwrapped_traj.npy", r)
    mat = types.SimpleNamespace(species_types=c["species_types"],
                                num_species_types=len(c["species_types"]))
    an = Analysis(mat, c["n_dim"], c["species_count"], c["n_traj"], c["t_final"],
                  c["time_interval"], c["msd_t_final"], c["trim_length"], c["temp"],
                  c["repr_time"], c["repr_dist"])
    out = an.compute_msd(tmp_path, {"unwrapped_traj": {"file_name": "unwrapped_traj.npy"}})
    assert np.array_equal(out.msd_data[:, 0], arr[pre + "_msd"][:, 0])
    _close(out.msd_data, arr[pre + "_msd"])
    _close(out.sem_data, arr[pre + "_sem"])
    assert out.file_name == c["file_name"] and out.species_types == c["out_species"]
    saved = np.load(tmp_path / f"MSD_Data_{c['file_name']}.npy")
    assert np.array_equal(saved, out.msd_data)
    report = (tmp_path / f"MSD_Analysis_{c['file_name']}.log").read_text()
    assert report.startswith(c["report_prefix"])


def _kmc_rows(n_traj=12, width=8):
    """Unwrapped rows of a batched KMC run on 108 corundum sites, 3 carriers
    (the batch is 8 carriers wide, so rows have a stride of 24 doubles)."""
    import torch
    system = wl.system_for("corundum", (3, 3, 1))
    A = system.get_precomputed_array_device("fp64")
    t_final, dt = 2e-10, 5e-13
    tables, run = wl.batched_tables(system, A, 3, [], 1.0, t_final, dt)
    rng = np.random.default_rng(4)
    occ = np.zeros((n_traj, width), np.int32)
    for t in range(n_traj):
        occ[t, :3] = rng.choice(tables.n_sites, 3, replace=False)
    bk = BatchedKmc(tables, occ, seed=5, chunk_steps=20000, unwrapped=True)
    for _ in range(200):
        bk.run(20000)
        if (bk.gather("status").cpu().numpy() == nat.TRAJ_DONE).all():
            break
    torch.cuda.synchronize()
    assert (bk.gather("status").cpu().numpy() == nat.TRAJ_DONE).all()
    return bk.gather("unwrapped"), t_final, dt, run


def test_msd_device_on_kmc_rows_matches_oracle(cuda_ready):
    rows, t_final, dt, run = _kmc_rows()
    S = 3
    host = rows.cpu().numpy()[:, :, :3 * S]
    o = mo.compute_msd(host, ["electron"], [S], 3, t_final, dt, 60 * dt * 1e9, 5, 300,
                       "ns", "angstrom")
    assert o["n_rows"] == rows.shape[1]
    res = msd_device(rows, [S], o["n_rows"], o["n_lags"], 5, 1 / K.ANG2BOHR,
                     dt * K.SEC2AUTIME, K.AUTIME2NS)
    _close(res["sd"].cpu().numpy(), o["sd"])
    _close(res["species_avg"].cpu().numpy(), o["species_avg"])
    _close(res["msd_data"].cpu().numpy(), o["msd_data"])
    _close(res["sem_data"].cpu().numpy(), o["sem_data"])
    _close(res["slopes"].cpu().numpy(), o["slopes"], 1e-10)
    stats = res["slope_stats"].cpu().numpy()
    assert np.allclose(stats[0], o["slopes"].mean(axis=0), rtol=1e-10, atol=0)


def test_msd_device_edges(cuda_ready):
    """Lags beyond the rows give NaN as the reference's empty mean; one
    trajectory gives zero standard error; two species types average apart."""
    import torch
    rng = np.random.default_rng(9)
    host = np.cumsum(rng.normal(0, 3.0, size=(1, 40, 9)), axis=1)
    rows = torch.from_numpy(host).cuda()
    res = msd_device(rows, [2, 1], 40, 55, 3, 0.5, 1.0, 1.0)
    sd = res["sd"].cpu().numpy()
    assert np.isnan(sd[0, 40:]).all() and np.isfinite(sd[0, :40]).all()
    assert (sd[0, 0] == 0).all()
    ref = mo.squared_displacements((host[0, :40] * 0.5).reshape(40, 3, 3), 40)
    _close(sd[0, :40], ref)
    avg = res["species_avg"].cpu().numpy()[0, :40]
    _close(avg[:, 0], ref[:, :2].mean(axis=1))
    _close(avg[:, 1], ref[:, 2])
    assert (res["sem_data"].cpu().numpy()[:40] == 0).all()


def test_msd_rejects_bad_descriptors(cuda_ready):
    import ctypes as C
    import torch
    rows = torch.zeros((2, 10, 6), dtype=torch.float64, device="cuda")
    with pytest.raises(ValueError):
        msd_device(rows, [3], 10, 5, 1, 1.0, 1.0, 1.0)  # 3 carriers need 9 columns
    out = torch.zeros(2 * 10 * 2 + 64, dtype=torch.float64, device="cuda")
    d = nat.MsdDesc()
    d.d_rows, d.n_traj, d.n_rows, d.traj_stride, d.row_stride = rows.data_ptr(), 2, 10, 60, 6
    d.n_species, d.n_types, d.n_lags, d.trim_length = 2, 1, 10, 5
    d.type_count[0] = 2
    d.dist_conversion = d.time_interval = d.time_conversion = 1.0
    p = out.data_ptr()
    lib = nat.lib()
    # slope fit over [5, 5): fewer than 2 lags
    with pytest.raises(nat.NativeError):
        nat.check(lib.pycd_msd_compute(C.byref(d), p, p, p, p, p, p, None))
    d.trim_length, d.type_count[0] = 1, 3  # type counts do not sum to n_species
    with pytest.raises(nat.NativeError):
        nat.check(lib.pycd_msd_compute(C.byref(d), p, p, p, p, p, p, None))
    d.type_count[0], d.row_stride = 2, 5  # a row cannot hold 2 carriers
    with pytest.raises(nat.NativeError):
        nat.check(lib.pycd_msd_compute(C.byref(d), p, None, None, None, None, None, None))
