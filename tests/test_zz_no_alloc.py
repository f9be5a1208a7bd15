"""GPU: the allocation-free Ewald build entry point.

``pycd_ewald_build_noalloc`` serves callers that must not allocate device
memory (for example a C or Fortran host that only receives input and output
device buffers from another runtime whose allocator owns the GPU).  Its
scratch is a fixed array inside the library.  Here it is called through the
C ABI and compared with ``pycd_ewald_build`` (caller workspace) within the
Ewald tolerance of the other tests (1e-10 eV per entry), twice in a row, so
that the shared scratch left by the first call cannot change the second, and
against the reference's own array rows of the 324-site corundum lattice.
This file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

import golden_io as gio
from pycd_gb300 import _native as nat
from pycd_gb300 import constants as K
from pycd_gb300 import ewald as ew
from pycd_gb300 import workloads as wl

pytestmark = pytest.mark.gpu
TOL_HA = 1e-10 * K.EV2HARTREE


def _reference_build(sysm, desc):
    import torch
    n = int(desc.n_sites)
    L = nat.lib()
    ws_bytes = ctypes.c_size_t()
    nat.check(L.pycd_ewald_workspace_size(ctypes.byref(desc), nat.EWALD_FP64_GEMM,
                                          ctypes.byref(ws_bytes)))
    ws = torch.empty(ws_bytes.value, dtype=torch.uint8, device="cuda")
    out = torch.empty((n, n), dtype=torch.float64, device="cuda")
    nat.check(L.pycd_ewald_build(ctypes.byref(desc), nat.EWALD_FP64_GEMM,
                                 out.data_ptr(), ws.data_ptr(), ws_bytes.value,
                                 nat.stream_handle(), None, None))
    return out


def test_noalloc_build_matches_workspace_build_twice(cuda_ready):
    import torch
    sysm = wl.corundum((3, 3, 3))
    desc, keep, _ = ew.make_desc(sysm, sysm.alpha, sysm.r_cut, sysm.k_cut)
    assert desc.n_sites == 324 and desc.n_kvec == 280
    ref = _reference_build(sysm, desc).cpu().numpy()
    L = nat.lib()
    for call in range(2):
        out = torch.full((324, 324), float("nan"), dtype=torch.float64, device="cuda")
        nat.check(L.pycd_ewald_build_noalloc(ctypes.byref(desc), out.data_ptr(),
                                             nat.stream_handle()))
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.isfinite(got).all(), call
        assert np.abs(got - ref).max() < TOL_HA, call
        # the reference's own rows and diagonal of this array
        cfg, arr = gio.load("corundum324")
        rows = np.asarray(cfg["A_rows"])
        assert np.abs(got[rows] - arr["A_rows"]).max() < TOL_HA, call
        assert np.abs(np.diag(got) - arr["A_diag"]).max() < TOL_HA, call


def test_noalloc_build_rejects_sizes_beyond_its_scratch(cuda_ready):
    import torch
    sysm = wl.corundum((10, 10, 3), neighbor_list=False)
    desc, keep, _ = ew.make_desc(sysm, sysm.alpha, sysm.r_cut, sysm.k_cut)
    out = torch.empty((1, 1), dtype=torch.float64, device="cuda")
    rc = nat.lib().pycd_ewald_build_noalloc(ctypes.byref(desc), out.data_ptr(),
                                            nat.stream_handle())
    assert rc == nat.ERR_WORKSPACE
    assert b"scratch" in nat.lib().pycd_last_error()


def test_noalloc_real_space_only_build_needs_no_k_scratch(cuda_ready):
    """A build without the Fourier part needs no per-k scratch, so a system
    whose full build exceeds the fixed scratch still runs real space only,
    equal to the workspace build of the same part."""
    import torch
    sysm = wl.corundum((10, 10, 3), neighbor_list=False)
    desc, keep, _ = ew.make_desc(sysm, sysm.alpha, sysm.r_cut, sysm.k_cut)
    desc.parts = nat.EWALD_PART_REAL
    ref = _reference_build(sysm, desc)
    out = torch.full_like(ref, float("nan"))
    for call in range(2):
        nat.check(nat.lib().pycd_ewald_build_noalloc(ctypes.byref(desc), out.data_ptr(),
                                                     nat.stream_handle()))
        torch.cuda.synchronize()
        assert torch.equal(out, ref), call
