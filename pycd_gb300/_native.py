"""ctypes binding of libpycd_gb300.so (include/pycd_gb300.h).

The library is the only compute path: importing this module does not need a
GPU, but every compute call raises ``NativeError`` when the library or the
device is missing.  There is no CPU fallback.
"""
import ctypes as C
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_lib" / "libpycd_gb300.so"

# status codes (PycdStatus)
OK = 0
ERR_INVALID_ARG = -1
ERR_CUDA = -2
ERR_STALLED = -3
ERR_BAD_INDEX = -4
ERR_NO_DEVICE = -5
ERR_WORKSPACE = -6

# trajectory status (PycdTrajStatus)
# ABI version of include/pycd_gb300.h that these ctypes structs mirror
ABI_VERSION = 4

TRAJ_RUNNING = 0
TRAJ_DONE = 1
TRAJ_NEED_UNIFORMS = 2
TRAJ_STALLED = 3
TRAJ_BAD_INDEX = 4
TRAJ_NO_EVENT = 5
TRAJ_STEP_LIMIT = 6
TRAJ_CANCELLED = 7
TRAJ_TIMEOUT = 8

# Ewald modes (PycdEwaldMode)
EWALD_FP64_DIRECT = 0
EWALD_FP64_GEMM = 1
EWALD_BF16X3 = 2
EWALD_TF32X3 = 3
EWALD_MODES = {"fp64_direct": EWALD_FP64_DIRECT, "fp64": EWALD_FP64_GEMM,
               "bf16x3": EWALD_BF16X3, "tf32x3": EWALD_TF32X3}


class NativeError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("pycd_gb300 native call failed (status %d): %s"
                         % (status, message))
        self.status = status


class EwaldDesc(C.Structure):
    _fields_ = [("n_sites", C.c_int64), ("n_kvec", C.c_int64),
                ("d_cart", C.c_void_p), ("d_pmiv", C.c_void_p),
                ("d_kvec", C.c_void_p), ("recip", C.c_double * 9),
                ("sim_cell", C.c_double * 9), ("sim_cell_inv", C.c_double * 9),
                ("pbc", C.c_int32 * 3), ("alpha", C.c_double),
                ("r_cut", C.c_double), ("volume", C.c_double),
                ("dielectric", C.c_double), ("parts", C.c_int32),
                ("supercell", C.c_int32 * 3), ("basis_sites", C.c_int32),
                ("split_form", C.c_int32), ("split_raster", C.c_int32)]


# PycdEwaldDesc.split_form
SPLIT_FORMS = {"auto": 0, "pair": 1, "single": 2}


EWALD_PART_REAL = 1
EWALD_PART_FOURIER = 2
EWALD_PART_SELF = 4
EWALD_PART_ALL = 7


class KmcSystem(C.Structure):
    _fields_ = [("d_A", C.c_void_p), ("d_phi_bg", C.c_void_p),
                ("d_e_rel", C.c_void_p), ("d_nbr", C.c_void_p),
                ("d_hop", C.c_void_p), ("d_lam", C.c_void_p),
                ("d_vab", C.c_void_p), ("d_field_shift", C.c_void_p),
                ("n_sites", C.c_int64), ("n_slots", C.c_int32),
                ("n_carriers", C.c_int32), ("carrier_charge", C.c_double),
                ("vn", C.c_double), ("kT", C.c_double),
                ("time_interval", C.c_double), ("n_path_steps", C.c_int64),
                ("d_rate_coef", C.c_void_p)]


class KmcState(C.Structure):
    _fields_ = [("n_traj", C.c_int32), ("max_carriers", C.c_int32),
                ("d_sys_index", C.c_void_p), ("d_occ", C.c_void_p),
                ("d_time", C.c_void_p), ("d_step", C.c_void_p),
                ("d_path_index", C.c_void_p), ("d_disp", C.c_void_p),
                ("d_last_row", C.c_void_p), ("d_energy", C.c_void_p),
                ("d_status", C.c_void_p), ("d_u_cursor", C.c_void_p),
                ("d_step_limit", C.c_void_p), ("d_csum", C.c_void_p),
                ("csum_stride", C.c_int32), ("csum_refresh", C.c_int32),
                ("d_cancel", C.c_void_p), ("time_limit_ns", C.c_int64),
                ("poll_interval", C.c_int32)]


class KmcOutputs(C.Structure):
    _fields_ = [("d_unwrapped", C.c_void_p), ("unwrapped_stride", C.c_int64),
                ("d_energy_grid", C.c_void_p), ("d_delg0_grid", C.c_void_p),
                ("d_step_time", C.c_void_p), ("d_step_proc", C.c_void_p),
                ("step_capacity", C.c_int64), ("step_offset", C.c_int64),
                ("d_drift", C.c_void_p)]


class KmcRng(C.Structure):
    _fields_ = [("d_uniforms", C.c_void_p), ("u_stride", C.c_int64),
                ("u_count", C.c_int64), ("seed", C.c_uint64),
                ("traj_offset", C.c_uint64), ("d_traj_ids", C.c_void_p)]


class KmcLaunch(C.Structure):
    _fields_ = [("lanes_per_traj", C.c_int32), ("warps_per_block", C.c_int32),
                ("blocks", C.c_int32), ("max_processes", C.c_int32),
                ("max_carriers", C.c_int32), ("min_blocks_per_sm", C.c_int32),
                ("sched_steps", C.c_int32), ("d_sched", C.c_void_p),
                ("sched_capacity", C.c_int64)]


MSD_MAX_SPECIES = 64
MSD_MAX_TYPES = 32


class MsdDesc(C.Structure):
    _fields_ = [("d_rows", C.c_void_p), ("n_traj", C.c_int64), ("n_rows", C.c_int64),
                ("traj_stride", C.c_int64), ("row_stride", C.c_int64),
                ("n_species", C.c_int32), ("n_types", C.c_int32),
                ("type_count", C.c_int32 * MSD_MAX_TYPES), ("n_lags", C.c_int64),
                ("trim_length", C.c_int64), ("dist_conversion", C.c_double),
                ("time_interval", C.c_double), ("time_conversion", C.c_double)]


P = C.POINTER
_PROTOS = {
    "pycd_last_error": (C.c_char_p, []),
    "pycd_abi_version": (C.c_int, []),
    "pycd_device_info": (C.c_int, [P(C.c_int32), P(C.c_int32), P(C.c_int32)]),
    "pycd_ewald_kvectors": (C.c_int, [P(C.c_double), P(C.c_int32), C.c_double,
                                      P(C.c_int32), C.c_int64, P(C.c_int64)]),
    "pycd_ewald_workspace_size": (C.c_int, [P(EwaldDesc), C.c_int,
                                            P(C.c_size_t)]),
    "pycd_ewald_build": (C.c_int, [P(EwaldDesc), C.c_int, C.c_void_p,
                                   C.c_void_p, C.c_size_t, C.c_void_p,
                                   P(C.c_float), P(C.c_float)]),
    "pycd_ewald_build_noalloc": (C.c_int, [P(EwaldDesc), C.c_void_p, C.c_void_p]),
    "pycd_potential_gemv": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p,
                                      C.c_void_p, C.c_void_p, C.c_void_p]),
    "pycd_kmc_workspace_size": (C.c_int, [P(KmcSystem), C.c_int32, P(C.c_size_t)]),
    "pycd_kmc_advance": (C.c_int, [P(KmcSystem), C.c_int32, P(KmcState),
                                   P(KmcOutputs), P(KmcRng), C.c_int64,
                                   P(KmcLaunch), C.c_void_p, C.c_size_t,
                                   C.c_void_p]),
    "pycd_kmc_upload_systems": (C.c_int, [P(KmcSystem), C.c_int32, C.c_void_p,
                                          C.c_size_t, C.c_void_p,
                                          P(KmcLaunch)]),
    "pycd_kmc_advance_uploaded": (C.c_int, [C.c_int32, P(KmcState),
                                            P(KmcOutputs), P(KmcRng),
                                            C.c_int64, P(KmcLaunch),
                                            C.c_void_p, C.c_size_t,
                                            C.c_void_p]),
    "pycd_kmc_default_lanes": (C.c_int, [C.c_int32, C.c_int32, C.c_int64,
                                         P(C.c_int32)]),
    "pycd_philox_uniforms": (C.c_int, [C.c_uint64, C.c_uint64, C.c_int64,
                                       C.c_int64, C.c_void_p, C.c_void_p]),
    "pycd_kmc_rate_coefficients": (C.c_int, [P(KmcSystem), C.c_void_p, C.c_void_p]),
    "pycd_potential_sparse": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p,
                                        C.c_int32, C.c_void_p, C.c_void_p]),
    "pycd_debug_exp": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p,
                                 C.c_void_p]),
    "pycd_debug_exp_table": (C.c_int, [C.c_void_p]),
    "pycd_debug_exp_table_fixed": (C.c_int, [C.c_void_p]),
    "pycd_ewald_kvector_energies": (C.c_int, [P(EwaldDesc), C.c_void_p, C.c_void_p,
                                              C.c_void_p]),
    "pycd_msd_compute": (C.c_int, [P(MsdDesc), C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
}

_lib = None


def lib():
    """Load (building first if needed) and return the shared library."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            from .build import build
            build()
        handle = C.CDLL(str(LIB_PATH))
        for name, (res, args) in _PROTOS.items():
            fn = getattr(handle, name)
            fn.restype = res
            fn.argtypes = args
        if handle.pycd_abi_version() != ABI_VERSION:
            raise NativeError(ERR_INVALID_ARG,
                              "%s has ABI version %d, this package needs %d: rebuild it"
                              % (LIB_PATH, handle.pycd_abi_version(), ABI_VERSION))
        _lib = handle
    return _lib


def exported_symbols():
    return list(_PROTOS)


def check(status):
    if status != OK:
        msg = lib().pycd_last_error().decode(errors="replace")
        raise NativeError(status, msg)
    return status


def require_device():
    """Raise NativeError unless an sm_103 GPU is current."""
    sm, ma, mi = C.c_int32(), C.c_int32(), C.c_int32()
    check(lib().pycd_device_info(C.byref(sm), C.byref(ma), C.byref(mi)))
    return sm.value, ma.value, mi.value


def ptr(t):
    """Device (or host) address of a tensor, or None."""
    if t is None:
        return None
    return t.data_ptr()


def stream_handle(stream=None):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)
