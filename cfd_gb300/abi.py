"""ctypes mirror of include/cfd_gpu.h and the loader of the in-tree CUDA library.

The library is cfd_gb300/_build/libcfd_gb300.so, built by cfd_gb300.build.build().
There is no CPU fallback: `lib()` raises if the library is missing or no CUDA device is
usable, so every product call runs the sm_103a kernels or fails loudly.
"""
import ctypes as C
import os

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "_build", "libcfd_gb300.so")

(CFD_OK, CFD_ERR_ARG, CFD_ERR_MESH, CFD_ERR_CUDA, CFD_ERR_NOMEM, CFD_ERR_NOT_CONVERGED,
 CFD_ERR_NONFINITE, CFD_ERR_BARRIER, CFD_ERR_LIMIT, CFD_ERR_STATE) = range(10)
STATUS_NAMES = {0: "CFD_OK", 1: "CFD_ERR_ARG", 2: "CFD_ERR_MESH", 3: "CFD_ERR_CUDA",
                4: "CFD_ERR_NOMEM", 5: "CFD_ERR_NOT_CONVERGED", 6: "CFD_ERR_NONFINITE",
                7: "CFD_ERR_BARRIER", 8: "CFD_ERR_LIMIT", 9: "CFD_ERR_STATE"}

CFD_PREC_FP64, CFD_PREC_MIXED = 0, 1
CFD_MASS_MASAS, CFD_MASS_GCL_LITERAL, CFD_MASS_GCL_CORRECTED = 0, 1, 2
CFD_MOTION_REFERENCE, CFD_MOTION_HARMONIC, CFD_MOTION_NEWMARK = 0, 1, 2
CFD_GUESS_PREVIOUS, CFD_GUESS_ZERO, CFD_GUESS_LEARNED, CFD_GUESS_EXTRAPOLATED = 0, 1, 2, 3
CFD_GUESS_LEARNED_EXTRAPOLATED = 4
CFD_ESTAB_REFERENCE, CFD_ESTAB_EXACT, CFD_ESTAB_REGULARIZED = 0, 1, 2
CFD_BICG_TOL_ABS, CFD_BICG_TOL_REL, CFD_BICG_TOL_REL_R0 = 0, 1, 2
CFD_SMOOTH_COLOUR, CFD_SMOOTH_NODE_ORDER = 0, 1

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_fp = C.POINTER(C.c_float)


class CfdParams(C.Structure):
    _fields_ = [
        ("irestart", C.c_int), ("maxiter", C.c_int), ("iprint", C.c_int), ("movie", C.c_int),
        ("itlocal", C.c_int), ("ngas", C.c_int), ("moving", C.c_int),
        ("fsafe", C.c_double), ("u_inf", C.c_double), ("v_inf", C.c_double),
        ("mach_inf", C.c_double), ("t_inf", C.c_double), ("rho_inf", C.c_double),
        ("p_inf", C.c_double), ("c_inf", C.c_double),
        ("fmu", C.c_double), ("fgx", C.c_double), ("fgy", C.c_double), ("qh", C.c_double),
        ("fk", C.c_double), ("fr", C.c_double), ("fcv", C.c_double), ("gama", C.c_double),
        ("cte", C.c_double),
        ("xref", C.c_double * 10), ("yref", C.c_double * 10),
        ("motion_law", C.c_int),
        ("heave_amp", C.c_double), ("pitch_amp", C.c_double), ("motion_freq", C.c_double),
        ("mass_mode", C.c_int), ("guess_mode", C.c_int),
        ("bicg_tol", C.c_double), ("bicg_maxit", C.c_int), ("estab_mode", C.c_int),
        ("bicg_tol_mode", C.c_int), ("reserved", C.c_int * 5),
    ]


class CfdMesh(C.Structure):
    _fields_ = [
        ("npoin", C.c_int), ("nelem", C.c_int),
        ("inpoel", _ip), ("x", _dp), ("y", _dp),
        ("nfixrho", C.c_int), ("ifixrho_node", _ip), ("rfixrho_value", _dp),
        ("nfixv", C.c_int), ("ifixv_node", _ip), ("rfixv_valuex", _dp), ("rfixv_valuey", _dp),
        ("nfixt", C.c_int), ("ifixt_node", _ip), ("rfixt_value", _dp),
        ("nwall", C.c_int), ("wall", _ip),
        ("nsets", C.c_int), ("nset_numb", C.c_int), ("ielem_sets", C.c_int * 10), ("iset", _ip),
        ("nmove", C.c_int), ("nfix_move", C.c_int), ("ilaux", _ip),
    ]


class CfdStepReport(C.Structure):
    _fields_ = [
        ("iter", C.c_int), ("status", C.c_int), ("time", C.c_double), ("dtmin", C.c_double),
        ("bicg_iters", C.c_int * 2), ("bicg_rz", C.c_double * 2),
        ("bicg_converged", C.c_int * 2),
        ("fx", C.c_double * 10), ("fy", C.c_double * 10), ("rm", C.c_double * 10),
        ("nset_numb", C.c_int), ("reserved0", C.c_int),
        ("bicg_relres", C.c_double * 2), ("reserved", C.c_int * 4),
    ]


class CfdSolveInfo(C.Structure):
    _fields_ = [("iters", C.c_int), ("converged", C.c_int), ("rz", C.c_double),
                ("relres", C.c_double)]


def dptr(a):
    """Pointer to a C-contiguous float64 numpy array (None -> NULL)."""
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"], "float64 C-contiguous expected"
    return a.ctypes.data_as(_dp)


def iptr(a):
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags["C_CONTIGUOUS"], "int32 C-contiguous expected"
    return a.ctypes.data_as(_ip)


# Every symbol include/cfd_gpu.h declares, with its ctypes signature.
_P = C.c_void_p
SIGNATURES = {
    "cfd_calcrhs": (C.c_int, [_dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _ip,
                              _ip, _ip, _dp, _dp]),
    "cfd_fuente": (C.c_int, [_dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _ip, _ip, _ip]),
    "cfd_estab": (C.c_int, [_dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _ip, _ip, _ip, _dp,
                            _dp, _dp, _dp, _dp]),
    "cfd_deltat": (C.c_int, [_dp, _dp, _dp, _dp, _dp, _dp, _ip, _ip, _ip, _dp, _dp, _dp]),
    "cfd_deriv": (C.c_int, [_dp, _dp, _ip, _ip, _ip, _dp, _dp, _dp, _dp, _dp, _dp, _dp]),
    "cfd_masas": (C.c_int, [_dp, _ip, _ip, _ip, _dp]),
    "cfd_gcl": (C.c_int, [_dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _ip, _ip, _ip, _dp,
                          C.c_int]),
    "cfd_get_esup": (C.c_int, [_ip, _ip, _ip, _ip, _ip]),
    "cfd_get_psup": (C.c_int, [_ip, _ip, _ip, _ip, _ip, _ip]),
    "cfd_laplace_pattern": (C.c_int, [_ip, _ip, _ip, _ip, _ip, _ip]),
    "cfd_laplace": (C.c_int, [_ip, _dp, _dp, _dp, _ip, _ip, _dp, _dp, _dp, _ip, _ip, _dp]),
    "cfd_bicg": (C.c_int, [_dp, _ip, _ip, _dp, _dp, _dp, _dp, _ip, _ip, _ip,
                           C.POINTER(CfdSolveInfo)]),
    "cfd_bicg_ex": (C.c_int, [_dp, _ip, _ip, _dp, _dp, _dp, _dp, _ip, _ip, _ip, C.c_double,
                              C.c_int, C.POINTER(CfdSolveInfo)]),
    "cfd_bicg_mode": (C.c_int, [_dp, _ip, _ip, _dp, _dp, _dp, _dp, _ip, _ip, _ip, C.c_double,
                                C.c_int, C.c_int, C.POINTER(CfdSolveInfo)]),
    "cfd_bicg_device_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                          C.c_double, C.c_int, C.c_void_p,
                                          C.POINTER(CfdSolveInfo)]),
    "cfd_mpnn_nparams": (C.c_int, []),
    "cfd_mpnn_create": (C.c_int, [C.POINTER(_P), _fp]),
    "cfd_mpnn_destroy": (None, [_P]),
    "cfd_mpnn_get_weights": (C.c_int, [_P, _fp]),
    "cfd_mpnn_set_weights": (C.c_int, [_P, _fp]),
    "cfd_mpnn_adam_state": (C.c_int, [_P, _fp, _fp, _ip]),
    "cfd_mpnn_graph_create": (C.c_int, [C.POINTER(_P), C.c_int, C.c_int, _ip, _dp, _dp, C.c_int,
                                        _ip, _ip]),
    "cfd_mpnn_graph_destroy": (None, [_P]),
    "cfd_mpnn_graph_set_bc": (C.c_int, [_P, _dp, _dp]),
    "cfd_mpnn_graph_globals": (C.c_int, [_P, _dp]),
    "cfd_mpnn_graph_set_target": (C.c_int, [_P, _dp, _dp, _dp]),
    "cfd_mpnn_loss_grad": (C.c_int, [_P, _P, _fp, _fp]),
    "cfd_mpnn_train_step": (C.c_int, [_P, _P, C.c_float, _fp]),
    "cfd_mpnn_forward": (C.c_int, [_P, _P, C.c_int, _dp, _dp]),
    "cfd_ctx_set_guess_net": (C.c_int, [_P, _P, C.c_double]),
    "cfd_ctx_guess_stats": (C.c_int, [_P, C.POINTER(C.c_longlong)]),
    "cfd_ctx_set_guess_refine": (C.c_int, [_P, C.c_int]),
    "cfd_ctx_guess_stats_ex": (C.c_int, [_P, C.POINTER(C.c_longlong)]),
    "cfd_ctx_graph_state": (C.c_int, [_P, C.POINTER(C.c_longlong)]),
    "cfd_ctx_set_force_visc": (C.c_int, [_P, C.c_int]),
    "cfd_ctx_smooth": (C.c_int, [_P, _ip, _dp]),
    "cfd_ctx_smooth_ex": (C.c_int, [_P, C.c_int, _ip, _dp]),
    "cfd_smoothing_ex": (C.c_int, [_dp, _dp, _ip, _ip, _ip, _ip, _dp, _dp, _ip, _dp, C.c_int]),
    "cfd_selftest_waits": (C.c_int, [C.c_longlong, _ip, _ip]),
    "cfd_selftest_div3": (C.c_int, [C.c_longlong, C.c_ulonglong, C.POINTER(C.c_ulonglong)]),
    "cfd_selftest_div_rcp": (C.c_int, [C.c_longlong, C.c_ulonglong, C.POINTER(C.c_ulonglong)]),
    "cfd_ctx_set_smoothing": (C.c_int, [_P, C.c_int]),
    "cfd_ctx_smoothing_stats": (C.c_int, [_P, C.POINTER(C.c_longlong)]),
    "cfd_smoothing": (C.c_int, [_dp, _dp, _ip, _ip, _ip, _ip, _dp, _dp, _ip, _dp]),
    "cfd_ctx_force_visc": (C.c_int, [_P, _dp, _dp, _dp]),
    "cfd_force_visc": (C.c_int, [_ip] * 7 + [_dp] * 4 + [_dp] * 10 + [_dp, _dp, _dp]),
    "cfd_ctx_create": (C.c_int, [C.POINTER(_P), C.POINTER(CfdMesh), C.POINTER(CfdParams),
                                 C.c_int]),
    "cfd_ctx_destroy": (None, [_P]),
    "cfd_ctx_upload_state": (C.c_int, [_P, _dp, _dp, _dp, _dp]),
    "cfd_ctx_upload_mesh": (C.c_int, [_P, _dp, _dp, _dp, _dp, _dp, _dp]),
    "cfd_ctx_set_clock": (C.c_int, [_P, C.c_int, C.c_double, C.c_double, C.c_int,
                                    C.c_double, C.c_double]),
    "cfd_step": (C.c_int, [_P, C.c_int, C.POINTER(CfdStepReport)]),
    "cfd_ctx_download_state": (C.c_int, [_P, _dp, _dp, _dp, _dp]),
    "cfd_ctx_download_fields": (C.c_int, [_P, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp]),
    "cfd_ctx_download_motion": (C.c_int, [_P, _dp, _dp]),
    "cfd_ctx_download_geometry": (C.c_int, [_P, _dp, _dp, _dp, _dp]),
    "cfd_ctx_download_laplace": (C.c_int, [_P, _dp]),
    "cfd_ctx_timers": (C.c_int, [_P, _dp, C.c_int, _ip]),
    "cfd_ctx_timer_calls": (C.c_int, [_P, C.POINTER(C.c_longlong), C.c_int, _ip]),
    "cfd_timer_name": (C.c_char_p, [C.c_int]),
    "cfd_ctx_stream": (C.c_void_p, [_P]),
    "cfd_ctx_mark": (C.c_int, [_P, C.c_int]),
    "cfd_ctx_elapsed": (C.c_int, [_P, C.c_int, C.c_int, _dp]),
    "cfd_set_device": (C.c_int, [C.c_int]),
    "cfd_kernel_launches": (C.c_longlong, []),
    "cfd_strerror": (C.c_char_p, [C.c_int]),
    "cfd_device_available": (C.c_int, []),
}

_LIB = None


class CfdError(RuntimeError):
    def __init__(self, where, status, msg=""):
        name = STATUS_NAMES.get(status, str(status))
        super().__init__(f"{where}: {name} ({status}) {msg}".rstrip())
        self.status = status


def load(path=LIB_PATH, require_device=False):
    """Load the shared library (no device needed unless require_device)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(path):
            raise RuntimeError(
                f"CUDA library {path} is missing; run cfd_gb300.build.build() first "
                "(there is no CPU fallback)")
        lib = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = lib
    if require_device and not _LIB.cfd_device_available():
        raise RuntimeError("no usable CUDA device for libcfd_gb300 (there is no CPU fallback)")
    return _LIB


def lib():
    """The library, with a usable CUDA device required."""
    return load(require_device=True)


def check(status, where):
    if status != CFD_OK:
        msg = load().cfd_strerror(status).decode()
        raise CfdError(where, status, msg)
