"""ctypes binding of libtopopt_gb300.so (include/topopt_gb300.h).

The library is built in-tree by ``topoptlab_gb300.build``; importing this
module never falls back to a CPU implementation: if the shared library is
missing or cannot be loaded, every call raises ``RuntimeError``.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libtopopt_gb300.so")

TG_OK, TG_EINVAL, TG_ENOTCONV, TG_ETIMEOUT, TG_ENAN, TG_ECUDA, TG_ENOMEM = range(7)
TG_PREC_FP64, TG_PREC_MIXED = 0, 1
TG_PRECOND_GMG, TG_PRECOND_JACOBI = 0, 1
(TG_FIELD_X, TG_FIELD_XPHYS, TG_FIELD_U, TG_FIELD_DC, TG_FIELD_DV, TG_FIELD_F) = range(6)
TG_TUNE_STENCIL_SMALL_PAIRS, TG_TUNE_OC_BARRIER_TIMEOUT = 1, 2
TG_TUNE_COARSE_TAIL, TG_TUNE_TAIL_BARRIER_TIMEOUT, TG_TUNE_STENCIL_TMA = 3, 4, 5
TG_TUNE_PDL, TG_TUNE_CONV_UMMA, TG_TUNE_CONV_TIMEOUT = 6, 7, 8
TG_LEARNED_WARM_START, TG_LEARNED_COARSE_CORRECTION = 1, 2
TG_ABI_VERSION = 6            # the header this binding follows
TG_NOALLOC_MAX_N = 2097152    # design variables tg_oc_noalloc's static scratch holds

_dp = C.POINTER(C.c_double)
_i64p = C.POINTER(C.c_int64)
_i32p = C.POINTER(C.c_int32)
_i8p = C.POINTER(C.c_int8)


class TgProblem(C.Structure):
    _fields_ = [
        ("ndim", C.c_int32), ("nnode_dof", C.c_int32),
        ("nelx", C.c_int32), ("nely", C.c_int32), ("nelz", C.c_int32),
        ("KE", _dp), ("fixed", _i64p), ("nfixed", C.c_int64), ("f", _dp),
        ("volfrac", C.c_double), ("rmin", C.c_double), ("eps", C.c_double),
        ("penal", C.c_double), ("move", C.c_double),
        ("ft", C.c_int32), ("el_flags", _i8p),
        ("precond", C.c_int32), ("precision", C.c_int32), ("nlevels", C.c_int32),
        ("nsmooth", C.c_int32), ("omega", C.c_double), ("rtol", C.c_double),
        ("maxiter", C.c_int32), ("inner_rtol", C.c_double), ("learned", C.c_int32),
        ("device", C.c_int32), ("nload", C.c_int32),
        ("filter_pde", C.c_int32), ("KF", _dp), ("unsmoothed", C.c_int32),
        ("nsmooth_coarse", C.c_int32),
    ]


class TgIterOut(C.Structure):
    _fields_ = [
        ("obj", C.c_double), ("vol", C.c_double), ("change", C.c_double), ("g", C.c_double),
        ("rel_res", C.c_double),
        ("pcg_iters", C.c_int32), ("vcycles", C.c_int32), ("refinements", C.c_int32),
        ("oc_steps", C.c_int32), ("fallback", C.c_int32), ("nlevels", C.c_int32),
        ("t_solve_ms", C.c_double), ("t_step_ms", C.c_double), ("warm_ratio", C.c_double),
    ]


class TgSolveInfo(C.Structure):
    _fields_ = [("iters", C.c_int32), ("vcycles", C.c_int32), ("refinements", C.c_int32),
                ("converged", C.c_int32), ("rel_res", C.c_double)]


# symbol -> (restype, argtypes); exactly the functions include/topopt_gb300.h declares
SIGNATURES = {
    "tg_abi_version": (C.c_int32, []),
    "tg_last_error": (C.c_char_p, [C.c_void_p]),
    "tg_create": (C.c_int32, [C.POINTER(TgProblem), C.POINTER(C.c_void_p)]),
    "tg_destroy": (None, [C.c_void_p]),
    "tg_step": (C.c_int32, [C.c_void_p, C.POINTER(TgIterOut)]),
    "tg_step_many": (C.c_int32, [C.POINTER(C.c_void_p), C.c_int32, C.POINTER(TgIterOut),
                                 C.POINTER(C.c_int32), C.c_int32]),
    "tg_get": (C.c_int32, [C.c_void_p, C.c_int32, _dp, C.c_int64]),
    "tg_set": (C.c_int32, [C.c_void_p, C.c_int32, _dp, C.c_int64]),
    "tg_kmul": (C.c_int32, [C.c_void_p, _dp, _dp, _dp, C.c_int32]),
    "tg_solve": (C.c_int32, [C.c_void_p, _dp, _dp, _dp, _dp, C.POINTER(TgSolveInfo)]),
    "tg_filter": (C.c_int32, [C.c_void_p, _dp, _dp, _dp, C.c_int32]),
    "tg_compliance": (C.c_int32, [C.c_void_p, _dp, _dp, _dp, _dp]),
    "tg_oc": (C.c_int32, [C.c_void_p, _dp, _dp, _dp, C.c_double, _dp, _dp, _i32p]),
    "tg_oc_raw": (C.c_int32, [C.c_int64, _dp, _dp, _dp, C.c_double, _i8p, C.c_double,
                              C.c_double, C.c_double, _dp, _dp, _i32p, C.c_int32]),
    "tg_oc_noalloc": (C.c_int32, [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double,
                                  C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_void_p,
                                  _dp, _i32p, C.c_void_p]),
    "tg_noalloc_last_error": (C.c_char_p, []),
    "tg_vcycle": (C.c_int32, [C.c_void_p, _dp, _dp, _dp, C.c_int32]),
    "tg_levels": (C.c_int32, [C.c_void_p, _i32p, _i64p]),
    "tg_coarse_stencil": (C.c_int32, [C.c_void_p, _dp, C.c_int32, _dp, C.c_int64]),
    "tg_cnn_create": (C.c_int32, [C.c_void_p, C.c_int32, C.c_uint64, C.POINTER(C.c_void_p)]),
    "tg_cnn_destroy": (None, [C.c_void_p]),
    "tg_cnn_attach": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "tg_cnn_record_begin": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "tg_cnn_record_end": (C.c_int32, [C.c_void_p, C.c_void_p]),
    "tg_cnn_train": (C.c_int32, [C.c_void_p, C.c_int32, C.c_double, C.c_uint64, _dp]),
    "tg_cnn_fit": (C.c_int32, [C.c_void_p, C.c_int32, C.POINTER(C.c_float), C.POINTER(C.c_float),
                               C.c_int32, C.c_double, C.c_uint64, _dp]),
    "tg_cnn_info": (C.c_int32, [C.c_void_p, _i64p, _i32p, _i32p]),
    "tg_cnn_params": (C.c_int32, [C.c_void_p, C.c_int32, C.POINTER(C.c_float), C.c_int64]),
    "tg_cnn_eval": (C.c_int32, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                C.POINTER(C.c_float), _dp, C.POINTER(C.c_float)]),
    "tg_cnn_infer": (C.c_int32, [C.c_void_p, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "tg_adjoint": (C.c_int32, [C.c_void_p, _dp, _dp, _dp, _dp, C.POINTER(TgSolveInfo)]),
    "tg_csr_pcg": (C.c_int32, [C.c_int64, _i64p, _i32p, _dp, _dp, _dp, _dp, C.c_double,
                               C.c_double, C.c_int32, C.c_int32, C.POINTER(TgSolveInfo),
                               C.c_int32]),
    "tg_csr_last_error": (C.c_char_p, []),
    "tg_timer": (C.c_int32, [C.c_void_p, C.c_int32, _dp]),
    "tg_profile_kernel": (C.c_int32, [C.c_int32]),
    "tg_stats": (C.c_int32, [C.c_int32, _i64p, _dp, _i64p]),
    "tg_tune": (C.c_int32, [C.c_int32, C.c_int64]),
    "tg_dense_inverse": (C.c_int32, [_dp, C.c_int64, _dp, C.c_int32, C.c_int32]),
    "tg_edofmat": (C.c_int32, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, _i32p,
                               C.c_int32]),
}

_lib = None


def load(path: str = LIB_PATH):
    """Load the shared library and bind every declared symbol."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            f"CUDA library {path} is missing: build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` (no CPU fallback exists)")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def dptr(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def check(rc: int, ctx=None, what: str = ""):
    if rc == TG_OK:
        return
    msg = load().tg_last_error(ctx).decode(errors="replace")
    text = f"{what}: {msg}" if what else msg
    if rc == TG_EINVAL:
        raise ValueError(text)
    raise RuntimeError(text)


def f64(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))
