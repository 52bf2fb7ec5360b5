"""ctypes binding of libdegpu.so (include/degpu.h).  The product path: there is no
Python or CPU fallback -- if the library or a GPU is missing, calls raise."""
from __future__ import annotations

import ctypes
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libdegpu.so"

OK, E_INVALID, E_COMPILE, E_CUDA, E_UNSUPPORTED = 0, -1, -2, -3, -4
(ALG_TSIT5, ALG_VERN7, ALG_ROSENBROCK23, ALG_RODAS5P, ALG_EM, ALG_RODAS4, ALG_VERN9, ALG_SIEA, ALG_KVAERNO3,
 ALG_KVAERNO5) = range(10)
TIME_F32, TIME_F64 = 0, 1
MODE_FAST, MODE_PARITY = 0, 1
DRIVER_AUTO, DRIVER_NAIVE, DRIVER_PERSISTENT = 0, 1, 2
JAC_AUTO, JAC_AD, JAC_FINITEDIFF = 0, 1, 2
RHS_HAS_JAC, RHS_HAS_TGRAD, RHS_HAS_NOISE, RHS_HAS_MASS = 1, 2, 4, 8
RET_DEFAULT, RET_SUCCESS, RET_TERMINATED, RET_DTLESSTHANMIN, RET_MAXITERS, RET_UNSTABLE = range(6)
RETCODE_NAMES = {0: "Default", 1: "Success", 2: "Terminated", 3: "DtLessThanMin", 4: "MaxIters", 5: "Unstable"}


class Problems(ctypes.Structure):
    _fields_ = [("u0", ctypes.c_void_p), ("p", ctypes.c_void_p), ("tspan", ctypes.c_void_p), ("B", ctypes.c_longlong)]


class Options(ctypes.Structure):
    _fields_ = [
        ("alg", ctypes.c_int), ("time_type", ctypes.c_int), ("mode", ctypes.c_int), ("driver", ctypes.c_int),
        ("jac", ctypes.c_int), ("save_everystep", ctypes.c_int), ("nsaveat", ctypes.c_int),
        ("saveat_per_traj", ctypes.c_int), ("saveat", ctypes.c_void_p), ("dt", ctypes.c_double),
        ("abstol", ctypes.c_double), ("reltol", ctypes.c_double), ("maxiters", ctypes.c_longlong),
        ("dt0", ctypes.c_void_p), ("tolscale", ctypes.c_void_p), ("seed", ctypes.c_ulonglong),
        ("traj_offset", ctypes.c_longlong), ("block", ctypes.c_int), ("chunk", ctypes.c_int),
        ("ntstops", ctypes.c_int), ("tstops", ctypes.c_void_p), ("callbacks", ctypes.c_void_p),
        ("order", ctypes.c_void_p),
    ]


class ContinuousCallbackC(ctypes.Structure):
    _fields_ = [("fn", ctypes.c_int), ("has_affect", ctypes.c_int), ("has_affect_neg", ctypes.c_int),
                ("rootfind", ctypes.c_int), ("abstol", ctypes.c_double), ("repeat_nudge", ctypes.c_double),
                ("dtrelax", ctypes.c_double)]


class CallbacksC(ctypes.Structure):
    _fields_ = [("n_continuous", ctypes.c_int), ("continuous", ctypes.POINTER(ContinuousCallbackC)),
                ("n_discrete", ctypes.c_int), ("discrete", ctypes.POINTER(ctypes.c_int))]


MAX_CALLBACKS = 8
ROOTFIND_LEFT, ROOTFIND_RIGHT, ROOTFIND_NONE = 0, 1, 2


class Outputs(ctypes.Structure):
    _fields_ = [("ts", ctypes.c_void_p), ("us", ctypes.c_void_p), ("L", ctypes.c_int),
                ("retcode", ctypes.c_void_p), ("naccept", ctypes.c_void_p), ("nreject", ctypes.c_void_p),
                ("dt_first", ctypes.c_void_p)]


class DegpuError(RuntimeError):
    """Error reported by libdegpu (message from degpu_last_error)."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"degpu error {code}: {msg}")
        self.code = code


# every symbol include/degpu.h declares, with its ctypes signature
_P = ctypes.c_void_p
SIGNATURES = {
    "degpu_version": (ctypes.c_char_p, []),
    "degpu_trim_memory": (None, []),
    "degpu_abi_struct_sizes": (None, [ctypes.POINTER(ctypes.c_int)] * 5),
    "degpu_last_error": (ctypes.c_char_p, []),
    "degpu_rhs_create": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(_P)]),
    "degpu_rhs_destroy": (None, [_P]),
    "degpu_builtin_rhs": (ctypes.c_char_p, [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                            ctypes.POINTER(ctypes.c_int)]),
    "degpu_vectorized_solve": (ctypes.c_int, [_P, ctypes.POINTER(Problems), ctypes.POINTER(Options), ctypes.POINTER(Outputs), _P]),
    "degpu_vectorized_asolve": (ctypes.c_int, [_P, ctypes.POINTER(Problems), ctypes.POINTER(Options), ctypes.POINTER(Outputs), _P]),
    "degpu_vectorized_solve_sde": (ctypes.c_int, [_P, ctypes.POINTER(Problems), ctypes.POINTER(Options), ctypes.POINTER(Outputs), _P]),
    "degpu_batch_solve_host": (ctypes.c_int, [_P, _P, _P, _P, ctypes.c_longlong, ctypes.POINTER(Options), ctypes.c_int,
                                              _P, _P, ctypes.c_int, _P, _P, _P, _P]),
    "degpu_plan_create": (ctypes.c_int, [_P, ctypes.POINTER(Problems), ctypes.POINTER(Options), ctypes.c_int,
                                         ctypes.POINTER(Outputs), _P, ctypes.POINTER(_P)]),
    "degpu_plan_launch": (ctypes.c_int, [_P, _P]),
    "degpu_plan_info": (ctypes.c_int, [_P] + [ctypes.POINTER(ctypes.c_int)] * 5),
    "degpu_plan_destroy": (None, [_P]),
    "degpu_autotune": (ctypes.c_int, [_P, ctypes.POINTER(Problems), ctypes.POINTER(Options), ctypes.c_int,
                                      ctypes.POINTER(Outputs), ctypes.c_longlong, _P, ctypes.POINTER(ctypes.c_int),
                                      ctypes.POINTER(ctypes.c_int)]),
    "degpu_rhs_check": (ctypes.c_int, [_P, ctypes.POINTER(Options), ctypes.c_int, ctypes.POINTER(ctypes.c_longlong)]),
    "degpu_fp32_peak": (ctypes.c_int, [ctypes.POINTER(ctypes.c_double), _P]),
    "degpu_mlp_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_ulonglong, ctypes.POINTER(_P)]),
    "degpu_mlp_destroy": (None, [_P]),
    "degpu_mlp_param_count": (ctypes.c_int, [_P]),
    "degpu_mlp_set_params": (ctypes.c_int, [_P, _P, _P, _P]),
    "degpu_mlp_get_params": (ctypes.c_int, [_P, _P, _P, _P, _P]),
    "degpu_mlp_infer": (ctypes.c_int, [_P, _P, ctypes.c_longlong, _P, _P, _P, ctypes.c_float, ctypes.c_float,
                                       ctypes.c_float, ctypes.c_float, _P]),
    "degpu_mlp_infer_problems": (ctypes.c_int, [_P, _P, ctypes.c_int, _P, ctypes.c_int, ctypes.c_float,
                                                ctypes.c_longlong, _P, _P, ctypes.c_float, ctypes.c_float,
                                                ctypes.c_float, ctypes.c_float, _P]),
    "degpu_learned_asolve": (ctypes.c_int, [_P, _P, ctypes.POINTER(Problems), ctypes.POINTER(Options), ctypes.c_float,
                                            ctypes.c_float, ctypes.c_float, ctypes.POINTER(Outputs), _P]),
    "degpu_learned_asolve_ex": (ctypes.c_int, [_P, _P, _P, ctypes.POINTER(Problems), ctypes.POINTER(Options),
                                               ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                               ctypes.POINTER(Outputs), _P]),
    "degpu_work_order": (ctypes.c_int, [_P, ctypes.c_longlong, _P, _P]),
    "degpu_learned_batch_solve_host": (ctypes.c_int, [_P, _P, _P, _P, _P, _P, ctypes.c_longlong,
                                                      ctypes.POINTER(Options), ctypes.c_float, ctypes.c_float,
                                                      ctypes.c_float, _P, _P, ctypes.c_int, _P, _P, _P, _P]),
    "degpu_learned_asolve_noalloc": (ctypes.c_int, [_P, _P, ctypes.POINTER(Problems), ctypes.POINTER(Options),
                                                    ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                                    ctypes.POINTER(Outputs), _P]),
    "degpu_mlp_grad": (ctypes.c_int, [_P, _P, _P, _P, ctypes.c_longlong, _P, _P]),
    "degpu_mlp_adam_step": (ctypes.c_int, [_P, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                           ctypes.c_float, _P]),
    "degpu_kernel_info": (ctypes.c_int, [_P, ctypes.POINTER(Options), ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                         ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
}

_lib = None


def lib():
    """Load libdegpu.so (built by diffeqgpu.jl_gb300/build.py).  Raises if it is missing."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(f"{LIB_PATH} is missing: run `python -c 'import __graft_entry__ as g; g.build()'` first "
                              "(degpu has no CPU fallback)")
        L = ctypes.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(rc: int) -> None:
    if rc != OK:
        raise DegpuError(rc, lib().degpu_last_error().decode(errors="replace"))


def extra_signatures(extra: dict) -> None:
    """Register signatures of additional entry points (used by sibling modules)."""
    L = lib()
    for name, (res, args) in extra.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
        SIGNATURES.setdefault(name, (res, args))
