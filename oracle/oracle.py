"""ctypes front-end of the CPU oracle (oracle/oracle.cpp) -- TEST INFRASTRUCTURE ONLY.

Used by tests/, __graft_entry__.smoke() and bench.py's CPU baseline / reference arm as
the checker or the timed CPU restatement; never by the product path.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"

ALG = {"tsit5": 0, "vern7": 1, "rosenbrock23": 2, "rodas5p": 3, "em": 4, "rodas4": 5, "vern9": 6, "siea": 7, "kvaerno3": 8, "kvaerno5": 9}
MODEL = {"lorenz": 0, "robertson": 1, "decay": 2, "growth": 3, "linear15": 4,
         "gbm": 5, "lorenz_addnoise": 6, "osc": 7, "ball": 8, "robertson_dae": 9}
JAC = {"ad": 0, "analytic": 1, "finitediff": 2}
RET = {"default": 0, "success": 1, "terminated": 2, "dtmin": 3, "maxiters": 4, "unstable": 5}


class OracleCfg(ctypes.Structure):
    _fields_ = [
        ("alg", ctypes.c_int), ("adaptive", ctypes.c_int), ("time_f64", ctypes.c_int),
        ("save_everystep", ctypes.c_int), ("L", ctypes.c_int), ("nsaveat", ctypes.c_int),
        ("saveat_per_traj", ctypes.c_int), ("jac", ctypes.c_int),
        ("saveat", ctypes.POINTER(ctypes.c_double)), ("dt", ctypes.c_double),
        ("abstol", ctypes.c_float), ("reltol", ctypes.c_float), ("maxiters", ctypes.c_longlong),
        ("seed", ctypes.c_ulonglong), ("dt0", ctypes.POINTER(ctypes.c_float)),
        ("tolscale", ctypes.POINTER(ctypes.c_float)),
        ("ntstops", ctypes.c_int), ("tstops", ctypes.POINTER(ctypes.c_double)),
        ("nccb", ctypes.c_int), ("ccb_fn", ctypes.c_int * 8), ("ccb_flags", ctypes.c_int * 8),
        ("ccb_abstol", ctypes.c_float * 8), ("ccb_nudge", ctypes.c_float * 8), ("ccb_dtrelax", ctypes.c_float * 8),
        ("ndcb", ctypes.c_int), ("dcb_fn", ctypes.c_int * 8),
    ]


def build(force: bool = False) -> Path:
    """Compile the oracle with its Makefile (gcc/g++ only)."""
    if force or not LIB_PATH.exists() or any(
            (HERE / f).stat().st_mtime > LIB_PATH.stat().st_mtime
            for f in ("oracle.cpp", "portable_math.h", "tableaus_gen.h")):
        subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB_PATH))
        L.oracle_solve.restype = ctypes.c_int
        L.oracle_solve.argtypes = [ctypes.c_int, ctypes.c_longlong, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_void_p, ctypes.POINTER(OracleCfg), ctypes.c_void_p,
                                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_int]
        L.oracle_vern9_f64.restype = ctypes.c_longlong
        L.oracle_vern9_f64.argtypes = [ctypes.c_int, ctypes.c_longlong, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                       ctypes.c_double, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_int]
        L.oracle_rodas5p_f64.restype = ctypes.c_longlong
        L.oracle_rodas5p_f64.argtypes = L.oracle_vern9_f64.argtypes
        for fn in ("oracle_pm_powf", "oracle_pm_logf", "oracle_pm_expf"):
            getattr(L, fn).restype = ctypes.c_float
        L.oracle_pm_powf.argtypes = [ctypes.c_float, ctypes.c_float]
        L.oracle_pm_logf.argtypes = [ctypes.c_float]
        L.oracle_pm_expf.argtypes = [ctypes.c_float]
        L.oracle_normals4.argtypes = [ctypes.c_ulonglong, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, ctypes.c_void_p]
        L.oracle_philox4x32_10.argtypes = [ctypes.c_void_p, ctypes.c_uint, ctypes.c_uint, ctypes.c_void_p]
        L.oracle_model_dims.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
        _lib = L
    return _lib


def dims(model: str):
    n, p = ctypes.c_int(), ctypes.c_int()
    if lib().oracle_model_dims(MODEL[model], ctypes.byref(n), ctypes.byref(p)) != 0:
        raise ValueError(model)
    return n.value, p.value


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def solve(model: str, alg: str, u0, p, tspan, *, adaptive: bool, dt: float, L: int,
          saveat=None, save_everystep=False, abstol=1e-6, reltol=1e-3, time_f64=False,
          jac="ad", maxiters=10**7, seed=0, dt0=None, tolscale=None, nthreads=0, tstops=None, ccb=(),
          dcb=()):
    """Run the oracle ensemble.  u0 [B,N] f32, p [B,P] f32, tspan [B,2] f64 (or [2]).

    tstops: shared ascending stop times; ccb: continuous callbacks as tuples
    (fn, has_affect, has_affect_neg, rootfind 0 left / 1 right / 2 none, abstol, repeat_nudge,
    dtrelax); dcb: discrete callback function indices.

    Returns (ts [B,L] (f32|f64), us [B,L,N] f32, retcode [B] i8, naccept [B] i32, nreject [B] i32).
    """
    u0 = np.ascontiguousarray(u0, dtype=np.float32)
    B = u0.shape[0]
    p = np.ascontiguousarray(p, dtype=np.float32).reshape(B, -1)
    tspan = np.asarray(tspan, dtype=np.float64)
    if tspan.ndim == 1:
        tspan = np.broadcast_to(tspan, (B, 2))
    tspan = np.ascontiguousarray(tspan)
    N = u0.shape[1]
    cfg = OracleCfg()
    cfg.alg = ALG[alg]
    cfg.adaptive = int(adaptive)
    cfg.time_f64 = int(time_f64)
    cfg.save_everystep = int(save_everystep)
    cfg.L = L
    sa = None
    if saveat is not None:
        sa = np.ascontiguousarray(saveat, dtype=np.float64)
        cfg.nsaveat = sa.shape[-1]
        cfg.saveat_per_traj = int(sa.ndim == 2)
        cfg.saveat = sa.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    cfg.jac = JAC[jac]
    cfg.dt = dt
    cfg.abstol = abstol
    cfg.reltol = reltol
    cfg.maxiters = maxiters
    cfg.seed = seed
    d0 = ts_ = None
    if dt0 is not None:
        d0 = np.ascontiguousarray(dt0, dtype=np.float32)
        cfg.dt0 = d0.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    if tolscale is not None:
        ts_ = np.ascontiguousarray(tolscale, dtype=np.float32)
        cfg.tolscale = ts_.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    tst = None
    if tstops is not None and np.size(tstops):
        tst = np.ascontiguousarray(np.sort(np.asarray(tstops, dtype=np.float64).ravel()))
        cfg.ntstops = tst.size
        cfg.tstops = tst.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    if len(ccb) > 8 or len(dcb) > 8:
        raise ValueError("at most 8 callbacks of each kind")
    cfg.nccb = len(ccb)
    for j, (fn, aff, neg, rf, atol, nudge, relax) in enumerate(ccb):
        cfg.ccb_fn[j] = fn
        cfg.ccb_flags[j] = (1 if aff else 0) | (2 if neg else 0) | (int(rf) << 2)
        cfg.ccb_abstol[j] = atol
        cfg.ccb_nudge[j] = nudge
        cfg.ccb_dtrelax[j] = relax
    cfg.ndcb = len(dcb)
    for j, fn in enumerate(dcb):
        cfg.dcb_fn[j] = fn
    ts = np.zeros((B, L), dtype=np.float64 if time_f64 else np.float32)
    us = np.zeros((B, L, N), dtype=np.float32)
    rc = np.zeros(B, dtype=np.int8)
    na = np.zeros(B, dtype=np.int32)
    nr = np.zeros(B, dtype=np.int32)
    r = lib().oracle_solve(MODEL[model], B, _ptr(u0), _ptr(p), _ptr(tspan), ctypes.byref(cfg), _ptr(ts),
                           _ptr(us), _ptr(rc), _ptr(na), _ptr(nr), nthreads)
    if r != 0:
        raise ValueError(f"oracle_solve failed ({r})")
    return ts, us, rc, na, nr


def vern9(model: str, u0, p, t0, stops, *, rtol=1e-12, atol=1e-12, nthreads=0, method="vern9"):
    """FP64 Vern9 states at `stops` ([nstop] shared or [B,nstop] per trajectory) -> [B,nstop,N].

    method="rodas5p" selects the FP64 Rodas5P oracle for stiff problems."""
    u0 = np.ascontiguousarray(u0, dtype=np.float64)
    B, N = u0.shape
    p = np.ascontiguousarray(p, dtype=np.float64).reshape(B, -1)
    t0 = np.ascontiguousarray(np.broadcast_to(np.asarray(t0, dtype=np.float64), (B,)))
    stops = np.ascontiguousarray(stops, dtype=np.float64)
    per = int(stops.ndim == 2)
    nstop = stops.shape[-1]
    out = np.zeros((B, nstop, N), dtype=np.float64)
    steps = np.zeros(B, dtype=np.int64)
    fn = lib().oracle_vern9_f64 if method == "vern9" else lib().oracle_rodas5p_f64
    fails = fn(MODEL[model], B, _ptr(u0), _ptr(p), _ptr(t0), nstop, _ptr(stops), per,
                                   rtol, atol, _ptr(out), _ptr(steps), nthreads)
    if fails:
        raise RuntimeError(f"Vern9 oracle failed on {fails} trajectories")
    return out, steps


def normals4(seed: int, step: int, traj: int, blk: int):
    z = np.zeros(4, dtype=np.float32)
    lib().oracle_normals4(seed, step, traj, blk, _ptr(z))
    return z


def philox(ctr, key):
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    out = np.zeros(4, dtype=np.uint32)
    lib().oracle_philox4x32_10(_ptr(c), int(key[0]), int(key[1]), _ptr(out))
    return out


def pm_powf(x: float, y: float) -> float:
    return lib().oracle_pm_powf(x, y)


def nthreads_default() -> int:
    return len(os.sched_getaffinity(0))
