"""Python mirror of DiffEqGPU.jl's EnsembleGPUKernel interface, on top of libdegpu.

Names, keyword arguments, defaults and errors follow the reference:
  solve(EnsembleProblem, GPUTsit5()|GPUVern7()|GPURosenbrock23()|GPURodas5P()|GPUEM(),
        EnsembleGPUKernel(dev); trajectories, batch_size, adaptive, dt, saveat,
        save_everystep, abstol, reltol)                    src/solve.jl:1-165, 174-287, 382-419
  vectorized_solve / vectorized_asolve                     src/ensemblegpukernel/lowerlevel_solve.jl
  make_prob_compatible                                     src/utils.jl:36-57
Device buffers are torch CUDA tensors (PyTorch is used only for device memory and
streams); all arithmetic runs in libdegpu's kernels.

Layout note: the reference returns ts::Matrix{Tt}(L, B) and us::Matrix{SVector{N}}(L, B)
(column i = trajectory i).  Here the same memory is a row-major tensor of shape (B, L)
and (B, L, N); `ts.T` indexes like the Julia matrix.
"""
from __future__ import annotations

import ctypes
import math
import time
from dataclasses import dataclass, field, replace
from typing import Any, Callable, Optional, Sequence

import numpy as np

from . import _lib
from ._lib import check, lib

# ---------------------------------------------------------------------- algorithms
# src/ensemblegpukernel/gpukernel_algorithms.jl; alg_order from alg_utils.jl:1-15


class GPUODEAlgorithm:
    alg_id = -1
    order = 0

    def __repr__(self):
        return f"{type(self).__name__}()"


class GPUODEImplicitAlgorithm(GPUODEAlgorithm):
    def __init__(self, autodiff: bool = True):
        self.autodiff = autodiff

    def __repr__(self):
        return f"{type(self).__name__}(autodiff={self.autodiff})"


class GPUSDEAlgorithm:
    alg_id = -1
    order = 0

    def __repr__(self):
        return f"{type(self).__name__}()"


class GPUTsit5(GPUODEAlgorithm):
    alg_id, order = _lib.ALG_TSIT5, 5


class GPUVern7(GPUODEAlgorithm):
    alg_id, order = _lib.ALG_VERN7, 7


class GPUVern9(GPUODEAlgorithm):
    alg_id, order = _lib.ALG_VERN9, 9


class GPURosenbrock23(GPUODEImplicitAlgorithm):
    alg_id, order = _lib.ALG_ROSENBROCK23, 2


class GPURodas5P(GPUODEImplicitAlgorithm):
    alg_id, order = _lib.ALG_RODAS5P, 5


class GPURodas4(GPUODEImplicitAlgorithm):
    alg_id, order = _lib.ALG_RODAS4, 4


class GPUKvaerno3(GPUODEImplicitAlgorithm):
    alg_id, order = _lib.ALG_KVAERNO3, 3


class GPUKvaerno5(GPUODEImplicitAlgorithm):
    alg_id, order = _lib.ALG_KVAERNO5, 5


# The reference has no Rodas5 (non-P) tableau; GPURodas5 is Rodas5P's coefficients.
GPURodas5 = GPURodas5P


class GPUEM(GPUSDEAlgorithm):
    alg_id, order = _lib.ALG_EM, 1


class GPUSIEA(GPUSDEAlgorithm):
    """Stochastic improved Euler, weak order 2, diagonal noise (gpu_siea_perform_step.jl)."""
    alg_id, order = _lib.ALG_SIEA, 2


def alg_order(alg) -> int:
    return alg.order


class EnsembleKernelAlgorithm:
    pass


class EnsembleGPUKernel(EnsembleKernelAlgorithm):
    """EnsembleGPUKernel(dev, cpu_offload=0.0) -- src/algorithms.jl:192-211.

    `dev` is a CUDA device index or torch device.  CPU offloading is not provided: the
    kernels are the only execution path (cpu_offload must be 0)."""

    def __init__(self, dev: Any = 0, cpu_offload: float = 0.0):
        if cpu_offload != 0.0:
            raise NotImplementedError("EnsembleGPUKernel here has no CPU offload path (cpu_offload must be 0.0)")
        self.dev = dev
        self.cpu_offload = cpu_offload

    def device(self):
        import torch
        d = self.dev
        if isinstance(d, int):
            return torch.device("cuda", d)
        return torch.device(d)


# ---------------------------------------------------------------------- functions and problems
class ODEFunction:
    """A right-hand side written in CUDA C (see include/degpu.h, degpu_rhs_create).

    ODEFunction(source, nstate, nparam, jac=False, tgrad=False, noise=False, mass_matrix=False)
    ODEFunction.builtin("lorenz")

    mass_matrix=True: the source defines degpu_mass(float* M), the constant mass matrix
    (ODEFunction's mass_matrix keyword; Rosenbrock methods only).
    """

    def __init__(self, source: str, nstate: int, nparam: int, *, jac: bool = False, tgrad: bool = False,
                 noise: bool = False, mass_matrix: bool = False, name: str = "user"):
        self.source = source
        self.nstate = int(nstate)
        self.nparam = int(nparam)
        self.flags = (_lib.RHS_HAS_JAC if jac else 0) | (_lib.RHS_HAS_TGRAD if tgrad else 0) | \
                     (_lib.RHS_HAS_NOISE if noise else 0) | (_lib.RHS_HAS_MASS if mass_matrix else 0)
        self.name = name
        self._handle = None

    @classmethod
    def builtin(cls, name: str) -> "ODEFunction":
        n, p, fl = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        src = lib().degpu_builtin_rhs(name.encode(), ctypes.byref(n), ctypes.byref(p), ctypes.byref(fl))
        if src is None:
            raise KeyError(f"unknown built-in model {name!r}")
        f = cls(src.decode(), n.value, p.value, name=name)
        f.flags = fl.value
        return f

    @property
    def has_jac(self):
        return bool(self.flags & _lib.RHS_HAS_JAC)

    @property
    def has_tgrad(self):
        return bool(self.flags & _lib.RHS_HAS_TGRAD)

    def handle(self):
        if self._handle is None:
            h = ctypes.c_void_p()
            check(lib().degpu_rhs_create(self.source.encode(), self.nstate, self.nparam, self.flags, ctypes.byref(h)))
            self._handle = h
        return self._handle

    def __del__(self):
        try:
            if self._handle is not None and _lib._lib is not None:
                _lib._lib.degpu_rhs_destroy(self._handle)
        except Exception:
            pass


SDEFunction = ODEFunction


def _time_dtype(tt):
    if tt in (np.float32, "float32", "Float32", 32):
        return np.float32
    if tt in (np.float64, "float64", "Float64", 64, float):
        return np.float64
    raise ValueError(f"time type must be float32 or float64, got {tt!r}")


@dataclass
class ODEProblem:
    """ODEProblem{false}(f, u0, tspan, p; saveat) with a CUDA C right-hand side.

    time_type is eltype(tspan): float32 reproduces the reference's Float32 runs; float64
    keeps FP64 time with FP32 state."""
    f: ODEFunction
    u0: Any
    tspan: Any
    p: Any = ()
    time_type: Any = np.float32
    kwargs: dict = field(default_factory=dict)
    seed: int = 0

    def __post_init__(self):
        self.time_type = _time_dtype(self.time_type)
        self.u0 = np.asarray(self.u0, dtype=np.float32).reshape(-1)
        self.p = np.asarray(self.p, dtype=np.float32).reshape(-1)
        self.tspan = np.asarray(self.tspan, dtype=self.time_type).reshape(2)
        if self.u0.shape[0] != self.f.nstate:
            raise ValueError(f"u0 has {self.u0.shape[0]} states, the right-hand side {self.f.nstate}")
        if self.p.shape[0] != self.f.nparam:
            raise ValueError(f"p has {self.p.shape[0]} entries, the right-hand side {self.f.nparam}")


@dataclass
class SDEProblem(ODEProblem):
    """SDEProblem(f, g, u0, tspan, p; seed): `f` carries both drift and diagonal noise."""


def remake(prob: ODEProblem, **kw) -> ODEProblem:
    return replace(prob, **kw)


def make_prob_compatible(prob):
    """src/utils.jl:36-40: the immutable, kernel-ready form (here: validated copy)."""
    return replace(prob)


def EnsembleContext(i, sim_seed=None):
    return {"sim_id": i, "sim_seed": sim_seed}


@dataclass
class EnsembleProblem:
    """EnsembleProblem(prob; prob_func, output_func, reduction, u_init, safetycopy).

    prob_func(prob, ctx) -> prob is called once per trajectory (src/solve.jl:186-202).
    reduction(u, batch, I) -> (u, converged) folds each batch of (output_func-mapped)
    solutions into u, starting from u_init (src/solve.jl:97-164).  For large ensembles,
    EnsembleProblem.from_arrays builds the batch in bulk."""
    prob: ODEProblem
    prob_func: Optional[Callable] = None
    output_func: Optional[Callable] = None
    safetycopy: bool = False
    arrays: Optional[dict] = None
    reduction: Optional[Callable] = None
    u_init: Any = None

    @classmethod
    def from_arrays(cls, prob: ODEProblem, *, u0=None, p=None, tspan=None, saveat=None):
        """Bulk construction: per-trajectory u0 [B,N], p [B,P], tspan [B,2], saveat [B,L]
        (any may be None to reuse prob's)."""
        return cls(prob, arrays={"u0": u0, "p": p, "tspan": tspan, "saveat": saveat})


# ---------------------------------------------------------------------- saveat normalisation
class Range:
    """Julia's `start:step:stop` for floats (elements start + i*step, i = 0..len-1)."""

    def __init__(self, start, step, stop):
        self.start, self.step, self.stop = float(start), float(step), float(stop)

    def __len__(self):
        n = (self.stop - self.start) / self.step
        return max(0, int(math.floor(n + 1e-10 * max(1.0, abs(n)))) + 1)

    def collect(self):
        return self.start + np.arange(len(self), dtype=np.float64) * self.step

    def first(self):
        return self.start

    def last(self):
        return self.start + (len(self) - 1) * self.step


def LinRange(start, stop, length):
    """range(start, stop, length=n)"""
    if length == 1:
        return np.array([float(start)])
    i = np.arange(length, dtype=np.float64)
    return (float(start) * (length - 1 - i) + float(stop) * i) / (length - 1)


MAX_SAVEAT_LENGTH = 100_000


def normalize_saveat(saveat, tspan, Tt, adaptive: bool):
    """Saveat normalisation of lowerlevel_solve.jl:88-102 (fixed) and :271-306 (adaptive).
    Returns a Tt numpy vector or None."""
    if saveat is None:
        return None
    t0, tf = (Tt(tspan[0]), Tt(tspan[1]))
    if np.isscalar(saveat):
        if Tt(saveat) == Tt(0.0):
            return np.array([t0, tf], dtype=Tt)
        num_points = int(math.ceil(float(abs(Tt(tf - t0)) / abs(Tt(saveat))))) + 1
        if adaptive and num_points > MAX_SAVEAT_LENGTH:
            raise ValueError(f"saveat would create too many save points ({num_points}). "
                             "Consider using a larger saveat value.")
        return LinRange(float(t0), float(tf), num_points).astype(Tt)
    if isinstance(saveat, Range):
        if adaptive:
            return saveat.collect().astype(Tt)
        return LinRange(float(Tt(saveat.first())), float(Tt(saveat.last())), len(saveat)).astype(Tt)
    if isinstance(saveat, range):
        return np.asarray(list(saveat), dtype=np.float64).astype(Tt)
    return np.asarray(saveat, dtype=np.float64).astype(Tt)


# ---------------------------------------------------------------------- callbacks
LeftRootFind, RightRootFind, NoRootFind = "LeftRootFind", "RightRootFind", "NoRootFind"
_ROOTFIND = {LeftRootFind: _lib.ROOTFIND_LEFT, RightRootFind: _lib.ROOTFIND_RIGHT, NoRootFind: _lib.ROOTFIND_NONE}
_SAVE_POS_MSG = ("Callback `save_positions` are incompatible with kernel-based GPU ODE solvers due requiring static "
                 "sizing. Please ensure `save_positions = (false,false)` is set in all callback definitions used "
                 "with such solvers.")


class ContinuousCallback:
    """GPUContinuousCallback (src/ensemblegpukernel/callbacks.jl:34-124).

    The condition and affects are CUDA C functions of the ODEFunction's source,
    `degpu_ccb_condition(fn, u, p, t)`, `degpu_ccb_affect(fn, I)` and
    `degpu_ccb_affect_neg(fn, I)`; `fn` selects which one.  `affect=False` stands for
    `affect! = nothing` and `affect_neg=False` for `affect_neg! = nothing`; by default
    affect_neg! is present exactly when affect! is (`affect_neg! = affect!`).  abstol defaults
    to 100 eps(Float32), the value a ContinuousCallback gets when converted for the kernels
    (callbacks.jl:112-119)."""

    default_abstol = 100 * float(np.finfo(np.float32).eps)

    def __init__(self, fn: int = 0, affect: bool = True, affect_neg=None, *, rootfind=LeftRootFind,
                 save_positions=(False, False), interp_points=10, dtrelax=1.0, abstol=None, reltol=0.0,
                 repeat_nudge=0.01):
        if tuple(save_positions) != (False, False):
            raise ValueError(_SAVE_POS_MSG)
        if rootfind not in _ROOTFIND:
            raise ValueError(f"rootfind must be one of {list(_ROOTFIND)}")
        self.fn = int(fn)
        self.affect = bool(affect)
        self.affect_neg = self.affect if affect_neg is None else bool(affect_neg)
        self.rootfind = rootfind
        self.save_positions = (False, False)
        self.interp_points = interp_points
        self.dtrelax = float(dtrelax)
        self.abstol = self.default_abstol if abstol is None else float(abstol)
        self.reltol = reltol
        self.repeat_nudge = float(repeat_nudge)


class GPUContinuousCallback(ContinuousCallback):
    """The kernels' own constructor: abstol defaults to 10 eps(Float32) (callbacks.jl:94-103)."""
    default_abstol = 10 * float(np.finfo(np.float32).eps)


class DiscreteCallback:
    """GPUDiscreteCallback (callbacks.jl:1-32): `degpu_dcb_condition(fn, u, p, t)` and
    `degpu_dcb_affect(fn, I)` of the ODEFunction's source."""

    def __init__(self, fn: int = 0, *, save_positions=(False, False)):
        if tuple(save_positions) != (False, False):
            raise ValueError(_SAVE_POS_MSG)
        self.fn = int(fn)
        self.save_positions = (False, False)


GPUDiscreteCallback = DiscreteCallback


class CallbackSet:
    """CallbackSet(cb...): continuous and discrete members in order (nested sets flatten)."""

    def __init__(self, *cbs):
        self.continuous, self.discrete = [], []
        for c in cbs:
            if c is None:
                continue
            if isinstance(c, CallbackSet):
                self.continuous += c.continuous
                self.discrete += c.discrete
            elif isinstance(c, ContinuousCallback):
                self.continuous.append(c)
            elif isinstance(c, DiscreteCallback):
                self.discrete.append(c)
            else:
                raise TypeError(f"not a GPU callback: {c!r}")
        if len(self.continuous) > _lib.MAX_CALLBACKS or len(self.discrete) > _lib.MAX_CALLBACKS:
            raise ValueError(f"at most {_lib.MAX_CALLBACKS} continuous and {_lib.MAX_CALLBACKS} discrete callbacks")

    def cstruct(self):
        """(degpu_callbacks, keep-alive) for the C ABI."""
        nc, nd = len(self.continuous), len(self.discrete)
        carr = (_lib.ContinuousCallbackC * max(nc, 1))()
        for j, c in enumerate(self.continuous):
            carr[j] = _lib.ContinuousCallbackC(c.fn, int(c.affect), int(c.affect_neg), _ROOTFIND[c.rootfind],
                                               c.abstol, c.repeat_nudge, c.dtrelax)
        darr = (ctypes.c_int * max(nd, 1))(*[d.fn for d in self.discrete])
        st = _lib.CallbacksC(nc, ctypes.cast(carr, ctypes.POINTER(_lib.ContinuousCallbackC)), nd,
                             ctypes.cast(darr, ctypes.POINTER(ctypes.c_int)))
        return st, (carr, darr)


def as_callback_set(callback):
    if callback is None:
        return None
    cs = callback if isinstance(callback, CallbackSet) else CallbackSet(callback)
    return cs if (cs.continuous or cs.discrete) else None


def tstops_extra_length(tspan, dt, tstops, Tt) -> int:
    """length(tstops) - count(x -> x in tstops, t0:dt:tf) (lowerlevel_solve.jl:73-77)."""
    t0, tf = float(Tt(tspan[0])), float(Tt(tspan[1]))
    n = fixed_step_length(tspan, dt, Tt)
    grid = np.asarray([Tt(t0 + k * float(Tt(dt))) for k in range(n)], dtype=Tt)
    ts = np.asarray(tstops, dtype=Tt)
    return int(ts.size - np.isin(grid, ts).sum())


def fixed_step_length(tspan, dt, Tt) -> int:
    """length(tspan[1]:dt:tspan[2]) (lowerlevel_solve.jl:73)."""
    t0, tf, dt = float(Tt(tspan[0])), float(Tt(tspan[1])), float(Tt(dt))
    n = (tf - t0) / dt
    r = round(n)
    if abs(n - r) <= 1e-6 * max(1.0, abs(n)):
        return int(r) + 1
    return int(math.floor(n)) + 1


# ---------------------------------------------------------------------- device batches
class DeviceProblems:
    """`adapt(backend, probs)`: the flattened problem batch in device memory."""

    def __init__(self, f: ODEFunction, u0, p, tspan, Tt, device, saveat=None, kind="ode"):
        import torch
        self.f = f
        self.Tt = Tt
        self.kind = kind
        tdt = torch.float32 if Tt == np.float32 else torch.float64
        def dev_array(a, dt):  # contiguous, writable host copy only when needed (read-only views warn)
            a = np.ascontiguousarray(a, dtype=dt)
            return torch.as_tensor(a if a.flags.writeable else a.copy(), device=device)
        self.u0 = dev_array(u0, np.float32)
        self.p = dev_array(p, np.float32)
        self.tspan = dev_array(tspan, Tt).to(tdt)
        self.saveat = None if saveat is None else dev_array(saveat, Tt)
        self.B = self.u0.shape[0]

    def __len__(self):
        return self.B

    def cstruct(self):
        return _lib.Problems(self.u0.data_ptr(), self.p.data_ptr() if self.p.numel() else None,
                             self.tspan.data_ptr(), self.B)


def adapt(device, probs: Sequence[ODEProblem]) -> DeviceProblems:
    """adapt(backend, probs): flatten a vector of compatible problems onto the device."""
    if not probs:
        raise ValueError("empty problem batch")
    f = probs[0].f
    Tt = probs[0].time_type
    u0 = np.stack([q.u0 for q in probs])
    p = np.stack([q.p for q in probs]) if f.nparam else np.zeros((len(probs), 0), np.float32)
    tsp = np.stack([q.tspan for q in probs]).astype(Tt)
    sa = [q.kwargs.get("saveat") for q in probs]
    saveat = None
    if sa[0] is not None:
        saveat = np.stack([np.asarray(s, dtype=Tt) for s in sa])
    return DeviceProblems(f, u0, p, tsp, Tt, _torch_device(device), saveat,
                          kind="sde" if isinstance(probs[0], SDEProblem) else "ode")


def _torch_device(dev):
    import torch
    if isinstance(dev, EnsembleGPUKernel):
        return dev.device()
    if isinstance(dev, int):
        return torch.device("cuda", dev)
    return torch.device(dev)


def _options(alg, Tt, *, dt, abstol=1e-6, reltol=1e-3, save_everystep=False, saveat_dev=None, nsaveat=0,
             per_traj=False, mode="fast", driver="auto", maxiters=0, dt0=None, tolscale=None, seed=0,
             traj_offset=0, block=0, chunk=0, jac="auto", tstops_dev=None, ntstops=0, callbacks_ptr=None,
             order=None):
    o = _lib.Options()
    o.alg = alg.alg_id
    o.time_type = _lib.TIME_F64 if Tt == np.float64 else _lib.TIME_F32
    o.mode = {"fast": _lib.MODE_FAST, "parity": _lib.MODE_PARITY}[mode]
    o.driver = {"auto": _lib.DRIVER_AUTO, "naive": _lib.DRIVER_NAIVE, "persistent": _lib.DRIVER_PERSISTENT}[driver]
    if jac == "auto" and isinstance(alg, GPUODEImplicitAlgorithm) and not alg.autodiff:
        jac = "finitediff_if_no_jac"
    o.jac = {"auto": _lib.JAC_AUTO, "ad": _lib.JAC_AD, "finitediff": _lib.JAC_FINITEDIFF,
             "finitediff_if_no_jac": _lib.JAC_AUTO}[jac]
    o.save_everystep = int(bool(save_everystep))
    o.nsaveat = nsaveat
    o.saveat_per_traj = int(per_traj)
    o.saveat = saveat_dev
    o.dt = float(dt)
    o.abstol = float(abstol)
    o.reltol = float(reltol)
    o.maxiters = int(maxiters)
    o.dt0 = dt0
    o.tolscale = tolscale
    o.seed = int(seed)
    o.traj_offset = int(traj_offset)
    o.block = int(block)
    o.chunk = int(chunk)
    o.ntstops = int(ntstops)
    o.tstops = tstops_dev
    o.callbacks = callbacks_ptr
    o.order = order
    return o


@dataclass
class KernelResult:
    ts: Any        # torch (B, L) Tt
    us: Any        # torch (B, L, N) f32
    retcode: Any   # torch (B,) int8
    naccept: Any   # torch (B,) int32
    nreject: Any   # torch (B,) int32
    dt_first: Any = None  # torch (B,) f32: first accepted dt (trace=True)


def _solve_device(probs: DeviceProblems, alg, adaptive: bool, *, dt, saveat=None, save_everystep=None,
                  abstol=1e-6, reltol=1e-3, stream=None, stats=True, trace=False, callback=None, tstops=None,
                  **kw) -> KernelResult:
    import torch
    f = probs.f
    Tt = probs.Tt
    dev = probs.u0.device
    if isinstance(alg, GPUSDEAlgorithm) and adaptive:
        raise NotImplementedError("Adaptive time-stepping is not supported yet with GPUEM.")
    if save_everystep is None:
        save_everystep = not adaptive  # vectorized_solve defaults true, vectorized_asolve false
    if probs.B == 0:  # empty ensemble: nothing to launch
        tdt = torch.float32 if Tt == np.float32 else torch.float64
        z = lambda *s, dt=torch.float32: torch.zeros(s, dtype=dt, device=dev)
        return KernelResult(z(0, 2, dt=tdt), z(0, 2, f.nstate), z(0, dt=torch.int8), z(0, dt=torch.int32),
                            z(0, dt=torch.int32), None)
    tsp0 = probs.tspan[0].cpu().numpy().astype(Tt)
    per_traj = probs.saveat is not None
    if per_traj:
        sa_dev = probs.saveat
        L = sa_dev.shape[1]
    else:
        sa = normalize_saveat(saveat, tsp0, Tt, adaptive)
        sa_dev = None if sa is None else torch.as_tensor(sa, device=dev)
        if sa is None:
            if save_everystep:
                L = fixed_step_length(tsp0, dt, Tt) if not adaptive else \
                    int(math.ceil(float(Tt(tsp0[1]) - Tt(tsp0[0])) / float(Tt(dt)))) + 1
                if tstops is not None and not adaptive:
                    L += tstops_extra_length(tsp0, dt, tstops, Tt)
            else:
                L = 2
        else:
            L = sa.shape[0]
    B = probs.B
    tdt = torch.float32 if Tt == np.float32 else torch.float64
    ts = torch.empty((B, L), dtype=tdt, device=dev)
    us = torch.empty((B, L, f.nstate), dtype=torch.float32, device=dev)
    rc = torch.zeros(B, dtype=torch.int8, device=dev)
    na = torch.zeros(B, dtype=torch.int32, device=dev) if stats else None
    nr = torch.zeros(B, dtype=torch.int32, device=dev) if stats else None
    dtf = torch.zeros(B, dtype=torch.float32, device=dev) if trace else None
    dt0 = kw.pop("dt0", None)
    tolscale = kw.pop("tolscale", None)
    order = kw.pop("order", None)
    step_model = kw.pop("step_model", None)  # learned controller (degpu.learned.StepSizeModel)
    work_model = kw.pop("work_model", None)  # learned visiting order (degpu.learned.fit_work_model)
    ts_dev = None
    if tstops is not None and np.size(tstops):
        ts_dev = torch.as_tensor(np.sort(np.asarray(tstops, dtype=Tt).ravel()), device=dev)
    cbs = as_callback_set(callback)
    cb_struct = cb_keep = None
    if cbs is not None:
        cb_struct, cb_keep = cbs.cstruct()
    opt = _options(alg, Tt, dt=dt, abstol=abstol, reltol=reltol, save_everystep=save_everystep,
                   saveat_dev=None if sa_dev is None else sa_dev.data_ptr(),
                   nsaveat=0 if sa_dev is None else L, per_traj=per_traj,
                   dt0=None if dt0 is None else dt0.data_ptr(),
                   tolscale=None if tolscale is None else tolscale.data_ptr(),
                   order=None if order is None else order.data_ptr(),
                   tstops_dev=None if ts_dev is None else ts_dev.data_ptr(),
                   ntstops=0 if ts_dev is None else ts_dev.numel(),
                   callbacks_ptr=None if cb_struct is None else ctypes.addressof(cb_struct), **kw)
    out = _lib.Outputs(ts.data_ptr(), us.data_ptr(), L, rc.data_ptr(), None if na is None else na.data_ptr(),
                       None if nr is None else nr.data_ptr(), None if dtf is None else dtf.data_ptr())
    st = stream if stream is not None else torch.cuda.current_stream(dev)
    pr = probs.cstruct()
    with torch.cuda.device(dev):
        if step_model is not None or work_model is not None:
            if not adaptive or isinstance(alg, GPUSDEAlgorithm):
                raise ValueError("step and work models apply to adaptive ODE solves")
            lo, hi = step_model.dt_range if step_model is not None else (1e-8, 1e3)
            smax = step_model.scale_range[1] if step_model is not None else 1.0
            check(lib().degpu_learned_asolve_ex(f.handle(), None if step_model is None else step_model.h,
                                                None if work_model is None else work_model.h, ctypes.byref(pr),
                                                ctypes.byref(opt), lo, hi, smax, ctypes.byref(out),
                                                ctypes.c_void_p(st.cuda_stream)))
            return KernelResult(ts, us, rc, na, nr, dtf)
        if isinstance(alg, GPUSDEAlgorithm):
            fn = lib().degpu_vectorized_solve_sde
        elif adaptive:
            fn = lib().degpu_vectorized_asolve
        else:
            fn = lib().degpu_vectorized_solve
        check(fn(f.handle(), ctypes.byref(pr), ctypes.byref(opt), ctypes.byref(out), ctypes.c_void_p(st.cuda_stream)))
    return KernelResult(ts, us, rc, na, nr, dtf)


def vectorized_solve(probs: DeviceProblems, prob: ODEProblem, alg, *, dt, saveat=None, save_everystep=True,
                     debug=False, callback=None, tstops=None, **kw):
    """Fixed-step batched solve (lowerlevel_solve.jl:53-131, 134-199).  Returns device (ts, us)."""
    r = _solve_device(probs, alg, False, dt=dt, saveat=saveat, save_everystep=save_everystep, callback=callback,
                      tstops=tstops, **kw)
    return r.ts, r.us


def vectorized_asolve(probs: DeviceProblems, prob: ODEProblem, alg, *, dt=0.1, saveat=None, save_everystep=False,
                      abstol=1.0e-6, reltol=1.0e-3, debug=False, callback=None, tstops=None, **kw):
    """Adaptive batched solve (lowerlevel_solve.jl:253-346).  Returns device (ts, us)."""
    if isinstance(alg, GPUSDEAlgorithm):
        raise NotImplementedError("Adaptive time-stepping is not supported yet with GPUEM.")
    r = _solve_device(probs, alg, True, dt=dt, saveat=saveat, save_everystep=save_everystep,
                      abstol=abstol, reltol=reltol, callback=callback, tstops=tstops, **kw)
    return r.ts, r.us


# ---------------------------------------------------------------------- solutions
RETCODE_SUCCESS, RETCODE_TERMINATED = "Success", "Terminated"


@dataclass
class ODESolution:
    t: Any
    u: Any
    prob: Any = None
    alg: Any = None
    retcode: str = RETCODE_SUCCESS


class _LazySolutions(Sequence):
    """Per-trajectory ODESolution views built on demand (the reference builds them eagerly
    in a host loop, src/solve.jl:256-283)."""

    def __init__(self, ts, us, t0, alg, output_func, probs_kind, offset=0):
        self.ts, self.us, self.t0, self.alg, self.output_func = ts, us, t0, alg, output_func
        self.offset = offset  # global index of row 0 (EnsembleContext sim_id)

    def __len__(self):
        return self.ts.shape[0]

    def __getitem__(self, i):
        if isinstance(i, slice):
            return [self[j] for j in range(*i.indices(len(self)))]
        if i < 0:
            i += len(self)
        ts = self.ts[i]
        nz = np.nonzero(ts != self.t0[i])[0]
        if nz.size == 0:
            raise RuntimeError("Batch solve failed")
        idx = nz[-1] + 1
        sol = ODESolution(ts[:idx], self.us[i, :idx], alg=self.alg,
                          retcode=RETCODE_SUCCESS if idx == ts.shape[0] else RETCODE_TERMINATED)
        if self.output_func is not None:
            return self.output_func(sol, EnsembleContext(self.offset + i))[0]
        return sol


@dataclass
class EnsembleSolution:
    u: Any
    elapsedTime: float
    converged: bool = True
    ts: Any = None          # (B, L) host arrays of the whole ensemble
    us: Any = None          # (B, L, N)
    retcodes: Any = None    # per-trajectory engine retcodes
    naccept: Any = None
    nreject: Any = None

    def __len__(self):
        return len(self.u)


def _build_batch(ens: EnsembleProblem, I: range):
    prob = ens.prob
    Tt = prob.time_type
    if ens.arrays is not None:
        a = ens.arrays
        B = len(I)

        def pick(x, default, shape):
            if x is None:
                return np.broadcast_to(default, (B,) + default.shape)
            return np.asarray(x)[I.start:I.stop]
        u0 = pick(a["u0"], prob.u0, None)
        p = pick(a["p"], prob.p, None)
        tsp = pick(a["tspan"], prob.tspan, None).astype(Tt)
        sa = None if a.get("saveat") is None else np.asarray(a["saveat"])[I.start:I.stop].astype(Tt)
        return u0, p, tsp, sa
    probs = []
    for i in I:
        q = ens.prob_func(remake(prob) if ens.safetycopy else prob, EnsembleContext(i)) if ens.prob_func else prob
        probs.append(make_prob_compatible(q))
    # src/solve.jl:206-245: all tspans equal, or equal-length saveats
    u0 = np.stack([q.u0 for q in probs])
    p = np.stack([q.p for q in probs]) if prob.f.nparam else np.zeros((len(probs), 0), np.float32)
    tsp = np.stack([q.tspan for q in probs]).astype(Tt)
    sas = [q.kwargs.get("saveat") for q in probs]
    sa = None
    if sas[0] is not None:
        if len({np.size(s) for s in sas}) != 1:
            raise ValueError("Using different saveat in EnsembleGPUKernel requires all of them to be of same length. "
                             "Use saveats of same size only.")
        sa = np.stack([np.asarray(s, dtype=Tt) for s in sas])
    return u0, p, tsp, sa


def solve(ens: EnsembleProblem, alg, ensemblealg: EnsembleGPUKernel, *, trajectories: int, batch_size=None,
          adaptive: bool = True, dt=None, saveat=None, save_everystep=None, abstol=1.0e-6, reltol=1.0e-3,
          callback=None, tstops=None, unstable_check=None, merge_callbacks=True, **kw) -> EnsembleSolution:
    """SciMLBase.solve for EnsembleGPUKernel (src/solve.jl:1-165, 174-287, 382-419)."""
    import torch
    if not isinstance(ensemblealg, EnsembleGPUKernel):
        raise TypeError("ensemblealg must be EnsembleGPUKernel")
    if isinstance(alg, GPUSDEAlgorithm) and adaptive:
        raise NotImplementedError("Adaptive EM is not supported yet.")
    if dt is None:
        if adaptive:
            dt = 0.1
        else:
            raise ValueError("dt is required for fixed time stepping")
    if batch_size is None:
        batch_size = trajectories
    dev = ensemblealg.device()
    prob = ens.prob
    Tt = prob.time_type
    if save_everystep is None:
        save_everystep = False if adaptive else True
    tstart = time.perf_counter()
    parts, t0s = [], []
    if ens.reduction is not None:
        # solve.jl:97-164: each batch is solved, turned into its solutions and folded into u
        u = [] if ens.u_init is None else ens.u_init
        converged = False
        for b0 in range(0, trajectories, batch_size):
            I = range(b0, min(trajectories, b0 + batch_size))
            u0, p, tsp, sa = _build_batch(ens, I)
            dp = DeviceProblems(prob.f, u0, p, tsp, Tt, dev, sa)
            r = _solve_device(dp, alg, adaptive, dt=dt, saveat=saveat, save_everystep=save_everystep,
                              abstol=abstol, reltol=reltol, traj_offset=b0, callback=callback, tstops=tstops, **kw)
            torch.cuda.synchronize(dev)
            ts_b = r.ts.cpu().numpy()
            sols = _LazySolutions(ts_b, r.us.cpu().numpy(), np.asarray(tsp)[:, 0].astype(ts_b.dtype), alg,
                                  ens.output_func, "ode", offset=b0)
            u, converged = ens.reduction(u, [sols[j] for j in range(len(sols))], I)
        return EnsembleSolution(u, time.perf_counter() - tstart, True)
    for b0 in range(0, trajectories, batch_size):
        I = range(b0, min(trajectories, b0 + batch_size))
        u0, p, tsp, sa = _build_batch(ens, I)
        if sa is None and saveat is None and not np.all(tsp == tsp[0]):
            if not adaptive and save_everystep:
                raise ValueError("Using different time-spans require either turning off save_everystep or using "
                                 "saveat. If using saveat, it should be of same length across the ensemble.")
        t0s.append(np.asarray(tsp)[:, 0])
        dp = DeviceProblems(prob.f, u0, p, tsp, Tt, dev, sa)
        r = _solve_device(dp, alg, adaptive, dt=dt, saveat=saveat, save_everystep=save_everystep,
                          abstol=abstol, reltol=reltol, traj_offset=b0, callback=callback, tstops=tstops, **kw)
        parts.append(r)
    # gather: one page-locked host array per output, each batch copied into its rows with an
    # asynchronous device-to-host copy (no per-batch host arrays, no concatenation)
    def gather(name):
        first = getattr(parts[0], name)
        host = torch.empty((trajectories,) + tuple(first.shape[1:]), dtype=first.dtype, pin_memory=True)
        row = 0
        for r in parts:
            a = getattr(r, name)
            host[row:row + a.shape[0]].copy_(a, non_blocking=True)
            row += a.shape[0]
        return host
    ts_h, us_h, rc_h, na_h, nr_h = (gather(n) for n in ("ts", "us", "retcode", "naccept", "nreject"))
    torch.cuda.synchronize(dev)
    ts, us, rc, na, nr = (x.numpy() for x in (ts_h, us_h, rc_h, na_h, nr_h))
    elapsed = time.perf_counter() - tstart
    t0 = np.concatenate(t0s).astype(ts.dtype)
    sols = _LazySolutions(ts, us, t0, alg, ens.output_func, "ode")
    return EnsembleSolution(sols, elapsed, True, ts, us, rc, na, nr)
