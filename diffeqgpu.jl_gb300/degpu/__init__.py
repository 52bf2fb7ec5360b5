"""degpu -- GB300-native EnsembleGPUKernel engine (DiffEqGPU.jl's kernel path).

The solver kernels are hand-written CUDA for sm_103a, JIT-compiled together with the
user's CUDA C right-hand side by libdegpu.so (C ABI: include/degpu.h).  This package is
the Python mirror of the reference's interface; there is no CPU fallback.
"""
from ._lib import DegpuError, RETCODE_NAMES, lib  # noqa: F401
from .api import (  # noqa: F401
    CallbackSet, ContinuousCallback, DiscreteCallback, GPUContinuousCallback, GPUDiscreteCallback, LeftRootFind,
    NoRootFind, RightRootFind, DeviceProblems, EnsembleGPUKernel, EnsembleProblem, EnsembleSolution, GPUEM, GPUSIEA, GPUKvaerno3, GPUKvaerno5, GPURodas4, GPURodas5, GPURodas5P,
    GPURosenbrock23, GPUTsit5, GPUVern7, GPUVern9, LinRange, ODEFunction, ODEProblem, ODESolution, Range, SDEFunction,
    SDEProblem, adapt, alg_order, make_prob_compatible, normalize_saveat, remake, solve, vectorized_asolve,
    vectorized_solve,
)

__version__ = "0.1.0"
