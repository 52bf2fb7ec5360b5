# DiffEqGPUNative.jl -- Julia binding of libdegpu (the GB300 EnsembleGPUKernel engine).
#
# Drop-in for DiffEqGPU.jl's lower-level kernel API: `vectorized_solve` /
# `vectorized_asolve` (src/ensemblegpukernel/lowerlevel_solve.jl:53-131, 253-346) keep their
# signatures and return device matrices (ts::CuMatrix{Tt}(L, B), us::CuMatrix{SVector{N,Float32}}(L, B)),
# so `batch_solve_up_kernel` (src/solve.jl:382-419) and `batch_solve` can call them unchanged.
# The right-hand side is CUDA C source (hand-written, or emitted from a trace of the Julia RHS);
# the engine JIT-compiles it with NVRTC for sm_103a together with the steppers.
#
# No Julia toolchain exists on the build machine, so this file is not exercised by the
# test suite; the C ABI it binds is (tests/test_abi.py, tests/test_gpu_parity.py).
module DiffEqGPUNative

using CUDA, StaticArrays

const libdegpu = joinpath(@__DIR__, "..", "degpu", "libdegpu.so")

struct Problems
    u0::Ptr{Float32}
    p::Ptr{Float32}
    tspan::Ptr{Cvoid}
    B::Clonglong
end

Base.@kwdef mutable struct Options
    alg::Cint = 0
    time_type::Cint = 0
    mode::Cint = 0
    driver::Cint = 0
    jac::Cint = 0
    save_everystep::Cint = 0
    nsaveat::Cint = 0
    saveat_per_traj::Cint = 0
    saveat::Ptr{Cvoid} = C_NULL
    dt::Cdouble = 0.1
    abstol::Cdouble = 1e-6
    reltol::Cdouble = 1e-3
    maxiters::Clonglong = 0
    dt0::Ptr{Float32} = C_NULL
    tolscale::Ptr{Float32} = C_NULL
    seed::Culonglong = 0
    traj_offset::Clonglong = 0
    block::Cint = 0
    chunk::Cint = 0
    ntstops::Cint = 0
    tstops::Ptr{Cvoid} = C_NULL          # CuArray of the time type (the `tstops` kwarg)
    callbacks::Ptr{Cvoid} = C_NULL       # Ref{Callbacks}, see below
    order::Ptr{Cint} = C_NULL            # optional CuArray{Cint} visiting order (degpu_work_order)
end

# GPUContinuousCallback fields the kernels use (callbacks.jl:34-124); the condition and
# affects are the CUDA C functions degpu_ccb_* of the right-hand side's source, chosen by fn.
struct ContinuousCallbackC
    fn::Cint
    has_affect::Cint
    has_affect_neg::Cint
    rootfind::Cint                       # 0 LeftRootFind, 1 RightRootFind, 2 NoRootFind
    abstol::Cdouble
    repeat_nudge::Cdouble
    dtrelax::Cdouble
end

struct Callbacks
    n_continuous::Cint
    continuous::Ptr{ContinuousCallbackC}
    n_discrete::Cint
    discrete::Ptr{Cint}                  # degpu_dcb_* function index of each GPUDiscreteCallback
end

struct Outputs
    ts::Ptr{Cvoid}
    us::Ptr{Float32}
    L::Cint
    retcode::Ptr{Int8}
    naccept::Ptr{Cint}
    nreject::Ptr{Cint}
    dt_first::Ptr{Float32}
end

const ALG = Dict(:GPUTsit5 => 0, :GPUVern7 => 1, :GPURosenbrock23 => 2, :GPURodas5P => 3, :GPURodas5 => 3, :GPUEM => 4)

function check(rc)
    rc == 0 && return nothing
    msg = unsafe_string(ccall((:degpu_last_error, libdegpu), Cstring, ()))
    error("degpu error $rc: $msg")
end

"""
    CudaRHS(source, N, P; jac=false, tgrad=false, noise=false)

A right-hand side written in CUDA C: `template <class T> __device__ void degpu_f(T* du,
const T* u, const float* p, T t)` (T is float or a forward-mode dual).
"""
mutable struct CudaRHS
    handle::Ptr{Cvoid}
    N::Int
    P::Int
    function CudaRHS(source::AbstractString, N::Integer, P::Integer; jac = false, tgrad = false, noise = false)
        h = Ref{Ptr{Cvoid}}(C_NULL)
        flags = (jac ? 1 : 0) | (tgrad ? 2 : 0) | (noise ? 4 : 0)
        check(ccall((:degpu_rhs_create, libdegpu), Cint, (Cstring, Cint, Cint, Cint, Ref{Ptr{Cvoid}}),
            source, N, P, flags, h))
        f = new(h[], N, P)
        finalizer(x -> ccall((:degpu_rhs_destroy, libdegpu), Cvoid, (Ptr{Cvoid},), x.handle), f)
        return f
    end
end

# flatten the isbits problem batch (make_prob_compatible + adapt) into SoA device arrays
function flatten(probs, ::Type{Tt}) where {Tt}
    u0 = CuArray(reduce(vcat, [Vector{Float32}(q.u0) for q in probs]))
    p = CuArray(reduce(vcat, [Vector{Float32}(q.p) for q in probs]))
    tspan = CuArray(reduce(vcat, [Tt[q.tspan[1], q.tspan[2]] for q in probs]))
    return u0, p, tspan
end

function _solve(f::CudaRHS, probs, alg::Symbol, adaptive::Bool; dt, saveat = nothing, save_everystep,
        abstol = 1.0f-6, reltol = 1.0f-3, Tt = Float32, mode = 0, driver = 0, maxiters = 0, seed = 0,
        order = nothing)
    B = length(probs)
    u0, p, tspan = flatten(probs, Tt)
    sa = saveat === nothing ? nothing : CuArray(Tt.(collect(saveat)))
    L = sa !== nothing ? length(sa) :
        save_everystep ? (adaptive ? ceil(Int, (probs[1].tspan[2] - probs[1].tspan[1]) / dt) + 1 :
                          length(probs[1].tspan[1]:dt:probs[1].tspan[2])) : 2
    ts = CUDA.fill(Tt(probs[1].tspan[1]), L, B)        # the reference pre-fills ts with tspan[1]
    us = CuArray{SVector{f.N, Float32}}(undef, L, B)    # same memory layout as [B][L][N]
    opt = Options(alg = ALG[alg], time_type = Tt === Float64 ? 1 : 0, mode = mode, driver = driver,
        save_everystep = save_everystep, nsaveat = sa === nothing ? 0 : length(sa),
        saveat = sa === nothing ? C_NULL : pointer(sa), dt = dt, abstol = abstol, reltol = reltol,
        maxiters = maxiters, seed = seed, order = order === nothing ? C_NULL : pointer(order))
    prs = Problems(pointer(u0), pointer(p), pointer(tspan), B)
    out = Outputs(pointer(ts), Ptr{Float32}(pointer(us)), L, C_NULL, C_NULL, C_NULL, C_NULL)
    fn = alg === :GPUEM ? :degpu_vectorized_solve_sde : adaptive ? :degpu_vectorized_asolve : :degpu_vectorized_solve
    check(ccall((fn, libdegpu), Cint, (Ptr{Cvoid}, Ref{Problems}, Ref{Options}, Ref{Outputs}, Ptr{Cvoid}),
        f.handle, prs, opt, out, CUDA.stream().handle))
    return ts, us
end

# Longest-first visiting order for the persistent driver from a per-trajectory work estimate
# (e.g. a work model's predicted attempts); pass it as `order` to vectorized_asolve.
function work_order(work::CuVector{Float32})
    order = CuVector{Cint}(undef, length(work))
    check(ccall((:degpu_work_order, libdegpu), Cint, (CuPtr{Float32}, Clonglong, CuPtr{Cint}, Ptr{Cvoid}),
        work, length(work), order, CUDA.stream().handle))
    return order
end

vectorized_solve(f::CudaRHS, probs, alg::Symbol; dt, saveat = nothing, save_everystep = true, kw...) =
    _solve(f, probs, alg, false; dt, saveat, save_everystep, kw...)
vectorized_asolve(f::CudaRHS, probs, alg::Symbol; dt = 0.1f0, saveat = nothing, save_everystep = false,
    abstol = 1.0f-6, reltol = 1.0f-3, kw...) =
    _solve(f, probs, alg, true; dt, saveat, save_everystep, abstol, reltol, kw...)

end # module
