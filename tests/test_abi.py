"""C-ABI surface and host logic without a GPU: the library loads, exports every symbol
include/degpu.h declares, JIT-compiles kernels with NVRTC, validates arguments like the
reference, and the host-side saveat / sizing / batching logic follows lowerlevel_solve.jl."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def header_symbols():
    text = (ROOT / "include" / "degpu.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(degpu_\w+)\s*\(", text)))


def test_library_exports_every_header_symbol(degpu_mod):
    L = degpu_mod.lib()
    syms = header_symbols()
    assert len(syms) >= 17
    for s in syms:
        assert hasattr(L, s), f"libdegpu.so does not export {s}"
    from degpu import _lib
    assert set(syms) <= set(_lib.SIGNATURES), set(syms) - set(_lib.SIGNATURES)


def test_struct_layouts_match_the_library(degpu_mod):
    """The ctypes mirrors of the ABI structs have the library's sizes."""
    from degpu import _lib
    v = [ctypes.c_int() for _ in range(5)]
    degpu_mod.lib().degpu_abi_struct_sizes(*[ctypes.byref(x) for x in v])
    mine = [_lib.Options, _lib.Outputs, _lib.Problems, _lib.ContinuousCallbackC, _lib.CallbacksC]
    assert [x.value for x in v] == [ctypes.sizeof(t) for t in mine]


def test_nvrtc_compiles_callback_kernels(degpu_mod):
    """Kernels with tstops and continuous / discrete callback sets compile for every
    algorithm (bouncing ball, decay with discrete events)."""
    from degpu import _lib
    n = ctypes.c_longlong()
    for model, cs in (("ball", degpu_mod.CallbackSet(degpu_mod.ContinuousCallback(0), degpu_mod.ContinuousCallback(1))),
                      ("decay", degpu_mod.CallbackSet(degpu_mod.DiscreteCallback(0), degpu_mod.DiscreteCallback(2)))):
        f = degpu_mod.ODEFunction.builtin(model)
        st, keep = cs.cstruct()
        for alg in ("GPUTsit5", "GPUVern7", "GPURosenbrock23", "GPURodas5P", "GPURodas4", "GPUVern9", "GPUKvaerno3", "GPUKvaerno5"):
            for adaptive in (0, 1):
                o = _opts(degpu_mod, getattr(degpu_mod, alg)(), tt=np.float32, mode="parity")
                o.callbacks = ctypes.addressof(st)
                _lib.check(degpu_mod.lib().degpu_rhs_check(f.handle(), ctypes.byref(o), adaptive, ctypes.byref(n)))
                assert n.value > 10_000


def test_callback_validation(degpu_mod):
    from degpu import _lib
    f = degpu_mod.ODEFunction.builtin("ball")
    bad = _lib.ContinuousCallbackC(0, 1, 1, 7, 1e-5, 0.01, 1.0)  # rootfind 7
    st = _lib.CallbacksC(1, ctypes.pointer(bad), 0, None)
    o = _opts(degpu_mod, degpu_mod.GPUTsit5())
    o.callbacks = ctypes.addressof(st)
    n = ctypes.c_longlong()
    assert degpu_mod.lib().degpu_rhs_check(f.handle(), ctypes.byref(o), 1, ctypes.byref(n)) == -1
    assert b"continuous callback" in degpu_mod.lib().degpu_last_error()
    o = _opts(degpu_mod, degpu_mod.GPUTsit5())
    o.ntstops = 3  # no pointer
    assert degpu_mod.lib().degpu_rhs_check(f.handle(), ctypes.byref(o), 1, ctypes.byref(n)) == -1


def test_mass_matrix_only_with_rosenbrock(degpu_mod):
    """A mass matrix is accepted by the Rosenbrock methods and refused by the others."""
    from degpu import _lib
    f = degpu_mod.ODEFunction.builtin("robertson_dae")
    assert f.flags & _lib.RHS_HAS_MASS
    n = ctypes.c_longlong()
    for alg in (degpu_mod.GPURosenbrock23(), degpu_mod.GPURodas4(), degpu_mod.GPURodas5P()):
        _lib.check(degpu_mod.lib().degpu_rhs_check(f.handle(), ctypes.byref(_opts(degpu_mod, alg, mode="parity")), 1,
                                                   ctypes.byref(n)))
    for alg in (degpu_mod.GPUTsit5(), degpu_mod.GPUKvaerno5()):
        assert degpu_mod.lib().degpu_rhs_check(f.handle(), ctypes.byref(_opts(degpu_mod, alg)), 1, ctypes.byref(n)) == -4
        assert b"mass matrix" in degpu_mod.lib().degpu_last_error()


def test_version_and_builtins(degpu_mod):
    assert degpu_mod.lib().degpu_version() == b"0.1.0"
    for name, (n, p) in {"lorenz": (3, 3), "robertson": (3, 3), "decay": (1, 1), "growth": (1, 1),
                         "linear15": (15, 1), "gbm": (1, 2), "lorenz_addnoise": (3, 3), "osc": (2, 1),
                         "ball": (2, 1), "robertson_dae": (3, 3)}.items():
        f = degpu_mod.ODEFunction.builtin(name)
        assert (f.nstate, f.nparam) == (n, p)
    with pytest.raises(KeyError):
        degpu_mod.ODEFunction.builtin("nope")


def _opts(degpu_mod, alg, tt=np.float64, **kw):
    return degpu_mod.api._options(alg, tt, dt=kw.pop("dt", 0.1), **kw)


@pytest.mark.parametrize("alg", ["GPUTsit5", "GPUVern7", "GPURosenbrock23", "GPURodas5P", "GPURodas4", "GPUVern9",
                                 "GPUKvaerno3", "GPUKvaerno5"])
@pytest.mark.parametrize("mode", ["fast", "parity"])
def test_nvrtc_compiles_every_algorithm(degpu_mod, alg, mode, tmp_path, monkeypatch):
    """NVRTC (sm_103a) compiles stepper + driver + right-hand side for each algorithm and
    driver, without a GPU."""
    from degpu import _lib
    f = degpu_mod.ODEFunction.builtin("robertson" if "Ro" in alg else "lorenz")
    a = getattr(degpu_mod, alg)()
    n = ctypes.c_longlong()
    for adaptive, driver in ((0, "auto"), (1, "naive"), (1, "persistent")):
        o = _opts(degpu_mod, a, mode=mode, driver=driver)
        _lib.check(degpu_mod.lib().degpu_rhs_check(f.handle(), ctypes.byref(o), adaptive, ctypes.byref(n)))
        assert n.value > 10_000


def test_nvrtc_em_and_user_rhs(degpu_mod):
    from degpu import _lib
    f = degpu_mod.ODEFunction.builtin("gbm")
    o = _opts(degpu_mod, degpu_mod.GPUEM(), tt=np.float32)
    n = ctypes.c_longlong()
    _lib.check(degpu_mod.lib().degpu_rhs_check(f.handle(), ctypes.byref(o), 0, ctypes.byref(n)))
    src = """
    // pendulum with time forcing: u1' = u2, u2' = -p1 sin(u1) + p2 cos(t)
    template <class T>
    __device__ void degpu_f(T* du, const T* u, const float* p, T t) {
      du[0] = u[1];
      du[1] = -p[0] * dsin(u[0]) + p[1] * dcos(t);
    }"""
    g = degpu_mod.ODEFunction(src, 2, 2)
    for alg in (degpu_mod.GPUTsit5(), degpu_mod.GPURodas5P()):
        o = _opts(degpu_mod, alg)
        _lib.check(degpu_mod.lib().degpu_rhs_check(g.handle(), ctypes.byref(o), 1, ctypes.byref(n)))


def test_compile_error_reports_log(degpu_mod):
    bad = degpu_mod.ODEFunction("template <class T> __device__ void degpu_f(T* du, const T* u, const float* p, T t)"
                                " { du[0] = undefined_symbol; }", 1, 0)
    o = _opts(degpu_mod, degpu_mod.GPUTsit5())
    with pytest.raises(degpu_mod.DegpuError) as e:
        from degpu import _lib
        _lib.check(degpu_mod.lib().degpu_rhs_check(bad.handle(), ctypes.byref(o), 1, None))
    assert e.value.code == -2 and "undefined_symbol" in str(e.value)


def _call(degpu_mod, fn, f, B, opt, L=2, ptrs=True):
    from degpu import _lib
    fake = 256 if ptrs else None  # never dereferenced: validation fails first
    pr = _lib.Problems(fake, fake, fake, B)
    out = _lib.Outputs(fake, fake, L, None, None, None)
    return getattr(degpu_mod.lib(), fn)(f.handle(), ctypes.byref(pr), ctypes.byref(opt), ctypes.byref(out), None)


def test_argument_validation_without_gpu(degpu_mod):
    """Errors the reference raises on the host are returned before any device work."""
    f = degpu_mod.ODEFunction.builtin("lorenz")
    T5 = degpu_mod.GPUTsit5()
    assert _call(degpu_mod, "degpu_vectorized_asolve", f, 10, _opts(degpu_mod, T5, dt=-0.1)) == -1
    assert _call(degpu_mod, "degpu_vectorized_asolve", f, -1, _opts(degpu_mod, T5)) == -1
    assert _call(degpu_mod, "degpu_vectorized_asolve", f, 10, _opts(degpu_mod, T5), L=3) == -1  # L must be 2
    o = _opts(degpu_mod, T5, nsaveat=5)
    assert _call(degpu_mod, "degpu_vectorized_asolve", f, 10, o, L=5) == -1  # saveat pointer missing
    assert _call(degpu_mod, "degpu_vectorized_asolve", f, 10, _opts(degpu_mod, T5, block=100)) == -1
    assert _call(degpu_mod, "degpu_vectorized_solve", f, 10, _opts(degpu_mod, degpu_mod.GPUEM())) == -1
    g = degpu_mod.ODEFunction.builtin("gbm")
    assert _call(degpu_mod, "degpu_vectorized_asolve", g, 10, _opts(degpu_mod, degpu_mod.GPUEM())) == -4
    assert "not supported" in degpu_mod.lib().degpu_last_error().decode()
    assert _call(degpu_mod, "degpu_vectorized_solve_sde", f, 10, _opts(degpu_mod, degpu_mod.GPUEM())) == -1
    assert _call(degpu_mod, "degpu_vectorized_asolve", f, 10, _opts(degpu_mod, T5), ptrs=False) == -1
    from degpu import _lib
    h = ctypes.c_void_p()
    assert degpu_mod.lib().degpu_rhs_create(b"x", 0, 0, 0, ctypes.byref(h)) == -1
    assert degpu_mod.lib().degpu_rhs_create(b"x", 3, 3, 64, ctypes.byref(h)) == -1


def test_work_order_validation_without_gpu(degpu_mod):
    """degpu_work_order / degpu_learned_asolve_ex argument checks come before device work;
    the host-buffer API refuses a visiting order (its chunks index the batch themselves)."""
    L = degpu_mod.lib()
    assert L.degpu_work_order(None, -1, None, None) == -1
    assert L.degpu_work_order(None, 0, None, None) == 0            # empty: nothing to order
    assert L.degpu_work_order(None, 10, None, None) == -1          # null buffers
    assert L.degpu_work_order(None, 1 << 31, None, None) == -1     # more than 2^31-1
    from degpu import _lib
    f = degpu_mod.ODEFunction.builtin("lorenz")
    o = _opts(degpu_mod, degpu_mod.GPUTsit5())
    pr = _lib.Problems()
    out = _lib.Outputs()
    assert L.degpu_learned_asolve_ex(None, None, None, ctypes.byref(pr), ctypes.byref(o), 1e-8, 1.0, 1.0,
                                     ctypes.byref(out), None) == -1
    pr.B = -1
    assert L.degpu_learned_asolve_ex(f.handle(), None, None, ctypes.byref(pr), ctypes.byref(o), 1e-8, 1.0, 1.0,
                                     ctypes.byref(out), None) == -1
    pr.B = 0
    assert L.degpu_learned_asolve_ex(f.handle(), None, None, ctypes.byref(pr), ctypes.byref(o), 1e-8, 1.0, 1.0,
                                     ctypes.byref(out), None) == 0
    # the learned host-buffer solve takes models for adaptive ODE solves only (refused before
    # any device work); with no model it is the plain host solve
    em = _opts(degpu_mod, degpu_mod.GPUEM())
    fake_model = ctypes.c_void_p(8)  # never dereferenced: validation fails first
    assert L.degpu_learned_batch_solve_host(f.handle(), fake_model, None, None, None, None, 4, ctypes.byref(em), 1e-8,
                                            1.0, 1.0, None, None, 2, None, None, None, None) == -1
    assert "adaptive ODE" in L.degpu_last_error().decode()
    assert L.degpu_learned_batch_solve_host(f.handle(), None, None, None, None, None, 0, ctypes.byref(o), 1e-8, 1.0,
                                            1.0, None, None, 2, None, None, None, None) == 0
    o.order = 8  # any non-null pointer: refused before it is read
    assert L.degpu_batch_solve_host(f.handle(), None, None, None, 4, ctypes.byref(o), 1, None, None, 2, None, None,
                                    None, None) == -1
    assert "visiting order" in L.degpu_last_error().decode()


# ----------------------------------------------------------------------------- host logic
def test_saveat_normalisation(degpu_mod):
    """lowerlevel_solve.jl:88-102 / 271-306 and test/gpu_kernel_de/conversions.jl."""
    ns = degpu_mod.normalize_saveat
    f32 = np.float32
    tsp = (f32(0), f32(10))
    assert np.array_equal(ns(range(1, 11), tsp, f32, True), np.arange(1, 11, dtype=f32))
    assert np.array_equal(ns(degpu_mod.Range(1, 0.1, 10), tsp, f32, True), (1 + np.arange(91) / 10).astype(f32))
    assert np.array_equal(ns(degpu_mod.Range(1, 1.0, 10), tsp, f32, False), np.arange(1, 11, dtype=f32))
    assert np.array_equal(ns(1.0, tsp, f32, True), np.arange(0, 11, dtype=f32))
    assert np.array_equal(ns(0.0, tsp, f32, True), np.array([0, 10], f32))
    assert np.array_equal(ns([1.0, 5.0, 10.0], tsp, f32, True), np.array([1, 5, 10], f32))
    assert ns(0.5, (0.0, 10.0), np.float64, False).shape == (21,)
    with pytest.raises(ValueError, match="too many save points"):
        ns(1e-5, tsp, f32, True)
    assert ns(None, tsp, f32, True) is None


def test_output_sizing(degpu_mod):
    """length(t0:dt:tf) for the fixed-step save_everystep output (lowerlevel_solve.jl:73)."""
    fl = degpu_mod.api.fixed_step_length
    assert fl((0.0, 10.0), 0.1, np.float32) == 101
    assert fl((0.0, 1.0), 0.01, np.float32) == 101
    assert fl((0.0, 1.0), 0.3, np.float64) == 4


def test_batch_building_and_errors(degpu_mod):
    """batch_solve (src/solve.jl:186-245): prob_func per trajectory; saveat lengths must agree."""
    f = degpu_mod.ODEFunction.builtin("lorenz")
    prob = degpu_mod.ODEProblem(f, [1, 0, 0], (0, 10), [10, 28, 8 / 3])
    ens = degpu_mod.EnsembleProblem(prob, prob_func=lambda q, ctx: degpu_mod.remake(q, p=q.p * (ctx["sim_id"] + 1)))
    u0, p, tsp, sa = degpu_mod.api._build_batch(ens, range(0, 4))
    assert p.shape == (4, 3) and np.allclose(p[3], prob.p * 4) and sa is None
    ens2 = degpu_mod.EnsembleProblem(prob, prob_func=lambda q, ctx: degpu_mod.remake(
        q, kwargs={"saveat": np.linspace(0, 10, 3 + ctx["sim_id"])}))
    with pytest.raises(ValueError, match="same length"):
        degpu_mod.api._build_batch(ens2, range(0, 2))
    with pytest.raises(ValueError):
        degpu_mod.ODEProblem(f, [1, 0], (0, 1), [1, 2, 3])
    with pytest.raises(NotImplementedError):
        degpu_mod.EnsembleGPUKernel(0, 0.5)
    assert degpu_mod.GPURodas5 is degpu_mod.GPURodas5P
    assert [degpu_mod.alg_order(a()) for a in (degpu_mod.GPUTsit5, degpu_mod.GPUVern7, degpu_mod.GPURosenbrock23,
                                              degpu_mod.GPURodas5P, degpu_mod.GPUEM)] == [5, 7, 2, 5, 1]
