"""GPU parity of the kernels against the CPU oracle (through libdegpu's C ABI).

Bars:
  * parity mode (no FMA, portable pow, Cramer solves): bit-identical to the oracle, for
    every algorithm and driver -- fixed step, adaptive, saveat dense output, stiff, EM;
  * fast mode (FMA, hardware pow, LU + refinement): FP32 tolerances against the oracle
    and FP64-oracle error bounds (tolerances written per test);
  * the reference's own test shapes and tolerances (public_interface.jl,
    gpu_kernel_de/conversions.jl, gpu_ode_regression.jl, stiff_ode/gpu_ode_regression.jl).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ALGS = {"tsit5": "GPUTsit5", "vern7": "GPUVern7", "rosenbrock23": "GPURosenbrock23", "rodas5p": "GPURodas5P",
        "rodas4": "GPURodas4", "vern9": "GPUVern9", "kvaerno3": "GPUKvaerno3", "kvaerno5": "GPUKvaerno5"}


def lorenz_batch(B, seed=0, chaotic=True):
    rng = np.random.default_rng(seed)
    scale = np.array([10, 28, 8 / 3]) if chaotic else np.array([10, 20, 8 / 3])
    p = (rng.random((B, 3)) * scale).astype(np.float32)
    u0 = np.tile(np.array([1, 0, 0], np.float32), (B, 1))
    return u0, p


def robertson_batch(B, seed=0):
    rng = np.random.default_rng(seed)
    k = (np.array([0.04, 3e7, 1e4]) * np.exp(rng.normal(0, 0.3, (B, 3)))).astype(np.float32)
    u0 = np.tile(np.array([1, 0, 0], np.float32), (B, 1))
    return u0, k


def gpu_solve(degpu, model, alg, u0, p, tspan, tt, *, adaptive, dt, saveat=None, save_everystep=False, **kw):
    import torch
    f = degpu.ODEFunction.builtin(model)
    B = u0.shape[0]
    tsp = np.broadcast_to(np.asarray(tspan, dtype=tt), (B, 2))
    probs = degpu.DeviceProblems(f, u0, p, tsp, tt, torch.device("cuda", 0))
    a = {"em": degpu.GPUEM, "siea": degpu.GPUSIEA}[alg]() if alg in ("em", "siea") else getattr(degpu, ALGS[alg])()
    r = degpu.api._solve_device(probs, a, adaptive, dt=dt, saveat=saveat, save_everystep=save_everystep, **kw)
    torch.cuda.synchronize()
    return (r.ts.cpu().numpy(), r.us.cpu().numpy(), r.retcode.cpu().numpy(), r.naccept.cpu().numpy(),
            r.nreject.cpu().numpy())


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32 if a.dtype == np.float32 else np.uint64)


def assert_bit_equal(a, b, what):
    ba, bb = bits(a), bits(b)
    bad = np.argwhere(ba != bb)
    assert bad.size == 0, f"{what}: {len(bad)} elements differ, first at {bad[0].tolist()}: {a[tuple(bad[0])]!r} vs {b[tuple(bad[0])]!r}"


def assert_saved_equal(us, ous, ts, t0):
    """Compare only the rows a trajectory actually saved (row 0 and rows whose saved time is
    not the t0 fill); unsaved rows are uninitialised memory, as in the reference."""
    saved = ts != t0
    saved[:, 0] = True
    assert_bit_equal(np.where(saved[..., None], us, 0), np.where(saved[..., None], ous, 0), "us (saved rows)")


# ----------------------------------------------------------------------------- fixed step
@pytest.mark.parametrize("alg", ["tsit5", "vern7", "vern9"])
@pytest.mark.parametrize("tt", [np.float32, np.float64])
def test_fixed_step_bit_parity_lorenz(degpu_mod, oracle_mod, alg, tt):
    """Lorenz ensemble, fixed dt=0.1f0, tspan (0,10), final state only: 10,000 trajectories
    with p = U(0,1)^3 .* [10,28,8/3] -- bit-identical to the oracle in parity mode."""
    u0, p = lorenz_batch(10_000, seed=1)
    ts, us, rc, na, _ = gpu_solve(degpu_mod, "lorenz", alg, u0, p, (0, 10), tt, adaptive=False, dt=0.1,
                                  save_everystep=False, mode="parity")
    ots, ous, orc, ona, _ = oracle_mod.solve("lorenz", alg, u0, p, [0, 10], adaptive=False, dt=float(tt(0.1)), L=2,
                                             time_f64=tt == np.float64)
    assert_bit_equal(us, ous, "us")
    assert_bit_equal(ts, ots, "ts")
    assert (rc == 1).all() and (na == ona).all() and (na == 100).all()


def test_fixed_step_save_everystep_parity(degpu_mod, oracle_mod):
    u0, p = lorenz_batch(257, seed=2)
    ts, us, rc, _, _ = gpu_solve(degpu_mod, "lorenz", "tsit5", u0, p, (0, 1), np.float32, adaptive=False, dt=0.01,
                                 save_everystep=True, mode="parity")
    L = ts.shape[1]
    assert L == 101
    ots, ous, _, _, _ = oracle_mod.solve("lorenz", "tsit5", u0, p, [0, 1], adaptive=False, dt=float(np.float32(0.01)),
                                         L=L, save_everystep=True)
    assert_bit_equal(us, ous, "us")
    assert_bit_equal(ts, ots, "ts")


@pytest.mark.parametrize("alg", ["tsit5", "vern7", "rosenbrock23", "rodas5p", "rodas4", "vern9", "kvaerno3", "kvaerno5"])
def test_fixed_step_saveat_parity(degpu_mod, oracle_mod, alg):
    u0, p = lorenz_batch(300, seed=3, chaotic=False)
    sa = np.array([0.0, 0.25, 2.0, 4.0, 5.05, 10.0], np.float32)
    ts, us, rc, _, _ = gpu_solve(degpu_mod, "lorenz", alg, u0, p, (0, 10), np.float32, adaptive=False, dt=0.01,
                                 saveat=sa, mode="parity")
    ots, ous, _, _, _ = oracle_mod.solve("lorenz", alg, u0, p, [0, 10], adaptive=False, dt=float(np.float32(0.01)),
                                         L=len(sa), saveat=sa.astype(np.float64))
    assert_bit_equal(us, ous, "us")
    assert_bit_equal(ts, ots, "ts")


def test_fixed_step_fast_mode_close(degpu_mod, oracle_mod):
    """FMA fast mode on non-chaotic members: within 1e-4 relative of the strict oracle."""
    u0, p = lorenz_batch(4096, seed=4, chaotic=False)
    _, us, _, _, _ = gpu_solve(degpu_mod, "lorenz", "tsit5", u0, p, (0, 10), np.float32, adaptive=False, dt=0.01,
                               mode="fast", save_everystep=False)
    _, ous, _, _, _ = oracle_mod.solve("lorenz", "tsit5", u0, p, [0, 10], adaptive=False, dt=float(np.float32(0.01)), L=2)
    rel = np.abs(us[:, 1] - ous[:, 1]).max(axis=1) / np.maximum(np.abs(ous[:, 1]).max(axis=1), 1.0)
    assert np.median(rel) < 1e-5 and np.quantile(rel, 0.99) < 1e-4, (np.median(rel), rel.max())


# ----------------------------------------------------------------------------- adaptive
@pytest.mark.parametrize("alg", ["tsit5", "vern7", "vern9"])
@pytest.mark.parametrize("driver", ["naive", "persistent"])
@pytest.mark.parametrize("tt", [np.float32, np.float64])
def test_adaptive_saveat_bit_parity(degpu_mod, oracle_mod, alg, driver, tt):
    """Adaptive Tsit5/Vern7 with saveat 0:0.5:10, reltol 1e-6, abstol 1e-8, perturbed u0:
    parity mode is bit-identical to the oracle (controller, dense output, end snap)."""
    B = 2048
    rng = np.random.default_rng(5)
    _, p = lorenz_batch(B, seed=5)
    u0 = (np.array([1, 0, 0]) + rng.normal(0, 0.1, (B, 3))).astype(np.float32)
    sa = np.arange(0, 10.0001, 0.5)
    ts, us, rc, na, nr = gpu_solve(degpu_mod, "lorenz", alg, u0, p, (0, 10), tt, adaptive=True, dt=0.1, saveat=sa,
                                   abstol=1e-8, reltol=1e-6, mode="parity", driver=driver)
    ots, ous, orc, ona, onr = oracle_mod.solve("lorenz", alg, u0, p, [0, 10], adaptive=True, dt=float(tt(0.1)),
                                               L=len(sa), saveat=sa.astype(tt).astype(np.float64), abstol=1e-8,
                                               reltol=1e-6, time_f64=tt == np.float64)
    assert (na == ona).all() and (nr == onr).all()
    assert (rc == orc).all() and (rc == 1).all()
    assert_bit_equal(us, ous, "us")
    assert_bit_equal(ts, ots, "ts")


@pytest.mark.parametrize("alg", ["rosenbrock23", "rodas5p", "rodas4", "kvaerno3", "kvaerno5"])
@pytest.mark.parametrize("jac", ["auto", "ad", "finitediff"])
def test_stiff_robertson_bit_parity(degpu_mod, oracle_mod, alg, jac):
    """Robertson kinetics, k scaled by lognormal(0,0.3), tspan (0,1e5), 32 log-spaced
    saveat points, reltol 1e-4, abstol 1e-7, FP64 time: bit-identical in parity mode."""
    if alg.startswith("kvaerno") and jac == "finitediff":
        # the absolute sqrt(eps) difference step (alg_utils.jl:17-27) is larger than the
        # intermediate species itself here; with it the ESDIRKs' Newton iteration never
        # converges and every trajectory runs to maxiters (the oracle shows the same)
        pytest.skip("finite-difference Jacobian unusable for the ESDIRKs on Robertson")
    u0, k = robertson_batch(512, seed=6)
    sa = np.concatenate([[0.0], np.logspace(-6, 0, 31) * 1e5])
    ts, us, rc, na, nr = gpu_solve(degpu_mod, "robertson", alg, u0, k, (0, 1e5), np.float64, adaptive=True, dt=1e-3,
                                   saveat=sa, abstol=1e-7, reltol=1e-4, mode="parity", jac=jac, driver="naive")
    ojac = {"auto": "analytic", "ad": "ad", "finitediff": "finitediff"}[jac]
    ots, ous, orc, ona, onr = oracle_mod.solve("robertson", alg, u0, k, [0, 1e5], adaptive=True, dt=1e-3, L=len(sa),
                                               saveat=sa, abstol=1e-7, reltol=1e-4, time_f64=True, jac=ojac)
    assert (na == ona).all() and (nr == onr).all() and (rc == orc).all()
    assert_bit_equal(ts, ots, "ts")
    assert_saved_equal(us, ous, ots, 0.0)


@pytest.mark.parametrize("alg", ["rosenbrock23", "rodas5p", "rodas4", "kvaerno3", "kvaerno5"])
def test_stiff_fast_mode_vs_fp64(degpu_mod, oracle_mod, alg):
    """Fast mode (pivoted LU + compensated residual refinement) against the FP64 stiff
    oracle: final-state relative error of the dominant species within 10x reltol."""
    u0, k = robertson_batch(256, seed=7)
    ts, us, rc, _, _ = gpu_solve(degpu_mod, "robertson", alg, u0, k, (0, 1e5), np.float64, adaptive=True, dt=1e-3,
                                 abstol=1e-7, reltol=1e-4, mode="fast")
    ref, _ = oracle_mod.vern9("robertson", u0.astype(np.float64), k.astype(np.float64), 0.0, np.array([1e5]),
                              rtol=1e-10, atol=1e-14, method="rodas5p")
    err = np.abs(us[:, 1, [0, 2]] - ref[:, 0, [0, 2]]) / np.abs(ref[:, 0, [0, 2]])
    assert (rc == 1).all()
    # the 3rd / 5th order ESDIRKs overshoot reltol on the stiff transient more than the
    # Rosenbrock methods (the oracle's own maxima: 1.1e-2 and 3.1e-3)
    tol = {"kvaerno3": 3e-2, "kvaerno5": 1e-2}.get(alg, 1e-3)
    assert err.max() < tol, err.max()


@pytest.mark.parametrize("alg,dt", [("rosenbrock23", 0.1), ("rodas4", 1e-3), ("rodas5p", 1e-3)])
def test_mass_matrix_dae_parity(degpu_mod, oracle_mod, alg, dt):
    """gpu_ode_mass_matrix.jl: Robertson DAE with mass matrix diag(1,1,0), 512 perturbed rate
    sets: parity mode bit-identical to the oracle; fast mode within the reference's 8e-4 of
    the FP64 ODE-form solution and on the constraint."""
    u0, k = robertson_batch(512, seed=9)
    sa = np.array([0.0, 1.0, 10.0, 100.0, 1e3, 1e4, 1e5])
    ts, us, rc, na, nr = gpu_solve(degpu_mod, "robertson_dae", alg, u0, k, (0, 1e5), np.float32, adaptive=True, dt=dt,
                                   saveat=sa, abstol=1e-5, reltol=1e-5, mode="parity")
    ots, ous, orc, ona, onr = oracle_mod.solve("robertson_dae", alg, u0, k, [0, 1e5], adaptive=True, dt=dt,
                                               L=len(sa), saveat=sa, abstol=1e-5, reltol=1e-5)
    assert (rc == orc).all() and (na == ona).all()
    assert_bit_equal(us, ous, "us")
    ts, us, rc, _, _ = gpu_solve(degpu_mod, "robertson_dae", alg, u0, k, (0, 1e5), np.float64, adaptive=True, dt=dt,
                                 saveat=sa, abstol=1e-5, reltol=1e-5, mode="fast")
    ref, _ = oracle_mod.vern9("robertson", u0.astype(np.float64), k.astype(np.float64), 0.0, sa, rtol=1e-10,
                              atol=1e-14, method="rodas5p")
    assert (rc == 1).all()
    assert np.abs(us - ref).max() < 8e-4
    assert np.abs(us.sum(axis=2) - 1.0).max() < 1e-5


def test_linear15_lu_path(degpu_mod, oracle_mod):
    """N = 15 exercises the partial-pivot LU solve (linsolve.jl:88-108) in both modes."""
    B = 64
    rng = np.random.default_rng(8)
    u0 = rng.random((B, 15)).astype(np.float32)
    p = np.ones((B, 1), np.float32)
    for mode in ("parity", "fast"):
        _, us, rc, _, _ = gpu_solve(degpu_mod, "linear15", "rodas5p", u0, p, (0, 1), np.float32, adaptive=True, dt=0.01,
                                    abstol=1e-7, reltol=1e-7, mode=mode)
        exact = u0 * np.exp(np.float32(1.01))
        assert (rc == 1).all()
        assert np.abs(us[:, 1] - exact).max() / np.abs(exact).max() < 1e-4
    _, us, _, _, _ = gpu_solve(degpu_mod, "linear15", "rodas5p", u0, p, (0, 1), np.float32, adaptive=True, dt=0.01,
                               abstol=1e-7, reltol=1e-7, mode="parity")
    _, ous, _, _, _ = oracle_mod.solve("linear15", "rodas5p", u0, p, [0, 1], adaptive=True, dt=float(np.float32(0.01)),
                                       L=2, abstol=1e-7, reltol=1e-7)
    assert_bit_equal(us, ous, "us")


def test_em_bit_parity(degpu_mod, oracle_mod):
    """GPUEM on GBM (gpu_sde_convergence.jl problem): parity mode reproduces the oracle's
    Philox/Box-Muller paths bit for bit, with saveat linear interpolation."""
    B = 1000
    u0 = np.full((B, 1), 0.1, np.float32)
    p = np.tile(np.array([1.5, 0.01], np.float32), (B, 1))
    sa = np.linspace(0, 1, 11)
    ts, us, rc, _, _ = gpu_solve(degpu_mod, "gbm", "em", u0, p, (0, 1), np.float32, adaptive=False,
                                 dt=float(np.float32(1 / 256)), saveat=sa, mode="parity", seed=1234)
    ots, ous, orc, _, _ = oracle_mod.solve("gbm", "em", u0, p, [0, 1], adaptive=False, dt=float(np.float32(1 / 256)),
                                           L=len(sa), saveat=sa.astype(np.float32).astype(np.float64), seed=1234)
    assert_bit_equal(us, ous, "us")
    assert (rc == 1).all()


@pytest.mark.parametrize("tt", [np.float32, np.float64])
def test_siea_bit_parity(degpu_mod, oracle_mod, tt):
    """GPUSIEA (gpu_siea_perform_step.jl) on GBM: parity mode reproduces the oracle's paths
    bit for bit (saveat linear interpolation, both time types)."""
    B = 1000
    u0 = np.full((B, 1), 0.1, np.float32)
    p = np.tile(np.array([1.5, 0.2], np.float32), (B, 1))
    sa = np.linspace(0, 1, 11)
    ts, us, rc, _, _ = gpu_solve(degpu_mod, "gbm", "siea", u0, p, (0, 1), tt, adaptive=False,
                                 dt=float(np.float32(1 / 64)), saveat=sa, mode="parity", seed=99)
    ots, ous, orc, _, _ = oracle_mod.solve("gbm", "siea", u0, p, [0, 1], adaptive=False, dt=float(np.float32(1 / 64)),
                                           L=len(sa), saveat=sa.astype(tt).astype(np.float64), seed=99,
                                           time_f64=tt == np.float64)
    assert_bit_equal(us, ous, "us")
    assert (rc == 1).all()


def test_siea_weak_order(degpu_mod):
    """gpu_sde_convergence.jl:34-45: weak order of GPUSIEA on du = 1.5 u dt + 0.01 u dW,
    E[u(1)] = 0.1 e^1.5, dts 1/64..1/16 -- |order - 2.1| < 0.4 (10^6 paths, fast mode)."""
    B = 1_000_000
    u0 = np.full((B, 1), 0.1, np.float32)
    p = np.tile(np.array([1.5, 0.01], np.float32), (B, 1))
    exact = 0.1 * np.exp(1.5)
    dts = [1 / 64, 1 / 32, 1 / 16]
    errs = []
    for dt in dts:
        _, us, rc, _, _ = gpu_solve(degpu_mod, "gbm", "siea", u0, p, (0, 1), np.float32, adaptive=False,
                                    dt=float(np.float32(dt)), save_everystep=False, mode="fast", seed=1234)
        errs.append(abs(us[:, 1, 0].astype(np.float64).mean() - exact))
    order = np.polyfit(np.log(dts), np.log(errs), 1)[0]
    assert abs(order - 2.1) < 0.4, (errs, order)


def test_em_weak_order_and_mean(degpu_mod):
    """gpu_sde_regression.jl:42 -- mean of GBM paths du = u dt + u dW from 0.5 matches 0.5 e^t
    (inf-norm < 6e-2), fast mode, 10^5 paths."""
    B = 100_000
    u0 = np.full((B, 1), 0.5, np.float32)
    p = np.tile(np.array([1.0, 1.0], np.float32), (B, 1))
    sa = np.linspace(0, 1, 11)
    ts, us, rc, _, _ = gpu_solve(degpu_mod, "gbm", "em", u0, p, (0, 1), np.float32, adaptive=False,
                                 dt=float(np.float32(1 / 256)), saveat=sa, mode="fast", seed=123)
    mean = us[:, :, 0].mean(axis=0)
    assert np.abs(mean - 0.5 * np.exp(ts[0])).max() < 6e-2


# ----------------------------------------------------------------------------- drivers and plans
def test_persistent_equals_naive_uneven(degpu_mod):
    """Uneven Lorenz batch (rho ~ U(0,100), tEnd ~ U(1,20)): the persistent driver's results
    equal the one-trajectory-per-thread driver's bit for bit (both fast mode)."""
    B = 20_000
    rng = np.random.default_rng(9)
    p = np.stack([np.full(B, 10.0), rng.uniform(0, 100, B), np.full(B, 8 / 3)], 1).astype(np.float32)
    u0 = np.tile(np.array([1, 0, 0], np.float32), (B, 1))
    import torch
    f = degpu_mod.ODEFunction.builtin("lorenz")
    tsp = np.stack([np.zeros(B), rng.uniform(1, 20, B)], 1)
    probs = degpu_mod.DeviceProblems(f, u0, p, tsp, np.float64, torch.device("cuda", 0))
    outs = {}
    for drv in ("naive", "persistent"):
        r = degpu_mod.api._solve_device(probs, degpu_mod.GPUTsit5(), True, dt=0.1, abstol=1e-8, reltol=1e-6,
                                        driver=drv, mode="fast")
        torch.cuda.synchronize()
        outs[drv] = (r.us.cpu().numpy(), r.ts.cpu().numpy(), r.naccept.cpu().numpy())
    assert_bit_equal(outs["naive"][0], outs["persistent"][0], "us")
    assert_bit_equal(outs["naive"][1], outs["persistent"][1], "ts")
    assert (outs["naive"][2] == outs["persistent"][2]).all()
    assert np.allclose(outs["naive"][1][:, 1], tsp[:, 1])


def test_plan_graph_matches_direct(degpu_mod):
    """A CUDA-graph plan (autotuned) produces the same bits as a direct solve."""
    import ctypes
    import torch
    from degpu import _lib
    B = 50_000
    u0, p = lorenz_batch(B, seed=10)
    f = degpu_mod.ODEFunction.builtin("lorenz")
    tsp = np.tile([0.0, 10.0], (B, 1))
    probs = degpu_mod.DeviceProblems(f, u0, p, tsp, np.float64, torch.device("cuda", 0))
    direct = degpu_mod.api._solve_device(probs, degpu_mod.GPUTsit5(), True, dt=0.1, abstol=1e-8, reltol=1e-6,
                                         driver="persistent")
    ts = torch.empty((B, 2), dtype=torch.float64, device="cuda")
    us = torch.empty((B, 2, 3), dtype=torch.float32, device="cuda")
    opt = degpu_mod.api._options(degpu_mod.GPUTsit5(), np.float64, dt=0.1, abstol=1e-8, reltol=1e-6, driver="persistent")
    out = _lib.Outputs(ts.data_ptr(), us.data_ptr(), 2, None, None, None)
    pr = probs.cstruct()
    plan = ctypes.c_void_p()
    st = torch.cuda.current_stream()
    _lib.check(_lib.lib().degpu_plan_create(f.handle(), ctypes.byref(pr), ctypes.byref(opt), 1, ctypes.byref(out),
                                            ctypes.c_void_p(st.cuda_stream), ctypes.byref(plan)))
    try:
        us.zero_()
        _lib.check(_lib.lib().degpu_plan_launch(plan, ctypes.c_void_p(st.cuda_stream)))
        _lib.check(_lib.lib().degpu_plan_launch(plan, ctypes.c_void_p(st.cuda_stream)))
        torch.cuda.synchronize()
        info = [ctypes.c_int() for _ in range(5)]
        _lib.check(_lib.lib().degpu_plan_info(plan, *[ctypes.byref(x) for x in info]))
        assert info[0].value in (64, 128, 256) and info[3].value == 2
    finally:
        _lib.lib().degpu_plan_destroy(plan)
    assert_bit_equal(us.cpu().numpy(), direct.us.cpu().numpy(), "us")


# ----------------------------------------------------------------------------- reference test shapes
def test_public_interface_shapes(degpu_mod):
    """test/public_interface.jl:26-42, 71-80."""
    import torch
    src = degpu_mod.ODEFunction.builtin("growth")
    prob = degpu_mod.ODEProblem(src, [1.0], (0.0, 0.2), [1.0])
    probs = degpu_mod.adapt(0, [degpu_mod.make_prob_compatible(prob) for _ in range(2)])
    ts, us = degpu_mod.vectorized_solve(probs, prob, degpu_mod.GPUTsit5(), dt=0.1, save_everystep=False)
    assert tuple(ts.shape) == (2, 2) and tuple(us.shape[:2]) == (2, 2)
    assert (us[:, 0, 0].cpu() == 1.0).all()
    ats, aus = degpu_mod.vectorized_asolve(probs, prob, degpu_mod.GPUTsit5(), dt=0.1, saveat=0.1, save_everystep=False)
    assert ats.shape[0] == 2 and aus.shape[0] == 2
    assert float(aus[0, 0, 0]) == 1.0
    sol = degpu_mod.solve(degpu_mod.EnsembleProblem(prob), degpu_mod.GPUTsit5(), degpu_mod.EnsembleGPUKernel(0),
                          trajectories=2, adaptive=False, dt=0.1)
    assert len(sol.u) == 2 and all(s.u[0][0] == 1.0 for s in sol.u)
    # SDE interface (public_interface.jl:44-59)
    g = degpu_mod.ODEFunction("template <class T> __device__ void degpu_f(T* du, const T* u, const float* p, T t) { du[0] = u[0]; }\n"
                              "template <class T> __device__ void degpu_g(T* g, const T* u, const float* p, T t) { g[0] = u[0]; }\n",
                              1, 1, noise=True)
    sprob = degpu_mod.SDEProblem(g, [1.0], (0.0, 0.2), [1.0])
    sprobs = degpu_mod.adapt(0, [sprob, sprob])
    sts, sus = degpu_mod.vectorized_solve(sprobs, sprob, degpu_mod.GPUEM(), dt=0.1, save_everystep=False)
    assert tuple(sts.shape) == (2, 2) and torch.isfinite(sus).all()


def test_saveat_conversions(degpu_mod):
    """test/gpu_kernel_de/conversions.jl: exact saved times for ranges, vectors, numbers."""
    f = degpu_mod.ODEFunction.builtin("lorenz")
    prob = degpu_mod.ODEProblem(f, [1.0, 0.0, 0.0], (0.0, 10.0), [10.0, 28.0, 8 / 3])
    rng = np.random.default_rng(11)
    P = (rng.random((10_000, 3)) * np.array([10, 28, 8 / 3])).astype(np.float32)
    ens = degpu_mod.EnsembleProblem.from_arrays(prob, p=P)
    K, EG, T5 = 10_000, degpu_mod.EnsembleGPUKernel(0), degpu_mod.GPUTsit5()
    R = degpu_mod.Range
    t = degpu_mod.solve(ens, T5, EG, trajectories=K, saveat=range(1, 11)).u[0].t
    assert np.array_equal(t, np.arange(1, 11, dtype=np.float32))
    t = degpu_mod.solve(ens, T5, EG, trajectories=K, saveat=R(1, 0.1, 10)).u[0].t
    assert np.array_equal(t, (1 + np.arange(91) / 10).astype(np.float32))
    t = degpu_mod.solve(ens, T5, EG, trajectories=K, saveat=1.0).u[0].t
    assert np.array_equal(t, np.arange(0, 11, dtype=np.float32))
    t = degpu_mod.solve(ens, T5, EG, trajectories=K, saveat=[1.0, 5.0, 10.0]).u[0].t
    assert np.array_equal(t, np.array([1, 5, 10], np.float32))


@pytest.mark.parametrize("alg", ["tsit5", "vern7"])
def test_reference_regression_tolerances(degpu_mod, oracle_mod, alg):
    """gpu_ode_regression.jl:24-46, 98-99: Lorenz p=[10,28,8/3], u0=[1,0,0], Float32 --
    fixed dt=0.01 within 5e-3 of Vern9 at the final time; adaptive 1e-7 within 1e-3."""
    u0 = np.array([[1, 0, 0]], np.float32)
    p = np.array([[10, 28, 8 / 3]], np.float32)
    ts, us, _, _, _ = gpu_solve(degpu_mod, "lorenz", alg, u0, p, (0, 10), np.float32, adaptive=False, dt=0.01)
    v9, _ = oracle_mod.vern9("lorenz", u0, p, 0.0, np.array([float(ts[0, -1])]))
    assert np.linalg.norm(us[0, -1] - v9[0, 0]) < 5e-3
    ts, us, _, _, _ = gpu_solve(degpu_mod, "lorenz", alg, u0, p, (0, 10), np.float32, adaptive=True, dt=0.01,
                                abstol=1e-7, reltol=1e-7)
    v9, _ = oracle_mod.vern9("lorenz", u0, p, 0.0, np.array([10.0]))
    assert np.linalg.norm(us[0, 1] - v9[0, 0]) < 1e-3


def test_fp64_oracle_error_adaptive_config(degpu_mod, oracle_mod):
    """Adaptive Tsit5/Vern7 (reltol 1e-6, abstol 1e-8, FP64 time, fast mode) against the FP64
    Vern9 oracle at reltol 1e-12 over the saveat grid: median relative error <= 1e-4 over
    members whose FP64 solution is stable (rho < 24, non-chaotic)."""
    B = 512
    rng = np.random.default_rng(12)
    p = np.stack([rng.uniform(0, 10, B), rng.uniform(0, 24, B), rng.uniform(0, 8 / 3, B)], 1).astype(np.float32)
    u0 = (np.array([1, 0, 0]) + rng.normal(0, 0.1, (B, 3))).astype(np.float32)
    sa = np.arange(0, 10.0001, 0.5)
    ref, _ = oracle_mod.vern9("lorenz", u0.astype(np.float64), p.astype(np.float64), 0.0, sa)
    for alg in ("tsit5", "vern7"):
        _, us, rc, _, _ = gpu_solve(degpu_mod, "lorenz", alg, u0, p, (0, 10), np.float64, adaptive=True, dt=0.1,
                                    saveat=sa, abstol=1e-8, reltol=1e-6, mode="fast")
        scale = np.maximum(np.abs(ref).max(axis=2), 1e-2)
        rel = np.abs(us - ref).max(axis=2) / scale
        assert (rc == 1).all()
        assert np.median(rel[:, -1]) < 1e-4, (alg, np.median(rel[:, -1]))


# ----------------------------------------------------------------------------- failures and edges
def test_retcodes_and_edges(degpu_mod):
    """maxiters cap -> MaxIters, NaN parameters -> Unstable, t0 == tf, empty ensemble,
    B not a multiple of the block size -- never a trap or a hang."""
    import torch
    u0, p = lorenz_batch(1001, seed=13)
    p[5] = np.nan
    _, us, rc, _, _ = gpu_solve(degpu_mod, "lorenz", "tsit5", u0, p, (0, 10), np.float64, adaptive=True, dt=0.1,
                                abstol=1e-8, reltol=1e-6, maxiters=50)
    assert rc[5] in (5, 4)
    rest = np.delete(rc, 5)
    assert set(np.unique(rest)) <= {1, 4} and (rest == 4).mean() > 0.9  # slow members may finish in < 50
    _, us, rc, na, _ = gpu_solve(degpu_mod, "lorenz", "tsit5", u0[:7], p[:7], (3, 3), np.float64, adaptive=True, dt=0.1)
    assert (na == 0).all() and np.array_equal(us[:, 1], u0[:7])
    f = degpu_mod.ODEFunction.builtin("lorenz")
    empty = degpu_mod.DeviceProblems(f, np.zeros((0, 3), np.float32), np.zeros((0, 3), np.float32),
                                     np.zeros((0, 2)), np.float64, torch.device("cuda", 0))
    r = degpu_mod.api._solve_device(empty, degpu_mod.GPUTsit5(), True, dt=0.1)
    assert r.us.shape[0] == 0


def test_invalid_arguments_raise(degpu_mod):
    import torch
    f = degpu_mod.ODEFunction.builtin("lorenz")
    u0, p = lorenz_batch(4)
    probs = degpu_mod.DeviceProblems(f, u0, p, np.tile([0, 1.0], (4, 1)), np.float64, torch.device("cuda", 0))
    with pytest.raises(NotImplementedError):
        degpu_mod.vectorized_asolve(probs, None, degpu_mod.GPUEM(), dt=0.1)
    with pytest.raises(degpu_mod.DegpuError):
        degpu_mod.api._solve_device(probs, degpu_mod.GPUTsit5(), True, dt=-1.0)


def test_ensemble_reduction_batches(degpu_mod):
    """test/reduction.jl on the kernel path: u' = 1.01 u from ra[i] * 0.5, output_func keeps
    the final state, reduction sums batch by batch (batch_size 20 of 100) -- equal to the
    sum of the unreduced solve, and to the exact 0.5 e^1.01 sum(ra)."""
    rng = np.random.default_rng(100)
    ra = rng.random(100)
    src = """template <class T>
__device__ __forceinline__ void degpu_f(T* du, const T* u, const float* p, T t) { du[0] = 1.01f * u[0]; }"""
    f = degpu_mod.ODEFunction(src, 1, 0)
    prob = degpu_mod.ODEProblem(f, np.array([0.5], np.float32), (0.0, 1.0), np.zeros(0, np.float32),
                                time_type=np.float64)
    prob_func = lambda pr, ctx: degpu_mod.remake(pr, u0=np.float32(ra[ctx["sim_id"]]) * pr.u0)
    output_func = lambda sol, ctx: (sol.u[-1], False)
    reduction = lambda u, batch, I: (u + sum(batch), False)
    e1 = degpu_mod.EnsembleProblem(prob, prob_func=prob_func, output_func=output_func)
    s1 = degpu_mod.solve(e1, degpu_mod.GPUTsit5(), degpu_mod.EnsembleGPUKernel(0), trajectories=100, batch_size=20,
                         reltol=1e-8, abstol=1e-8)
    e2 = degpu_mod.EnsembleProblem(prob, prob_func=prob_func, output_func=output_func, reduction=reduction,
                                   u_init=np.zeros(1, np.float32))
    s2 = degpu_mod.solve(e2, degpu_mod.GPUTsit5(), degpu_mod.EnsembleGPUKernel(0), trajectories=100, batch_size=20,
                         reltol=1e-8, abstol=1e-8)
    total = sum(s1.u[i] for i in range(100))
    assert np.allclose(total, s2.u, rtol=1e-6)
    assert np.allclose(s2.u, 0.5 * np.exp(1.01) * ra.astype(np.float32).sum(), rtol=1e-4)


@pytest.mark.parametrize("alg", ["GPUTsit5", "GPUVern7", "GPUVern9", "GPURosenbrock23", "GPURodas4"])
def test_lower_level_api_lorenz(degpu_mod, oracle_mod, alg):
    """test/lower_level_api.jl: 10,000 Lorenz problems with rand(Float32, 3) .* p, analytic
    Jacobian and time gradient, Float32 tspan (0, 10); make_prob_compatible -> adapt ->
    vectorized_solve / vectorized_asolve (save_everystep=false, dt=0.1f0, the default
    tolerances).  The reference only runs them; here every member must end finite in fast
    mode, and parity mode must reproduce the oracle bit for bit."""
    import torch
    rng = np.random.default_rng(0)
    B = 10_000
    base = np.array([10.0, 28.0, 8 / 3.0], np.float32)
    base_src = degpu_mod.ODEFunction.builtin("lorenz").source
    jac_src = """
__device__ __forceinline__ void degpu_jac(float* J, const float* u, const float* p, float t) {
  J[0] = -p[0]; J[1] = p[1] - u[2]; J[2] = u[1];
  J[3] = p[0];  J[4] = -1.0f;       J[5] = u[0];
  J[6] = 0.0f;  J[7] = -u[0];       J[8] = -p[2];
}
__device__ __forceinline__ void degpu_tgrad(float* dT, const float* u, const float* p, float t) {
  dT[0] = 0.0f; dT[1] = 0.0f; dT[2] = 0.0f;
}
"""
    f = degpu_mod.ODEFunction(base_src + jac_src, 3, 3, jac=True, tgrad=True)  # lorenz_jac / lorenz_tgrad
    prob = degpu_mod.ODEProblem(f, np.array([1, 0, 0], np.float32), (0.0, 10.0), base)
    ps = (rng.random((B, 3)).astype(np.float32) * base).astype(np.float32)
    probs = [degpu_mod.make_prob_compatible(degpu_mod.remake(prob, p=ps[i])) for i in range(B)]
    gpu_probs = degpu_mod.adapt(0, probs)
    a = getattr(degpu_mod, alg)()
    oalg = {"GPUTsit5": "tsit5", "GPUVern7": "vern7", "GPUVern9": "vern9", "GPURosenbrock23": "rosenbrock23",
            "GPURodas4": "rodas4"}[alg]
    u0 = np.tile(np.array([1, 0, 0], np.float32), (B, 1))
    for adaptive, fn in ((False, degpu_mod.vectorized_solve), (True, degpu_mod.vectorized_asolve)):
        ts, us = fn(gpu_probs, prob, a, save_everystep=False, dt=0.1)  # fast mode: every member finite
        assert torch.isfinite(us[:, 1]).all()
        ts, us = fn(gpu_probs, prob, a, save_everystep=False, dt=0.1, mode="parity")
        kw = dict(abstol=1e-6, reltol=1e-3) if adaptive else {}
        ots, ous, _, _, _ = oracle_mod.solve("lorenz", oalg, u0, ps, [0.0, 10.0], adaptive=adaptive,
                                             dt=float(np.float32(0.1)), L=2, jac="analytic", **kw)
        assert_bit_equal(us.cpu().numpy(), ous, f"us ({'asolve' if adaptive else 'solve'})")
        assert_bit_equal(ts.cpu().numpy(), ots, "ts")
