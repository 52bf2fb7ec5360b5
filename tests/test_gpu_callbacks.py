"""tstops and GPU callbacks (continuous with ITP root finding, discrete, terminate!) through
the C ABI, bit-identical to the oracle in parity mode.

Cases follow the reference's callback tests: the bouncing ball of
test/gpu_kernel_de/gpu_ode_continuous_callbacks.jl (condition u[1], affect! u += (0,-2).*u,
tspan (0, 15), plain / CallbackSet(cb, cb) / saveat [0, 9.1] / save_everystep=false, fixed
and adaptive) and the decay problem of test/gpu_kernel_de/gpu_ode_discrete_callbacks.jl
(events at t == 2.4 and t == 4.0 reached through tstops), with GPURosenbrock23 / GPURodas5P
for the stiff variants (stiff_ode/gpu_ode_*_callbacks.jl).  The reference compares against
CPU OrdinaryDiffEq solves with tolerances of 2e-6 .. 1e-2; here the bar is the oracle bit for
bit, plus the analytic solution with the reference's tolerances."""
import numpy as np
import pytest

from test_gpu_parity import assert_bit_equal, assert_saved_equal

pytestmark = pytest.mark.gpu

EPS32 = float(np.finfo(np.float32).eps)
ALGS = {"tsit5": "GPUTsit5", "vern7": "GPUVern7", "rosenbrock23": "GPURosenbrock23", "rodas5p": "GPURodas5P",
        "rodas4": "GPURodas4", "vern9": "GPUVern9", "kvaerno3": "GPUKvaerno3", "kvaerno5": "GPUKvaerno5"}


def run_pair(degpu, oracle, model, alg, u0, p, tspan, tt, *, adaptive, dt, callbacks, tstops=None, saveat=None,
             save_everystep=None, mode="parity", driver="auto", **kw):
    """Solve on the GPU through the public API and with the oracle on the same inputs."""
    import torch
    f = degpu.ODEFunction.builtin(model)
    B = u0.shape[0]
    tsp = np.broadcast_to(np.asarray(tspan, dtype=tt), (B, 2))
    probs = degpu.DeviceProblems(f, u0, p, tsp, tt, torch.device("cuda", 0))
    if save_everystep is None:
        save_everystep = not adaptive
    cs = degpu.CallbackSet(*callbacks)
    r = degpu.api._solve_device(probs, getattr(degpu, ALGS[alg])(), adaptive, dt=dt, saveat=saveat,
                                save_everystep=save_everystep, callback=cs, tstops=tstops, mode=mode, driver=driver,
                                **kw)
    torch.cuda.synchronize()
    g = [r.ts.cpu().numpy(), r.us.cpu().numpy(), r.retcode.cpu().numpy(), r.naccept.cpu().numpy()]
    L = g[0].shape[1]
    ccb = [(c.fn, c.affect, c.affect_neg, {"LeftRootFind": 0, "RightRootFind": 1, "NoRootFind": 2}[c.rootfind],
            c.abstol, c.repeat_nudge, c.dtrelax) for c in cs.continuous]
    dcb = [d.fn for d in cs.discrete]
    okw = {k: v for k, v in kw.items() if k in ("abstol", "reltol")}
    o = oracle.solve(model, alg, u0, p, list(tspan), adaptive=adaptive, dt=float(tt(dt)), L=L, saveat=saveat,
                     save_everystep=save_everystep, time_f64=tt == np.float64, tstops=tstops, ccb=ccb, dcb=dcb, **okw)
    return g, o


def check_parity(g, o):
    ts, us, rc, na = g
    ots, ous, orc, ona = o[:4]
    assert_bit_equal(ts, ots, "ts")
    assert_saved_equal(us, ous, ts, ts[:, :1])
    assert (rc == orc).all(), (rc, orc)
    assert (na == ona).all(), (na, ona)


def ball_batch(B, seed=0, vary=False):
    u0 = np.tile(np.array([45.0, 0.0], np.float32), (B, 1))
    p = np.full((B, 1), 10.0, np.float32)
    if vary:
        rng = np.random.default_rng(seed)
        u0[:, 0] = rng.uniform(5.0, 50.0, B).astype(np.float32)
        p[:, 0] = rng.uniform(5.0, 15.0, B).astype(np.float32)
    return u0, p


def ball_exact(h0, g, t):
    """Height and velocity of the elastic bouncing ball at time t."""
    T = np.sqrt(2 * h0 / g)            # first contact
    if t < T:
        return np.array([h0 - 0.5 * g * t * t, -g * t])
    period = 2 * T
    s = (t - T) % period                # time since the last contact
    v0 = g * T
    return np.array([v0 * s - 0.5 * g * s * s, v0 - g * s])


# ----------------------------------------------------------------------------- continuous
@pytest.mark.parametrize("alg", ["tsit5", "vern7", "vern9"])
@pytest.mark.parametrize("adaptive", [False, True])
@pytest.mark.parametrize("tt", [np.float32, np.float64])
def test_bouncing_ball_parity(degpu_mod, oracle_mod, alg, adaptive, tt):
    """gpu_ode_continuous_callbacks.jl: ContinuousCallback(condition, affect!), dt 0.1f0."""
    u0, p = ball_batch(2)
    cb = degpu_mod.ContinuousCallback(0)
    kw = dict(abstol=1e-6, reltol=1e-3) if adaptive else {}
    g, o = run_pair(degpu_mod, oracle_mod, "ball", alg, u0, p, (0.0, 15.0), tt, adaptive=adaptive, dt=0.1,
                    callbacks=[cb], save_everystep=False if adaptive else True, **kw)
    check_parity(g, o)
    # the reference's tolerance against a CPU solve (1e-2 adaptive, 2e-3 fixed) -- here against
    # the exact bounce: contact at t = 3, 9, 15 with |v| = 30
    # (the last contact is at t = 15 itself: the final velocity is -30 or, if the located root
    # falls just before 15, +30 after the bounce)
    fin = g[1][0, -1]
    assert abs(fin[0]) < 5e-2 and abs(abs(fin[1]) - 30.0) < 5e-2, fin


@pytest.mark.parametrize("adaptive", [False, True])
def test_callbackset_saveat_save_everystep(degpu_mod, oracle_mod, adaptive):
    """CallbackSet(cb, cb); saveat [0, 9.1]; save_everystep=false (the reference's sub-cases)."""
    u0, p = ball_batch(2)
    cb = degpu_mod.ContinuousCallback(0)
    dt = 0.1 if adaptive else 1.0
    kw = dict(abstol=1e-6, reltol=1e-6) if adaptive else {}
    for cbs, saveat, sev in (([cb, cb], None, None), ([cb, cb], np.array([0.0, 9.1]), None), ([cb], None, False)):
        g, o = run_pair(degpu_mod, oracle_mod, "ball", "tsit5", u0, p, (0.0, 15.0), np.float32, adaptive=adaptive,
                        dt=dt if saveat is not None else 0.1, callbacks=cbs, saveat=saveat,
                        save_everystep=sev, **kw)
        check_parity(g, o)


def test_bouncing_ball_ensemble_parity_and_physics(degpu_mod, oracle_mod):
    """20,000 balls of different heights and gravities, adaptive Tsit5 + saveat, persistent
    driver: bit parity with the oracle and every saved point close to the exact bounce."""
    u0, p = ball_batch(20_000, seed=3, vary=True)
    sa = np.linspace(0.0, 12.0, 25)
    cb = degpu_mod.ContinuousCallback(0)
    g, o = run_pair(degpu_mod, oracle_mod, "ball", "tsit5", u0, p, (0.0, 12.0), np.float64, adaptive=True, dt=0.01,
                    callbacks=[cb], saveat=sa, abstol=1e-7, reltol=1e-7, driver="persistent")
    check_parity(g, o)
    us = g[1]
    for i in range(0, 20_000, 997):
        ex = np.stack([ball_exact(float(u0[i, 0]), float(p[i, 0]), t) for t in sa])
        assert np.abs(us[i] - ex).max() < 2e-2 * max(1.0, np.abs(ex).max() / 10), i


def test_terminate_and_rootfind_modes(degpu_mod, oracle_mod):
    """terminate! from a continuous affect (retcode Terminated, final state at the contact);
    RightRootFind and NoRootFind event placement."""
    u0, p = ball_batch(64, seed=4, vary=True)
    term = degpu_mod.ContinuousCallback(1)
    g, o = run_pair(degpu_mod, oracle_mod, "ball", "tsit5", u0, p, (0.0, 20.0), np.float32, adaptive=True, dt=0.1,
                    callbacks=[term], abstol=1e-7, reltol=1e-6)
    check_parity(g, o)
    assert (g[2] == 2).all()  # Terminated
    T = np.sqrt(2 * u0[:, 0] / p[:, 0])
    assert np.abs(g[0][:, 1] - T).max() < 1e-4
    for rf in ("RightRootFind", "NoRootFind"):
        cb = degpu_mod.ContinuousCallback(0, rootfind=rf)
        g, o = run_pair(degpu_mod, oracle_mod, "ball", "tsit5", u0, p, (0.0, 10.0), np.float32, adaptive=True,
                        dt=0.1, callbacks=[cb], abstol=1e-7, reltol=1e-6)
        check_parity(g, o)


@pytest.mark.parametrize("alg", ["rosenbrock23", "rodas5p", "rodas4", "kvaerno3", "kvaerno5"])
@pytest.mark.parametrize("adaptive", [False, True])
def test_stiff_bouncing_ball_parity(degpu_mod, oracle_mod, alg, adaptive):
    """stiff_ode/gpu_ode_continuous_callbacks.jl: tspan (0, 16.5), dt 0.1f0."""
    u0, p = ball_batch(2)
    cb = degpu_mod.ContinuousCallback(0)
    kw = dict(abstol=1e-6, reltol=1e-3) if adaptive else {}
    g, o = run_pair(degpu_mod, oracle_mod, "ball", alg, u0, p, (0.0, 16.5), np.float32, adaptive=adaptive, dt=0.1,
                    callbacks=[cb], save_everystep=False if adaptive else True, **kw)
    check_parity(g, o)
    # exact state at 16.5: 1.5 s after the contact at t = 15
    ex = ball_exact(45.0, 10.0, 16.5)
    assert np.linalg.norm(g[1][0, -1] - ex) < 0.5


# ----------------------------------------------------------------------------- discrete
@pytest.mark.parametrize("alg", ["tsit5", "vern7", "rosenbrock23", "rodas5p", "rodas4", "vern9", "kvaerno3",
                                 "kvaerno5"])
def test_discrete_tstops_parity(degpu_mod, oracle_mod, alg):
    """gpu_ode_discrete_callbacks.jl: condition t == 2.4f0 with tstops [2.4f0], dt 1f0; the
    dt 0.01f0 / tstops [4.0f0] truncation case; CallbackSet at 2.4 and 4.0 with saveat [0, 6]
    and with save_everystep=false; adaptive with tstops [4.0f0]."""
    u0 = np.full((2, 1), 10.0, np.float32)
    p = np.ones((2, 1), np.float32)
    c0, c1 = degpu_mod.DiscreteCallback(0), degpu_mod.DiscreteCallback(1)
    cases = [
        dict(adaptive=False, dt=1.0, callbacks=[c0], tstops=[2.4]),
        dict(adaptive=False, dt=0.01, callbacks=[c1], tstops=[4.0]),
        dict(adaptive=False, dt=1.0, callbacks=[c0, c1], tstops=[2.4, 4.0]),
        dict(adaptive=False, dt=1.0, callbacks=[c0, c1], tstops=[2.4, 4.0], saveat=np.array([0.0, 6.0])),
        dict(adaptive=False, dt=1.0, callbacks=[c0, c1], tstops=[2.4, 4.0], save_everystep=False),
        dict(adaptive=True, dt=1.0, callbacks=[c1], tstops=[4.0], abstol=1e-6, reltol=1e-3),
        dict(adaptive=True, dt=1.0, callbacks=[c0, c1], tstops=[2.4, 4.0], saveat=np.array([0.0, 6.0]),
             abstol=1e-7, reltol=1e-6),
    ]
    for c in cases:
        g, o = run_pair(degpu_mod, oracle_mod, "decay", alg, u0, p, (0.0, 10.0), np.float32, **c)
        check_parity(g, o)
        if alg.startswith("kvaerno") and not c["adaptive"]:
            # the reference's fixed-step ESDIRKs solve a step clipped to a tstop with the
            # unclipped dt in their Newton iteration (gpu_kvaerno3_perform_step.jl:34-38), so
            # only parity is checked there
            continue
        # exact: u = 10 e^{-t} plus 10 e^{-(t - s)} for each event s <= t
        ev = [2.4 if cb.fn == 0 else 4.0 for cb in c["callbacks"]]
        ts, us = g[0][0], g[1][0, :, 0]
        n = len(ts) if c.get("save_everystep", True) or c.get("saveat") is not None else 2
        for l in range(n):
            t = float(ts[l])
            # a row saved at an event time holds the value before the affect
            exact = 10 * np.exp(-t) + sum(10 * np.exp(-(t - s)) for s in ev if s < t - 1e-5)
            rt = {"tsit5": 5e-3, "vern7": 5e-3, "rosenbrock23": 0.15, "rodas5p": 2e-2, "rodas4": 2e-2, "vern9": 5e-3,
                  "kvaerno3": 0.1, "kvaerno5": 2e-2}[alg]  # fixed dt 1 on u' = -u
            assert abs(us[l] - exact) < rt * max(1.0, exact), (c, l, t, us[l], exact)


@pytest.mark.parametrize("tt", [np.float32, np.float64])
def test_discrete_terminate_and_time_types(degpu_mod, oracle_mod, tt):
    """terminate! from a discrete affect (u < 1 after t ~ 2.3); FP64 time with tstops."""
    u0 = np.full((128, 1), 10.0, np.float32)
    p = np.linspace(0.5, 2.0, 128, dtype=np.float32)[:, None]
    for adaptive in (False, True):
        kw = dict(abstol=1e-7, reltol=1e-6) if adaptive else {}
        g, o = run_pair(degpu_mod, oracle_mod, "decay", "tsit5", u0, p, (0.0, 10.0), tt, adaptive=adaptive,
                        dt=0.05, callbacks=[degpu_mod.DiscreteCallback(2)], save_everystep=False, **kw)
        check_parity(g, o)
        assert (g[2] == 2).all()
        assert (g[1][:, 1, 0] < 1.0).all()
        g, o = run_pair(degpu_mod, oracle_mod, "decay", "tsit5", u0, p, (0.0, 10.0), tt, adaptive=adaptive,
                        dt=0.05, callbacks=[degpu_mod.DiscreteCallback(0), degpu_mod.DiscreteCallback(1)],
                        tstops=[2.4, 4.0], save_everystep=False, **kw)
        check_parity(g, o)
        assert (g[2] == 1).all()


def test_fast_mode_callbacks_close_to_oracle(degpu_mod, oracle_mod):
    """Fast mode (FMA, approximate division): same events, results within 1e-3."""
    u0, p = ball_batch(4096, seed=7, vary=True)
    cb = degpu_mod.ContinuousCallback(0)
    g, o = run_pair(degpu_mod, oracle_mod, "ball", "tsit5", u0, p, (0.0, 10.0), np.float64, adaptive=True, dt=0.01,
                    callbacks=[cb], saveat=np.linspace(0, 10, 11), abstol=1e-7, reltol=1e-7, mode="fast")
    assert (g[2] == 1).all()
    scale = np.maximum(1.0, np.abs(o[1]))
    assert np.abs(g[1] - o[1]).max() / scale.max() < 1e-3 or np.abs((g[1] - o[1]) / scale).max() < 1e-3


def test_tstops_without_callbacks_and_plain_kernels_unchanged(degpu_mod, oracle_mod):
    """tstops alone (no callbacks) for fixed and adaptive steps; a solve without tstops or
    callbacks still matches the oracle (the callback code is compiled out of it)."""
    from test_gpu_parity import lorenz_batch
    u0, p = lorenz_batch(1000, seed=8)
    for adaptive in (False, True):
        kw = dict(abstol=1e-8, reltol=1e-6) if adaptive else {}
        g, o = run_pair(degpu_mod, oracle_mod, "lorenz", "tsit5", u0, p, (0.0, 2.0), np.float32, adaptive=adaptive,
                        dt=0.1, callbacks=[], tstops=[0.55, 1.25, 1.3], save_everystep=False, **kw)
        check_parity(g, o)
        g, o = run_pair(degpu_mod, oracle_mod, "lorenz", "tsit5", u0, p, (0.0, 2.0), np.float32, adaptive=adaptive,
                        dt=0.1, callbacks=[], save_everystep=False, **kw)
        check_parity(g, o)


def test_callback_argument_errors(degpu_mod):
    with pytest.raises(ValueError, match="save_positions"):
        degpu_mod.ContinuousCallback(0, save_positions=(True, False))
    with pytest.raises(ValueError, match="save_positions"):
        degpu_mod.DiscreteCallback(0, save_positions=(False, True))
    with pytest.raises(ValueError):
        degpu_mod.CallbackSet(*[degpu_mod.DiscreteCallback(0)] * 9)
