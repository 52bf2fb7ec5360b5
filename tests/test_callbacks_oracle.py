"""The oracle's tstops / callback restatement (integrator_utils.jl:52-479) against exact
answers, and the callback API's host-side checks -- CPU only."""
import numpy as np
import pytest

EPS32 = float(np.finfo(np.float32).eps)
CB = (0, True, True, 0, 100 * EPS32, 0.01, 1.0)  # bounce, LeftRootFind, converted-ContinuousCallback abstol


@pytest.mark.parametrize("alg", ["tsit5", "vern7", "rosenbrock23", "rodas5p"])
def test_oracle_bouncing_ball_exact(oracle_mod, alg):
    """Elastic ball from 45 m, g = 10: contacts at 3, 9, 15 s with |v| = 30 m/s."""
    u0 = np.array([[45.0, 0.0]], np.float32)
    p = np.array([[10.0]], np.float32)
    sa = np.array([0.0, 3.0, 6.0, 9.0, 12.0, 14.0])
    ts, us, rc, na, nr = oracle_mod.solve("ball", alg, u0, p, [0.0, 14.0], adaptive=True, dt=0.1, L=6, saveat=sa,
                                          abstol=1e-8, reltol=1e-8, ccb=[CB])
    exact = np.array([[45, 0], [0, -30], [45, 0], [0, -30], [45, 0], [25, -20]], np.float64)
    tol = {"tsit5": 2e-2, "vern7": 2e-2, "rosenbrock23": 0.5, "rodas5p": 5e-2}[alg]
    assert rc[0] == 1
    # contact rows (t = 3, 9): height ~ 0 and |v| = 30 -- the row is saved just before or just
    # after the bounce depending on which side of the save time the located root falls
    contact = [1, 3]
    free = [0, 2, 4, 5]
    assert np.abs(us[0, free] - exact[free]).max() < tol, us[0]
    assert np.abs(us[0, contact, 0]).max() < tol and np.abs(np.abs(us[0, contact, 1]) - 30).max() < tol, us[0]


def test_oracle_event_without_affect_is_ignored(oracle_mod):
    """affect! = nothing and affect_neg! = nothing: the ball falls through the floor."""
    u0 = np.array([[45.0, 0.0]], np.float32)
    p = np.array([[10.0]], np.float32)
    ts, us, rc, _, _ = oracle_mod.solve("ball", "tsit5", u0, p, [0.0, 5.0], adaptive=True, dt=0.1, L=2,
                                        abstol=1e-8, reltol=1e-8, ccb=[(0, False, False, 0, 1e-5, 0.01, 1.0)])
    assert abs(us[0, 1, 0] - (45 - 5 * 25)) < 1e-3 and rc[0] == 1


def test_oracle_terminate(oracle_mod):
    u0 = np.array([[20.0, 0.0]], np.float32)
    p = np.array([[9.81]], np.float32)
    ts, us, rc, _, _ = oracle_mod.solve("ball", "tsit5", u0, p, [0.0, 10.0], adaptive=True, dt=0.1, L=2,
                                        abstol=1e-8, reltol=1e-8, ccb=[(1, True, True, 0, 1e-5, 0.01, 1.0)])
    assert rc[0] == 2  # Terminated
    assert abs(ts[0, 1] - np.sqrt(2 * 20 / 9.81)) < 1e-5
    assert abs(us[0, 1, 0]) < 1e-4


@pytest.mark.parametrize("time_f64", [False, True])
def test_oracle_discrete_tstops_fixed(oracle_mod, time_f64):
    """t == 2.4 with tstops [2.4], dt 1: the grid is 0, 1, 2, 2.4, 3.4, ... and u jumps by 10
    after the saved pre-affect value at 2.4 (gpu_ode_discrete_callbacks.jl:26-44)."""
    u0 = np.full((1, 1), 10.0, np.float32)
    p = np.ones((1, 1), np.float32)
    ts, us, rc, na, _ = oracle_mod.solve("decay", "tsit5", u0, p, [0.0, 10.0], adaptive=False, dt=1.0, L=12,
                                         save_everystep=True, tstops=[2.4], dcb=[0], time_f64=time_f64)
    grid = np.array([0, 1, 2, 2.4, 3.4, 4.4, 5.4, 6.4, 7.4, 8.4, 9.4, 10])
    assert np.abs(ts[0] - grid).max() < 1e-5
    exact = np.array([10 * np.exp(-t) + (10 * np.exp(-(t - 2.4)) if t > 2.4 + 1e-6 else 0) for t in grid])
    assert np.abs(us[0, :, 0] - exact).max() < 5e-3 * 10


def test_oracle_adaptive_tstop_snaps(oracle_mod):
    """Adaptive steps stop exactly on every tstop (u interpolated there) and keep going."""
    u0 = np.full((1, 1), 10.0, np.float32)
    p = np.ones((1, 1), np.float32)
    stops = [0.3, 1.7, 4.0]
    ts, us, rc, na, _ = oracle_mod.solve("decay", "tsit5", u0, p, [0.0, 10.0], adaptive=True, dt=1.0, L=2,
                                         tstops=stops, dcb=[1], abstol=1e-8, reltol=1e-8)
    assert rc[0] == 1
    assert abs(us[0, 1, 0] - (10 * np.exp(-10) + 10 * np.exp(-6))) < 1e-5


def test_itp_helpers_match_julia_semantics(oracle_mod):
    """Host copies of eps/nextfloat used by the root finder behave like Julia's (the oracle
    exports none of them directly; this pins them through numpy's definitions)."""
    for x in (1.0, 3.0, 1e-30, 2.0 ** -127):
        e = np.spacing(np.float32(x))
        assert e > 0
    assert np.nextafter(np.float32(0), np.float32(1)) == np.float32(2.0 ** -149)


def test_callback_api_host_checks(degpu_mod):
    d = degpu_mod
    cs = d.CallbackSet(d.ContinuousCallback(0), d.CallbackSet(d.DiscreteCallback(1), d.ContinuousCallback(2)))
    assert [c.fn for c in cs.continuous] == [0, 2] and [c.fn for c in cs.discrete] == [1]
    st, keep = cs.cstruct()
    assert st.n_continuous == 2 and st.n_discrete == 1
    assert st.continuous[1].fn == 2 and st.discrete[0] == 1
    c = d.ContinuousCallback(0, affect=True)
    assert c.affect_neg and abs(c.abstol - 100 * EPS32) < 1e-12
    assert abs(d.GPUContinuousCallback(0).abstol - 10 * EPS32) < 1e-12
    assert not d.ContinuousCallback(0, affect=False).affect_neg
    with pytest.raises(ValueError):
        d.ContinuousCallback(0, rootfind="Sideways")
    from degpu.api import tstops_extra_length
    assert tstops_extra_length((0.0, 10.0), 1.0, [2.4], np.float32) == 1
    assert tstops_extra_length((0.0, 10.0), 1.0, [2.4, 4.0], np.float32) == 1
