"""Longest-first visiting order for the persistent driver (degpu_work_order, options.order,
degpu_learned_asolve_ex) and the learned work model.

Bars: the order is a permutation that lists the trajectories by non-increasing work
class; a solve in any visiting order is bit-identical to the solve in index order (each
trajectory's arithmetic does not depend on which lane or warp runs it); entries outside
[0, B) are skipped; the work model predicts attempts well enough to order by them.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _order(degpu_mod, work_np):
    import torch
    from degpu import learned
    w = torch.as_tensor(np.asarray(work_np, np.float32), device="cuda")
    o = learned.work_order(w)
    torch.cuda.synchronize()
    return o.cpu().numpy()


@pytest.mark.parametrize("B", [1, 17, 2048, 2048 * 8 + 5, 300_001])
def test_work_order_is_a_longest_first_permutation(degpu_mod, B):
    rng = np.random.default_rng(B)
    w = np.exp(rng.uniform(-1.0, 12.0, B)).astype(np.float32)  # below 1 .. ~1.6e5 attempts
    if B > 20:
        w[:5] = [np.nan, 0.0, -3.0, np.inf, 2.0 ** 40]  # NaN / < 1 -> lowest class; huge -> top class
    o = _order(degpu_mod, w)
    assert np.array_equal(np.sort(o), np.arange(B)), "not a permutation"
    # consecutive entries: the later one exceeds the earlier one by less than one class
    # (2^(1/4), both in the same class), never more; NaN and < 1 count as 1 (class 0), and
    # everything from 2^31.75 up as 2^31.75 (class 127)
    v = w[o].astype(np.float64)
    v = np.where(np.isnan(v) | (v < 1.0), 1.0, np.minimum(v, 2.0 ** 31.75))
    assert np.all(v[1:] <= v[:-1] * 2.0 ** 0.25 * (1 + 1e-5))
    if B > 20:
        assert set(o[:2].tolist()) == {3, 4}  # inf and 2^40 lead


def test_work_order_empty(degpu_mod):
    import torch
    from degpu import learned
    o = learned.work_order(torch.empty(0, dtype=torch.float32, device="cuda"))
    assert o.numel() == 0


def _lorenz_probs(degpu_mod, B, seed=3):
    import torch
    rng = np.random.default_rng(seed)
    p = (rng.random((B, 3)) * np.array([10, 28, 8 / 3])).astype(np.float32)
    u0 = (np.array([1, 0, 0]) + rng.normal(0, 0.1, (B, 3))).astype(np.float32)
    f = degpu_mod.ODEFunction.builtin("lorenz")
    tsp = np.tile(np.array([0.0, 10.0]), (B, 1))
    return f, u0, p, degpu_mod.DeviceProblems(f, u0, p, tsp, np.float64, torch.device("cuda", 0))


def _solve(degpu_mod, probs, **kw):
    import torch
    r = degpu_mod.api._solve_device(probs, degpu_mod.GPUTsit5(), True, dt=0.1, abstol=1e-8, reltol=1e-6,
                                    saveat=np.arange(0.0, 10.0 + 1e-9, 0.5), driver="persistent", **kw)
    torch.cuda.synchronize()
    return [x.cpu().numpy() for x in (r.ts, r.us, r.retcode, r.naccept, r.nreject)]


def _same(a, b):
    """(ts, us, retcode, naccept, nreject) bit-identical; saved rows compared for the
    trajectories that succeeded (a failed one leaves rows it never reached unwritten)."""
    assert np.array_equal(a[2], b[2]) and np.array_equal(a[3], b[3]) and np.array_equal(a[4], b[4])
    ok = a[2] == 1
    assert ok.mean() > 0.99
    for x, y in zip(a[:2], b[:2]):
        assert np.array_equal(np.ascontiguousarray(x[ok]).view(np.uint8), np.ascontiguousarray(y[ok]).view(np.uint8))


@pytest.mark.parametrize("mode", ["fast", "parity"])
def test_solve_in_any_order_is_bit_identical(degpu_mod, mode):
    import torch
    B = 20_000
    f, u0, p, probs = _lorenz_probs(degpu_mod, B)
    base = _solve(degpu_mod, probs, mode=mode)
    rng = np.random.default_rng(1)
    for perm in (np.arange(B)[::-1], rng.permutation(B)):
        o = torch.as_tensor(np.ascontiguousarray(perm, np.int32), device="cuda")
        _same(base, _solve(degpu_mod, probs, mode=mode, order=o))
    # longest-first by the true attempts
    o = torch.as_tensor(_order(degpu_mod, (base[3] + base[4]).astype(np.float32)), device="cuda")
    _same(base, _solve(degpu_mod, probs, mode=mode, order=o))


def test_order_entries_outside_the_batch_are_skipped(degpu_mod):
    import torch
    B = 4096
    f, u0, p, probs = _lorenz_probs(degpu_mod, B)
    base = _solve(degpu_mod, probs)
    perm = np.arange(B, dtype=np.int32)
    skipped = [5, 77, 4095]
    perm[skipped] = [-1, B, 1 << 30]
    r = _solve(degpu_mod, probs, order=torch.as_tensor(perm, device="cuda"))
    keep = np.setdiff1d(np.arange(B), skipped)
    assert np.all(r[2][skipped] == 0)  # never run: retcode left at its zero fill
    assert np.array_equal(r[1][keep].view(np.uint32), base[1][keep].view(np.uint32))
    assert np.array_equal(r[3][keep], base[3][keep])


def test_work_model_and_learned_asolve_ex(degpu_mod):
    """A work model trained on the plain solver's attempts predicts them (held-out
    correlation of log attempts); degpu_learned_asolve_ex with it gives the plain results,
    and with a step model too gives degpu_learned_asolve's results."""
    import torch
    from degpu import _lib, learned
    B = 65_536
    f, u0, p, probs = _lorenz_probs(degpu_mod, B, seed=11)
    wm, info = learned.fit_work_model(f, u0, p, (0.0, 10.0), np.float64, degpu_mod.GPUTsit5(), reltol=1e-6,
                                      abstol=1e-8, epochs=6)
    assert info["holdout_corr_log_attempts"] > 0.9, info
    sa = torch.as_tensor(np.arange(0.0, 10.0 + 1e-9, 0.5), device="cuda")
    L = sa.numel()
    st = torch.cuda.current_stream()

    def run(m, w):
        ts = torch.empty((B, L), dtype=torch.float64, device="cuda")
        us = torch.empty((B, L, 3), dtype=torch.float32, device="cuda")
        rc = torch.zeros(B, dtype=torch.int8, device="cuda")
        na = torch.zeros(B, dtype=torch.int32, device="cuda")
        nr = torch.zeros(B, dtype=torch.int32, device="cuda")
        out = _lib.Outputs(ts.data_ptr(), us.data_ptr(), L, rc.data_ptr(), na.data_ptr(), nr.data_ptr(), None)
        opt = degpu_mod.api._options(degpu_mod.GPUTsit5(), np.float64, dt=0.1, abstol=1e-8, reltol=1e-6,
                                     saveat_dev=sa.data_ptr(), nsaveat=L, driver="persistent")
        pr = probs.cstruct()
        if m is not None and w is None:
            rcode = _lib.lib().degpu_learned_asolve(f.handle(), m.h, ctypes.byref(pr), ctypes.byref(opt), 1e-8, 1e3,
                                                    1e3, ctypes.byref(out), ctypes.c_void_p(st.cuda_stream))
        else:
            rcode = _lib.lib().degpu_learned_asolve_ex(f.handle(), None if m is None else m.h,
                                                       None if w is None else w.h, ctypes.byref(pr),
                                                       ctypes.byref(opt), 1e-8, 1e3, 1e3, ctypes.byref(out),
                                                       ctypes.c_void_p(st.cuda_stream))
        _lib.check(rcode)
        torch.cuda.synchronize()
        return [x.cpu().numpy() for x in (ts, us, rc, na, nr)]

    plain = _solve(degpu_mod, probs)
    _same(plain, run(None, wm))
    sm, _ = learned.fit_step_model(f, u0[:16384], p[:16384], (0.0, 10.0), np.float64, degpu_mod.GPUTsit5(),
                                   reltol=1e-6, abstol=1e-8, epochs=2)
    _same(run(sm, None), run(sm, wm))


def test_work_model_with_per_trajectory_spans(degpu_mod):
    """With per-trajectory tspans the work model also reads the span tf - t0 (input width
    N + P + 2, fed from the tspan array inside the library); the ordered solve through
    _solve_device(work_model=...) equals the index-order solve."""
    import torch
    rng = np.random.default_rng(5)
    B = 65_536
    p = np.stack([np.full(B, 10.0), rng.uniform(0, 100, B), np.full(B, 8 / 3)], 1).astype(np.float32)
    u0 = np.tile(np.array([1, 0, 0], np.float32), (B, 1))
    tsp = np.stack([np.zeros(B), rng.uniform(1, 20, B)], 1)
    f = degpu_mod.ODEFunction.builtin("lorenz")
    from degpu import learned
    wm, info = learned.fit_work_model(f, u0, p, tsp, np.float64, degpu_mod.GPUTsit5(), reltol=1e-6, abstol=1e-8,
                                      epochs=6)
    assert wm.n_in == 3 + 3 + 2
    assert info["holdout_corr_log_attempts"] > 0.9, info
    probs = degpu_mod.DeviceProblems(f, u0, p, tsp, np.float64, torch.device("cuda", 0))

    def run(**kw):
        r = degpu_mod.api._solve_device(probs, degpu_mod.GPUTsit5(), True, dt=0.1, abstol=1e-8, reltol=1e-6,
                                        driver="persistent", **kw)
        torch.cuda.synchronize()
        return [x.cpu().numpy() for x in (r.ts, r.us, r.retcode, r.naccept, r.nreject)]
    _same(run(), run(work_model=wm))
