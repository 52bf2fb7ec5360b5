"""Host-side logic of the learned parts (no GPU): feature layout (with and without the span
input), the tolerance-scale targets, the scheduling simulation that motivates the
longest-first order, and the ABI of the models' entry points."""
import numpy as np


def test_features_layout(degpu_mod):
    from degpu import learned
    u0 = np.arange(6, dtype=np.float32).reshape(2, 3)
    p = np.arange(6, 12, dtype=np.float32).reshape(2, 3)
    x = learned.features(u0, p, 1e-6)
    assert x.shape == (2, 7) and x.dtype == np.float32
    assert np.array_equal(x[:, :3], u0) and np.array_equal(x[:, 3:6], p) and np.allclose(x[:, 6], -6.0)
    xs = learned.features(u0, p, np.array([1e-6, 1e-3]), span=np.array([10.0, 2.5]))
    assert xs.shape == (2, 8) and np.allclose(xs[:, 6], [-6.0, -3.0]) and np.allclose(xs[:, 7], [10.0, 2.5])


def test_scale_targets_monotone_prefix(degpu_mod):
    """The target scale is the largest s whose error and every smaller scale's error stay
    under the target; a member that misses it at s = 1 keeps s = 1."""
    from degpu import learned
    scales = (1, 2, 4, 8)
    errs = np.array([[1e-6, 1e-6, 1e-3, 1e-6],     # s = 1
                     [2e-6, 1e-6, 1e-3, 1e-6],     # s = 2
                     [9e-6, 5e-5, 1e-3, 1e-6],     # s = 4
                     [1e-6, 1e-6, 1e-3, 1e-6]])    # s = 8 (below target again after a miss)
    s = learned.scale_targets(errs, scales, 1e-5)
    assert s.tolist() == [8.0, 2.0, 1.0, 8.0]


def _drain_sim(att, W, chunk=32):
    """Warp-iteration count of the persistent driver's schedule (each warp claims `chunk`
    trajectories, a lane refills as soon as its trajectory ends, all warps step together)."""
    B = len(att)
    rem = np.zeros((W, 32), np.int64)
    qn = np.zeros(W, np.int64)
    qe = np.zeros(W, np.int64)
    g = 0
    iters = np.zeros(W, np.int64)
    alive = np.ones(W, bool)
    while alive.any():
        for w in np.nonzero(alive)[0]:
            idle = np.nonzero(rem[w] == 0)[0]
            if len(idle):
                if qn[w] >= qe[w] and g < B:
                    qn[w], qe[w] = g, min(g + chunk, B)
                    g = qe[w]
                k = min(len(idle), qe[w] - qn[w])
                rem[w, idle[:k]] = att[qn[w]:qn[w] + k]
                qn[w] += k
        act = rem > 0
        alive = act.any(1) | (qn < qe) | (g < B)
        iters += alive
        rem[act] -= 1
    return iters.max(), att.sum() / 32 / W


def test_longest_first_shortens_the_drain():
    """With step counts spread like the adaptive Lorenz ensemble's (27..484, mean ~190),
    index order leaves a long drain; longest-first visiting brings the last warp's
    iterations close to the balanced ideal -- the reason for degpu_work_order."""
    rng = np.random.default_rng(0)
    att = np.clip(rng.gamma(4.0, 48.0, 8192), 27, 484).astype(np.int64)
    W = 16
    last_idx, ideal = _drain_sim(att, W)
    last_lpt, _ = _drain_sim(np.sort(att)[::-1].copy(), W)
    assert last_idx > 1.05 * ideal
    assert last_lpt < last_idx and last_lpt < 1.03 * ideal


def test_learned_entry_points_declared(degpu_mod):
    from degpu import _lib
    for name in ("degpu_work_order", "degpu_learned_asolve_ex", "degpu_learned_batch_solve_host",
                 "degpu_learned_asolve", "degpu_learned_asolve_noalloc"):
        assert name in _lib.SIGNATURES and hasattr(degpu_mod.lib(), name)
