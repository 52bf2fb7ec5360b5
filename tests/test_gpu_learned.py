"""Learned step control on the GPU: gradients and tensor-core inference of libdegpu's BF16
MLP against the CPU oracle (oracle/mlp_oracle.py), training convergence, and what the
trained network gains over the plain controller at equal FP64-oracle error."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def model_and_batch(degpu_mod):
    import torch
    from degpu.learned import StepSizeModel
    rng = np.random.default_rng(0)
    m = StepSizeModel(7, seed=3)
    P, _, _, _ = m.get()
    P = (P + rng.normal(0, 0.05, P.shape)).astype(np.float32)  # non-trivial biases too
    mean = rng.normal(0, 1, 7).astype(np.float32)
    std = rng.uniform(0.5, 2, 7).astype(np.float32)
    m.set(P, mean, std)
    x = rng.normal(0, 2, (1000, 7)).astype(np.float32)
    t = rng.normal(0, 1, (1000, 2)).astype(np.float32)
    w = rng.uniform(0, 1, (1000, 2)).astype(np.float32)
    return m, P, mean, std, x, t, w


def test_mlp_gradient_matches_oracle(model_and_batch):
    import torch
    import mlp_oracle
    m, P, mean, std, x, t, w = model_and_batch
    dev = torch.device("cuda", 0)
    loss = m.grad(torch.as_tensor(x, device=dev), torch.as_tensor(t, device=dev), torch.as_tensor(w, device=dev))
    torch.cuda.synchronize()
    _, g, _, _ = m.get()
    lo, go = mlp_oracle.grad(P, mean, std, x.astype(np.float64), t, w)
    assert abs(float(loss) - lo) / lo < 1e-4
    rel = np.linalg.norm(g - go) / np.linalg.norm(go)
    cos = g @ go / np.linalg.norm(g) / np.linalg.norm(go)
    assert rel < 2e-3 and cos > 0.99999, (rel, cos)
    # every parameter block agrees, not just the norm
    for a, b, name in ((0, 448, "W1"), (512, 4608, "W2"), (4672, 4800, "W3")):
        r = np.linalg.norm(g[a:b] - go[a:b]) / np.linalg.norm(go[a:b])
        assert r < 5e-3, (name, r)


def test_mlp_tensor_core_inference_matches_oracle(model_and_batch):
    import torch
    import mlp_oracle
    m, P, mean, std, x, t, w = model_and_batch
    y = m.infer(torch.as_tensor(x, device="cuda"), raw=True).cpu().numpy()
    yo, _ = mlp_oracle.forward(P, mean, std, x.astype(np.float64))
    err = np.abs(y - yo).max() / np.abs(yo).max()
    assert err < 1e-2, err
    # B not a multiple of the 16-row tile
    y2 = m.infer(torch.as_tensor(x[:37], device="cuda"), raw=True).cpu().numpy()
    assert np.array_equal(y2, y[:37])


def test_mlp_training_converges(degpu_mod):
    """Fit a smooth 7 -> 2 map; the GPU-trained network must reach a small loss."""
    import torch
    from degpu.learned import StepSizeModel
    rng = np.random.default_rng(1)
    x = rng.uniform(-1, 1, (65536, 7)).astype(np.float32)
    t = np.stack([np.sin(2 * x[:, 0]) + x[:, 1] * x[:, 2], np.log1p(np.exp(3 * x[:, 3])) - x[:, 6]], 1).astype(np.float32)
    m = StepSizeModel(7, seed=0)
    hist = m.fit(x, t, epochs=12, batch=4096, lr=3e-3)
    print("training loss history", hist)
    assert hist[-1] < 0.1 * hist[0], hist


def test_learned_controller_gains_at_equal_error(degpu_mod, oracle_mod):
    """Train on plain-solver traces of the adaptive Lorenz ensemble (Tsit5, reltol 1e-6),
    evaluate on fresh trajectories: fewer step attempts than the plain controller while the
    FP64 Vern9 final-state error (p90 over members with a stable FP64 solution) stays at the
    plain controller's level."""
    import torch
    from degpu import learned
    rng = np.random.default_rng(7)

    def draw(B):
        p = (rng.random((B, 3)) * np.array([10, 28, 8 / 3])).astype(np.float32)
        u0 = (np.array([1, 0, 0]) + rng.normal(0, 0.1, (B, 3))).astype(np.float32)
        return u0, p
    f = degpu_mod.ODEFunction.builtin("lorenz")
    alg = degpu_mod.GPUTsit5()
    u0, p = draw(65536)
    model, info = learned.fit_step_model(f, u0, p, (0.0, 10.0), np.float64, alg, reltol=1e-6, abstol=1e-8, epochs=6,
                                         log=print)
    ue, pe = draw(4096)
    dev = torch.device("cuda", 0)
    probs = degpu_mod.DeviceProblems(f, ue, pe, np.tile([0.0, 10.0], (4096, 1)), np.float64, dev)
    plain = degpu_mod.api._solve_device(probs, alg, True, dt=0.1, abstol=1e-8, reltol=1e-6)
    x = torch.as_tensor(learned.features(ue, pe, np.full(4096, 1e-6)), device=dev)
    dt0, sc = model.infer(x)
    lrn = degpu_mod.api._solve_device(probs, alg, True, dt=0.1, abstol=1e-8, reltol=1e-6, dt0=dt0, tolscale=sc)
    torch.cuda.synchronize()
    w_plain = (plain.naccept + plain.nreject).sum().item()
    w_lrn = (lrn.naccept + lrn.nreject).sum().item()
    ref, _ = oracle_mod.vern9("lorenz", ue.astype(np.float64), pe.astype(np.float64), 0.0, np.array([10.0]))
    pert, _ = oracle_mod.vern9("lorenz", ue.astype(np.float64) * (1 + 1e-8), pe.astype(np.float64), 0.0, np.array([10.0]))
    ref, pert = ref[:, 0], pert[:, 0]
    nrm = np.maximum(np.linalg.norm(ref, axis=1), 1e-3)
    stable = np.linalg.norm(ref - pert, axis=1) / nrm < 1e-5
    e_plain = np.linalg.norm(plain.us[:, 1].cpu().numpy() - ref, axis=1)[stable] / nrm[stable]
    e_lrn = np.linalg.norm(lrn.us[:, 1].cpu().numpy() - ref, axis=1)[stable] / nrm[stable]
    q_plain, q_lrn = np.quantile(e_plain, 0.9), np.quantile(e_lrn, 0.9)
    print(f"attempts plain {w_plain} learned {w_lrn} ratio {w_plain / w_lrn:.3f}; p90 err plain {q_plain:.3e} "
          f"learned {q_lrn:.3e}; stable {stable.mean():.3f}; {info}")
    assert (lrn.retcode.cpu().numpy() == 1).all()
    assert w_lrn < w_plain  # fewer step attempts than the plain controller ...
    assert q_lrn <= max(1.5 * q_plain, 1e-6) and q_lrn <= 1e-4  # ... at the plain controller's error level


def test_learned_asolve_matches_two_step_path(degpu_mod):
    """degpu_learned_asolve (inference from the problem batch + solve, one C-ABI call) gives
    the same bits as inference on explicit features followed by vectorized_asolve."""
    import ctypes
    import torch
    from degpu import _lib, learned
    rng = np.random.default_rng(11)
    B = 3000
    p = (rng.random((B, 3)) * np.array([10, 28, 8 / 3])).astype(np.float32)
    u0 = (np.array([1, 0, 0]) + rng.normal(0, 0.1, (B, 3))).astype(np.float32)
    m = learned.StepSizeModel(7, seed=5)
    P, _, _, _ = m.get()
    m.set(P, np.concatenate([u0.mean(0), p.mean(0), [-6.0]]), np.concatenate([u0.std(0), p.std(0), [1.0]]))
    m.scale_range = (1.0, 64.0)
    f = degpu_mod.ODEFunction.builtin("lorenz")
    dev = torch.device("cuda", 0)
    probs = degpu_mod.DeviceProblems(f, u0, p, np.tile([0.0, 10.0], (B, 1)), np.float64, dev)
    x = torch.as_tensor(learned.features(u0, p, np.full(B, 1e-6)), device=dev)
    dt0, sc = m.infer(x)
    ref = degpu_mod.api._solve_device(probs, degpu_mod.GPUTsit5(), True, dt=0.1, abstol=1e-8, reltol=1e-6, dt0=dt0,
                                      tolscale=sc)
    ts = torch.empty((B, 2), dtype=torch.float64, device=dev)
    us = torch.empty((B, 2, 3), dtype=torch.float32, device=dev)
    rc = torch.zeros(B, dtype=torch.int8, device=dev)
    opt = degpu_mod.api._options(degpu_mod.GPUTsit5(), np.float64, dt=0.1, abstol=1e-8, reltol=1e-6)
    out = _lib.Outputs(ts.data_ptr(), us.data_ptr(), 2, rc.data_ptr(), None, None, None)
    pr = probs.cstruct()
    st = torch.cuda.current_stream()
    _lib.check(_lib.lib().degpu_learned_asolve(f.handle(), m.h, ctypes.byref(pr), ctypes.byref(opt),
                                               m.dt_range[0], m.dt_range[1], m.scale_range[1], ctypes.byref(out),
                                               ctypes.c_void_p(st.cuda_stream)))
    torch.cuda.synchronize()
    assert torch.equal(us, ref.us) and torch.equal(ts, ref.ts) and torch.equal(rc, ref.retcode)
