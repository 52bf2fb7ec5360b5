"""degpu_batch_solve_host (batch_solve_up_kernel with host buffers): copies in, solve, copies
out.  Large batches are pipelined in chunks over two streams; the results must be the
device API's, bit for bit, whatever the chunking."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _host_solve(degpu, f, alg, u0, p, tsp, Tt, opt, adaptive, L, pinned=True):
    import torch
    from degpu import _lib
    B, N = u0.shape
    pin = (lambda t: t.pin_memory()) if pinned else (lambda t: t)
    hu0, hp, htsp = [pin(torch.from_numpy(np.ascontiguousarray(a))) for a in (u0, p, tsp.astype(Tt))]
    hts = pin(torch.empty((B, L), dtype=torch.float64 if Tt == np.float64 else torch.float32))
    hus = pin(torch.empty((B, L, N), dtype=torch.float32))
    hrc = pin(torch.zeros(B, dtype=torch.int8))
    hna = pin(torch.zeros(B, dtype=torch.int32))
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(_lib.lib().degpu_batch_solve_host(f.handle(), hu0.data_ptr(), hp.data_ptr(), htsp.data_ptr(), B,
                                                 ctypes.byref(opt), int(adaptive), hts.data_ptr(), hus.data_ptr(), L,
                                                 hrc.data_ptr(), hna.data_ptr(), None, st))
    return hts.numpy(), hus.numpy(), hrc.numpy(), hna.numpy()


@pytest.mark.parametrize("path", ["direct", "staged", "staged_chunked"])
def test_host_api_matches_device(degpu_mod, monkeypatch, path):
    """300,000 Lorenz trajectories, adaptive Tsit5, saveat 0:0.5:10, FP64 time: outputs
    written straight into page-locked host memory by the kernel; staged on the device and
    copied back in one piece; staged and pipelined in 6 chunks (DEGPU_HOST_CHUNK=50000)."""
    import torch
    if path != "direct":
        monkeypatch.setenv("DEGPU_HOST_DIRECT", "0")
    if path == "staged_chunked":
        monkeypatch.setenv("DEGPU_HOST_CHUNK", "50000")
    B = 300_000
    rng = np.random.default_rng(11)
    p = (rng.random((B, 3)) * np.array([10, 28, 8 / 3])).astype(np.float32)
    u0 = (np.array([1, 0, 0]) + rng.normal(0, 0.1, (B, 3))).astype(np.float32)
    tsp = np.tile([0.0, 10.0], (B, 1))
    sa = np.arange(0.0, 10.0001, 0.5)
    f = degpu_mod.ODEFunction.builtin("lorenz")
    probs = degpu_mod.DeviceProblems(f, u0, p, tsp, np.float64, torch.device("cuda", 0))
    r = degpu_mod.api._solve_device(probs, degpu_mod.GPUTsit5(), True, dt=0.1, saveat=sa, abstol=1e-8, reltol=1e-6)
    torch.cuda.synchronize()
    hsa = torch.from_numpy(sa.copy()).pin_memory()
    opt = degpu_mod.api._options(degpu_mod.GPUTsit5(), np.float64, dt=0.1, abstol=1e-8, reltol=1e-6,
                                 saveat_dev=hsa.data_ptr(), nsaveat=len(sa))
    ts, us, rc, na = _host_solve(degpu_mod, f, degpu_mod.GPUTsit5(), u0, p, tsp, np.float64, opt, True, len(sa))
    assert np.array_equal(us.view(np.uint32), r.us.cpu().numpy().view(np.uint32))
    assert np.array_equal(ts, r.ts.cpu().numpy())
    assert np.array_equal(rc, r.retcode.cpu().numpy()) and np.array_equal(na, r.naccept.cpu().numpy())


def test_host_api_chunked_em_and_per_trajectory_saveat(degpu_mod, monkeypatch):
    """EM noise is keyed by the global trajectory index, so a chunked host solve reproduces
    the one-launch device solve; per-trajectory saveat rows follow their chunk."""
    import torch
    monkeypatch.setenv("DEGPU_HOST_CHUNK", "333")
    B = 2000
    rng = np.random.default_rng(12)
    u0 = np.full((B, 1), 0.5, np.float32)
    p = np.tile(np.array([1.5, 0.1], np.float32), (B, 1))
    tsp = np.tile([0.0, 1.0], (B, 1)).astype(np.float32)
    f = degpu_mod.SDEFunction.builtin("gbm") if hasattr(degpu_mod, "SDEFunction") else degpu_mod.ODEFunction.builtin("gbm")
    probs = degpu_mod.DeviceProblems(f, u0, p, tsp, np.float32, torch.device("cuda", 0), kind="sde")
    r = degpu_mod.api._solve_device(probs, degpu_mod.GPUEM(), False, dt=0.01, save_everystep=False, seed=77)
    torch.cuda.synchronize()
    opt = degpu_mod.api._options(degpu_mod.GPUEM(), np.float32, dt=0.01, seed=77)
    ts, us, rc, _ = _host_solve(degpu_mod, f, degpu_mod.GPUEM(), u0, p, tsp, np.float32, opt, False, 2,
                                pinned=False)  # pageable: staged and chunked
    assert np.array_equal(us.view(np.uint32), r.us.cpu().numpy().view(np.uint32))

    # per-trajectory saveat (each trajectory its own 5 points), Lorenz fixed step
    u0l = np.tile(np.array([1, 0, 0], np.float32), (B, 1))
    pl = (rng.random((B, 3)) * np.array([10, 28, 8 / 3])).astype(np.float32)
    tspl = np.tile([0.0, 2.0], (B, 1)).astype(np.float32)
    sal = np.sort(rng.uniform(0.0, 2.0, (B, 5)), axis=1).astype(np.float32)
    fl = degpu_mod.ODEFunction.builtin("lorenz")
    pr = degpu_mod.DeviceProblems(fl, u0l, pl, tspl, np.float32, torch.device("cuda", 0), saveat=sal)
    rl = degpu_mod.api._solve_device(pr, degpu_mod.GPUTsit5(), False, dt=0.01)
    torch.cuda.synchronize()
    hsal = torch.from_numpy(sal.copy()).pin_memory()
    opt = degpu_mod.api._options(degpu_mod.GPUTsit5(), np.float32, dt=0.01, saveat_dev=hsal.data_ptr(), nsaveat=5,
                                 per_traj=True)
    ts, us, rc, _ = _host_solve(degpu_mod, fl, degpu_mod.GPUTsit5(), u0l, pl, tspl, np.float32, opt, False, 5)
    assert np.array_equal(us.view(np.uint32), rl.us.cpu().numpy().view(np.uint32))
    assert np.array_equal(ts, rl.ts.cpu().numpy())


@pytest.mark.parametrize("path", ["direct", "staged_chunked"])
def test_learned_host_api_matches_device(degpu_mod, monkeypatch, path):
    """degpu_learned_batch_solve_host (host buffers, step and work models) gives the device
    solve's bits: the models run on the device copies of the inputs (per chunk on the
    pipelined path) and the visiting order changes no result."""
    import torch
    from degpu import _lib, learned
    if path != "direct":
        monkeypatch.setenv("DEGPU_HOST_DIRECT", "0")
        monkeypatch.setenv("DEGPU_HOST_CHUNK", "40000")
    B = 120_000
    rng = np.random.default_rng(21)
    p = (rng.random((B, 3)) * np.array([10, 28, 8 / 3])).astype(np.float32)
    u0 = (np.array([1, 0, 0]) + rng.normal(0, 0.1, (B, 3))).astype(np.float32)
    tsp = np.tile([0.0, 10.0], (B, 1))
    sa = np.arange(0.0, 10.0001, 0.5)
    L = len(sa)
    f = degpu_mod.ODEFunction.builtin("lorenz")
    sm, _ = learned.fit_step_model(f, u0[:16384], p[:16384], (0.0, 10.0), np.float64, degpu_mod.GPUTsit5(),
                                   reltol=1e-6, abstol=1e-8, epochs=2)
    wm, _ = learned.fit_work_model(f, u0[:32768], p[:32768], (0.0, 10.0), np.float64, degpu_mod.GPUTsit5(),
                                   reltol=1e-6, abstol=1e-8, epochs=2)
    probs = degpu_mod.DeviceProblems(f, u0, p, tsp, np.float64, torch.device("cuda", 0))
    r = degpu_mod.api._solve_device(probs, degpu_mod.GPUTsit5(), True, dt=0.1, saveat=sa, abstol=1e-8, reltol=1e-6,
                                    step_model=sm)
    torch.cuda.synchronize()
    pin = (lambda t: t.pin_memory()) if path == "direct" else (lambda t: t)
    hu0, hp, htsp = [pin(torch.from_numpy(np.ascontiguousarray(a))) for a in (u0, p, tsp)]
    hts = pin(torch.empty((B, L), dtype=torch.float64))
    hus = pin(torch.empty((B, L, 3), dtype=torch.float32))
    hrc = pin(torch.zeros(B, dtype=torch.int8))
    hna = pin(torch.zeros(B, dtype=torch.int32))
    hsa = torch.from_numpy(sa.copy()).pin_memory()
    opt = degpu_mod.api._options(degpu_mod.GPUTsit5(), np.float64, dt=0.1, abstol=1e-8, reltol=1e-6,
                                 saveat_dev=hsa.data_ptr(), nsaveat=L)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(_lib.lib().degpu_learned_batch_solve_host(
        f.handle(), sm.h, wm.h, hu0.data_ptr(), hp.data_ptr(), htsp.data_ptr(), B, ctypes.byref(opt), sm.dt_range[0],
        sm.dt_range[1], sm.scale_range[1], hts.data_ptr(), hus.data_ptr(), L, hrc.data_ptr(), hna.data_ptr(), None, st))
    assert np.array_equal(hus.numpy().view(np.uint32), r.us.cpu().numpy().view(np.uint32))
    assert np.array_equal(hts.numpy(), r.ts.cpu().numpy())
    assert np.array_equal(hrc.numpy(), r.retcode.cpu().numpy()) and np.array_equal(hna.numpy(), r.naccept.cpu().numpy())
    # models apply to adaptive ODE solves only
    assert _lib.lib().degpu_learned_batch_solve_host(
        f.handle(), sm.h, wm.h, hu0.data_ptr(), hp.data_ptr(), htsp.data_ptr(), B, ctypes.byref(
            degpu_mod.api._options(degpu_mod.GPUEM(), np.float64, dt=0.1)), 1e-8, 1.0, 1.0, hts.data_ptr(),
        hus.data_ptr(), L, None, None, None, st) == -1
