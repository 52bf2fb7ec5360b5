"""degpu_learned_asolve_noalloc: the learned-controller solve for callers that may not
allocate device memory while they solve (host callbacks, fixed-budget or real-time
runtimes that own all device memory).  It takes its scratch from a static array in the
library instead of the stream-ordered allocator.  Checked through the C ABI against the
allocating degpu_learned_asolve on two calls in a row; larger-than-supported batches are
rejected with a clear error.  This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(degpu_mod, B, seed=21):
    import torch
    from degpu import _lib, learned
    rng = np.random.default_rng(seed)
    p = (rng.random((B, 3)) * np.array([10, 28, 8 / 3])).astype(np.float32)
    u0 = (np.array([1, 0, 0]) + rng.normal(0, 0.1, (B, 3))).astype(np.float32)
    m = learned.StepSizeModel(7, seed=9)
    P, _, _, _ = m.get()
    m.set(P, np.concatenate([u0.mean(0), p.mean(0), [-6.0]]), np.concatenate([u0.std(0), p.std(0), [1.0]]))
    f = degpu_mod.ODEFunction.builtin("lorenz")
    dev = torch.device("cuda", 0)
    probs = degpu_mod.DeviceProblems(f, u0, p, np.tile([0.0, 10.0], (B, 1)), np.float64, dev)
    sa = torch.as_tensor(np.arange(0.0, 10.0001, 0.5), device=dev)
    opt = degpu_mod.api._options(degpu_mod.GPUTsit5(), np.float64, dt=0.1, abstol=1e-8, reltol=1e-6,
                                 saveat_dev=sa.data_ptr(), nsaveat=21)
    return m, f, probs, opt, sa, _lib


def _outputs(B, L, _lib):
    import torch
    o = dict(ts=torch.empty((B, L), dtype=torch.float64, device="cuda"),
             us=torch.empty((B, L, 3), dtype=torch.float32, device="cuda"),
             rc=torch.zeros(B, dtype=torch.int8, device="cuda"), na=torch.zeros(B, dtype=torch.int32, device="cuda"))
    o["c"] = _lib.Outputs(o["ts"].data_ptr(), o["us"].data_ptr(), L, o["rc"].data_ptr(), o["na"].data_ptr(), None, None)
    return o


def test_noalloc_matches_allocating_entry_point(degpu_mod):
    import torch
    B = 20_000
    m, f, probs, opt, sa, _lib = _setup(degpu_mod, B)
    pr = probs.cstruct()
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    ref = _outputs(B, 21, _lib)
    _lib.check(_lib.lib().degpu_learned_asolve(f.handle(), m.h, ctypes.byref(pr), ctypes.byref(opt), 1e-8, 1e3, 64.0,
                                               ctypes.byref(ref["c"]), st))
    torch.cuda.synchronize()
    for call in range(2):  # two calls in a row share (and reuse) the static scratch
        out = _outputs(B, 21, _lib)
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        _lib.check(_lib.lib().degpu_learned_asolve_noalloc(f.handle(), m.h, ctypes.byref(pr), ctypes.byref(opt),
                                                           1e-8, 1e3, 64.0, ctypes.byref(out["c"]), st))
        torch.cuda.synchronize()
        if call == 1:  # after set-up, a call takes no device memory
            assert torch.cuda.mem_get_info()[0] >= free_before
        # same kernels on the same inputs: the results agree exactly (tolerance 0)
        assert torch.equal(out["rc"], ref["rc"]) and (out["rc"] == 1).all()
        assert torch.equal(out["na"], ref["na"])
        assert torch.equal(out["ts"], ref["ts"])
        assert torch.allclose(out["us"], ref["us"], rtol=0, atol=0)


def test_noalloc_rejects_oversized_batch(degpu_mod):
    import torch
    from degpu import _lib
    B = 262_145  # one more than DEGPU_NOALLOC_MAX_TRAJECTORIES
    m, f, probs, opt, sa, _lib = _setup(degpu_mod, 8)
    pr = _lib.Problems(probs.u0.data_ptr(), probs.p.data_ptr(), probs.tspan.data_ptr(), B)
    out = _lib.Outputs(256, 256, 21, None, None, None, None)  # never touched: the size check comes first
    rc = _lib.lib().degpu_learned_asolve_noalloc(f.handle(), m.h, ctypes.byref(pr), ctypes.byref(opt), 1e-8, 1e3, 64.0,
                                                 ctypes.byref(out), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == -1
    assert "262144" in _lib.lib().degpu_last_error().decode()
