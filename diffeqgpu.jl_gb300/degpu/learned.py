"""Learned step control: a BF16 MLP predicting each trajectory's initial dt and tolerance
scale from (u0, p, log10 reltol), trained on the GPU by libdegpu's own kernels on traces
that the plain solver generates.  No counterpart in the reference.

A second network of the same shape, the work model, predicts each trajectory's step
attempts (first output, log scale) from the same features; degpu_work_order turns the
predictions into a longest-first visiting order for the persistent driver, which shortens
the drain at the end of an ensemble with uneven step counts.  Results do not depend on the
order; only the schedule does.

Step-model targets, from plain solves of the training ensemble (all on the GPU):
  * log dt0    -- the first step the plain controller accepted (accepted-step trace);
  * log scale  -- how far the trajectory's tolerances can be relaxed before its final-state
    error reaches a common target: err_i(s) is the distance of the plain solution at
    tolerance scale s (1, 2, 4, ..., 64) to a 64x tighter plain solve, and the target scale
    is the largest s whose error, and that of every smaller s, stays at or below the target.
    Scales are >= 1: the learned run is never asked for tighter tolerances than the plain
    run, and members the plain run does not resolve (chaotic ones) keep the plain
    tolerances.  The embedded error estimate still accepts or rejects every step.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import check, lib

N_OUT = 2     # DEGPU_MLP_OUT
HIDDEN = 64   # DEGPU_MLP_HIDDEN


def _sigs():
    """Signatures live in _lib.SIGNATURES; kept for callers that registered them explicitly."""
    lib()


def features(u0, p, reltol, span=None):
    """x = (u0, p, log10 reltol) per trajectory, float32 [B, N + P + 1], followed by the
    span tf - t0 of each trajectory's tspan when given ([B, N + P + 2])."""
    u0 = np.asarray(u0, np.float32)
    p = np.asarray(p, np.float32).reshape(u0.shape[0], -1)
    lt = np.broadcast_to(np.log10(np.asarray(reltol, np.float64)), (u0.shape[0],)).astype(np.float32)
    cols = [u0, p, lt[:, None]]
    if span is not None:
        cols.append(np.broadcast_to(np.asarray(span, np.float64), (u0.shape[0],)).astype(np.float32)[:, None])
    return np.concatenate(cols, axis=1).astype(np.float32)


class StepSizeModel:
    """libdegpu's BF16 MLP (degpu_mlp_*), device-resident."""

    def __init__(self, n_in: int, seed: int = 0):
        _sigs()
        h = ctypes.c_void_p()
        check(lib().degpu_mlp_create(n_in, seed, ctypes.byref(h)))
        self.h = h
        self.n_in = n_in
        self.count = lib().degpu_mlp_param_count(h)
        self.dt_range = (1e-8, 1e3)
        self.scale_range = (1.0, 1e3)

    def __del__(self):
        try:
            if getattr(self, "h", None) is not None and _lib._lib is not None:
                _lib._lib.degpu_mlp_destroy(self.h)
        except Exception:
            pass

    # -------------------------------------------------------------- parameters
    def get(self):
        p = np.zeros(self.count, np.float32)
        g = np.zeros(self.count, np.float32)
        mu = np.zeros(self.n_in, np.float32)
        sd = np.zeros(self.n_in, np.float32)
        check(lib().degpu_mlp_get_params(self.h, p.ctypes.data, g.ctypes.data, mu.ctypes.data, sd.ctypes.data))
        return p, g, mu, sd

    def set(self, params=None, mean=None, std=None):
        def ptr(a):
            return None if a is None else np.ascontiguousarray(a, np.float32).ctypes.data
        keep = [None if a is None else np.ascontiguousarray(a, np.float32) for a in (params, mean, std)]
        check(lib().degpu_mlp_set_params(self.h, *(None if a is None else a.ctypes.data for a in keep)))

    def shift_log_scale(self, delta):
        """Lower the predicted log tolerance scale by `delta` (output bias b3[1])."""
        p, _, mu, sd = self.get()
        p[-1] -= np.float32(delta)
        self.set(p, mu, sd)

    def save(self, path):
        p, _, mu, sd = self.get()
        np.savez(path, params=p, mean=mu, std=sd, n_in=self.n_in, dt_range=self.dt_range, scale_range=self.scale_range)

    @classmethod
    def load(cls, path):
        z = np.load(path)
        m = cls(int(z["n_in"]))
        m.set(z["params"], z["mean"], z["std"])
        m.dt_range = tuple(z["dt_range"])
        m.scale_range = tuple(z["scale_range"])
        return m

    # -------------------------------------------------------------- kernels
    def grad(self, x_dev, t_dev, w_dev=None, stream=None):
        import torch
        st = stream or torch.cuda.current_stream()
        loss = torch.zeros(1, dtype=torch.float32, device=x_dev.device)
        check(lib().degpu_mlp_grad(self.h, x_dev.data_ptr(), t_dev.data_ptr(), None if w_dev is None else w_dev.data_ptr(),
                                   x_dev.shape[0], loss.data_ptr(), ctypes.c_void_p(st.cuda_stream)))
        return loss

    def adam(self, lr, beta1=0.9, beta2=0.999, eps=1e-8, wd=0.0, stream=None):
        import torch
        st = stream or torch.cuda.current_stream()
        check(lib().degpu_mlp_adam_step(self.h, lr, beta1, beta2, eps, wd, ctypes.c_void_p(st.cuda_stream)))

    def infer(self, x_dev, raw=False, stream=None):
        """Tensor-core inference.  Returns (dt0, tolscale) device tensors, or raw y [B,2]."""
        import torch
        st = stream or torch.cuda.current_stream()
        B = x_dev.shape[0]
        y = torch.empty((B, 2), dtype=torch.float32, device=x_dev.device) if raw else None
        d0 = None if raw else torch.empty(B, dtype=torch.float32, device=x_dev.device)
        sc = None if raw else torch.empty(B, dtype=torch.float32, device=x_dev.device)
        check(lib().degpu_mlp_infer(self.h, x_dev.data_ptr(), B, None if y is None else y.data_ptr(),
                                    None if d0 is None else d0.data_ptr(), None if sc is None else sc.data_ptr(),
                                    self.dt_range[0], self.dt_range[1], self.scale_range[0], self.scale_range[1],
                                    ctypes.c_void_p(st.cuda_stream)))
        return y if raw else (d0, sc)

    # -------------------------------------------------------------- training
    def fit(self, x, targets, weights=None, *, epochs=8, batch=8192, lr=3e-3, seed=0, log=None,
            normalize_targets=True):
        """Adam on the weighted MSE; x, targets, weights are host arrays or device tensors.

        With normalize_targets, each output is trained on its target standardised over the
        samples that weight it, and the output layer is rescaled afterwards (W3 row * std,
        b3 * std + mean), so the network predicts the targets in their own units: Adam moves
        each weight by about lr per step, and an output offset of several units (log step
        attempts ~ 5) would otherwise take thousands of steps to reach."""
        import torch
        dev = torch.device("cuda", torch.cuda.current_device())
        x = torch.as_tensor(np.asarray(x, np.float32) if not torch.is_tensor(x) else x, device=dev)
        t = torch.as_tensor(np.asarray(targets, np.float32) if not torch.is_tensor(targets) else targets, device=dev)
        w = None if weights is None else torch.as_tensor(
            np.asarray(weights, np.float32) if not torch.is_tensor(weights) else weights, device=dev)
        mean = x.mean(0).cpu().numpy()
        std = x.std(0).clamp_min(1e-6).cpu().numpy()
        self.set(mean=mean, std=std)
        t_mu = np.zeros(N_OUT)
        t_sd = np.ones(N_OUT)
        if normalize_targets:
            td = t.double()
            for o in range(N_OUT):
                sel = td[:, o] if w is None else td[:, o][w[:, o] > 0]
                if sel.numel() > 1:
                    t_mu[o] = float(sel.mean())
                    t_sd[o] = max(float(sel.std()), 1e-6)
            t = ((td - torch.as_tensor(t_mu, device=dev)) / torch.as_tensor(t_sd, device=dev)).float().contiguous()
        n = x.shape[0]
        g = torch.Generator(device=dev)
        g.manual_seed(seed)
        hist = []
        steps = max(1, epochs * ((n + batch - 1) // batch))
        k = 0
        for ep in range(epochs):
            perm = torch.randperm(n, device=dev, generator=g)
            tot = torch.zeros((), device=dev)
            for b0 in range(0, n, batch):
                idx = perm[b0:b0 + batch]
                xb, tb = x[idx].contiguous(), t[idx].contiguous()
                wb = None if w is None else w[idx].contiguous()
                loss = self.grad(xb, tb, wb)
                # cosine learning-rate decay
                cur = lr * 0.5 * (1 + np.cos(np.pi * k / steps))
                self.adam(cur)
                tot += loss[0] * xb.shape[0]
                k += 1
            hist.append(float(tot) / n)
            if log:
                log(f"epoch {ep}: loss {hist[-1]:.5f}")
        if normalize_targets:
            p, _, mu, sd = self.get()
            o_b3 = self.count - N_OUT
            o_W3 = o_b3 - N_OUT * HIDDEN
            W3 = p[o_W3:o_b3].reshape(N_OUT, HIDDEN).astype(np.float64)
            b3 = p[o_b3:].astype(np.float64)
            p[o_W3:o_b3] = (W3 * t_sd[:, None]).ravel().astype(np.float32)
            p[o_b3:] = (b3 * t_sd + t_mu).astype(np.float32)
            self.set(p, mu, sd)
        return hist


def solver_traces(f, u0, p, tspan, time_type, alg, *, reltol, abstol, dt=0.1, scales=(1, 2, 4, 8, 16, 32, 64),
                  tighten=64.0, device=None, driver="persistent"):
    """Accepted-step traces of the plain solver on a training ensemble (all on the GPU).

    Returns the first accepted dt at the base tolerances, the final-state error proxy at
    each tolerance scale s (distance to a `tighten` x tighter plain solve, relative to its
    norm) as an array [len(scales), B], and the attempts per trajectory at s = 1."""
    import torch

    from .api import DeviceProblems, _solve_device
    dev = device or torch.device("cuda", torch.cuda.current_device())
    B = u0.shape[0]
    tsp = np.broadcast_to(np.asarray(tspan, dtype=time_type), (B, 2)) if np.ndim(tspan) == 1 else np.asarray(tspan)
    probs = DeviceProblems(f, u0, p, tsp, time_type, dev)
    ref = _solve_device(probs, alg, True, dt=dt, abstol=abstol / tighten, reltol=reltol / tighten, driver=driver)
    ur = ref.us[:, 1].double()
    nr = ur.norm(dim=1).clamp_min(1e-3)
    errs, dtf, work = [], None, None
    for s in scales:
        r = _solve_device(probs, alg, True, dt=dt, abstol=abstol * s, reltol=reltol * s, trace=(s == scales[0]),
                          driver=driver)
        e = ((r.us[:, 1].double() - ur).norm(dim=1) / nr)
        e = torch.where(r.retcode == 1, e, torch.full_like(e, float("inf")))
        errs.append(e.cpu().numpy())
        if s == scales[0]:
            dtf = r.dt_first.cpu().numpy()
            work = (r.naccept + r.nreject).cpu().numpy()
    return dtf, np.stack(errs), work


def scale_targets(errs, scales, target_err):
    """Largest measured tolerance scale whose error, and that of every smaller scale, stays
    at or below the target (1 if even the base tolerance misses it)."""
    ok = np.cumprod(errs <= target_err, axis=0).astype(bool)  # monotone prefix
    idx = ok.sum(axis=0) - 1
    sc = np.asarray(scales, np.float64)
    return np.where(idx >= 0, sc[np.clip(idx, 0, len(sc) - 1)], sc[0])


def fit_step_model(f, u0, p, tspan, time_type, alg, *, reltol, abstol, target_quantile=0.9, safety=0.5,
                   scales=(1, 2, 4, 8, 16, 32, 64), epochs=8, seed=0, calib_frac=0.125, calib_margin=1.1, log=None,
                   expectile=0.1, expectile_rounds=3, dt=0.1, resolved=1e-3):
    """Train a StepSizeModel on the plain solver's traces of the given ensemble.

    The common error target is `safety` times the `target_quantile` of the plain run's
    error proxy at the base tolerances; each trajectory's scale target is the largest
    tolerance scale at which its measured error proxy stays under that target.  A held-out
    `calib_frac` of the ensemble then calibrates the model: the predicted log scale is
    shifted down by the smallest margin at which the learned run's error-proxy quantile
    is within `calib_margin` of the plain run's (regression to the mean would otherwise
    over-relax the most sensitive trajectories; the margin absorbs the few-percent change
    that a different initial step alone makes to the quantile).

    With `expectile` set, the scale output is then refined towards that expectile of the
    targets (asymmetric squared loss by iteratively reweighted least squares: residuals
    where the network over-relaxes weigh 1 - expectile, the others expectile), so that its
    predictions stay below the targets where they are uncertain and the calibration shift
    that follows can be small.

    `tspan` is one (t0, tf) or per-trajectory [B, 2]; in the second case the span tf - t0
    is a model input too.  `dt` is the plain solver's initial step.

    Members whose plain error proxy is above `resolved` (chaotic ones over long spans, where
    no FP32 solve tracks the tighter one) neither set the common error target nor enter the
    calibration quantiles, and their scale target is 1: the error level the learned run
    must hold is that of the members the plain run actually resolves."""
    import torch

    from .api import DeviceProblems, _solve_device
    B = u0.shape[0]
    nc = int(B * calib_frac)
    per_traj = np.ndim(tspan) == 2
    tsp_all = np.asarray(tspan) if per_traj else np.broadcast_to(np.asarray(tspan, dtype=time_type), (B, 2))
    span = (tsp_all[:, 1].astype(np.float64) - tsp_all[:, 0]) if per_traj else None
    ut, pt, uc, pc = u0[nc:], p[nc:], u0[:nc], p[:nc]
    tt, tc = tsp_all[nc:], tsp_all[:nc]
    st, sc_span = (span[nc:], span[:nc]) if per_traj else (None, None)
    dtf, errs, _ = solver_traces(f, ut, pt, tt, time_type, alg, reltol=reltol, abstol=abstol, scales=scales, dt=dt)
    res = np.isfinite(errs[0]) & (errs[0] <= resolved)
    e1 = errs[0][res] if res.any() else errs[0][np.isfinite(errs[0])]
    target = safety * float(np.quantile(e1, target_quantile))
    s = np.where(res, scale_targets(errs, scales, target), 1.0)
    ok = np.isfinite(dtf) & (dtf > 0)
    y = np.stack([np.log(np.where(ok, dtf, 1.0)), np.log(s)], 1).astype(np.float32)
    w = np.stack([ok, np.ones_like(ok)], 1).astype(np.float32)
    x = features(ut, pt, np.full(ut.shape[0], reltol), st)
    m = StepSizeModel(x.shape[1], seed=seed)
    m.scale_range = (1.0, float(max(scales)))
    m.fit(x, y, w, epochs=epochs, seed=seed, log=log)
    if expectile is not None and expectile_rounds > 0:
        dev = torch.device("cuda", torch.cuda.current_device())
        xd = torch.as_tensor(x, device=dev)
        for r in range(expectile_rounds):
            yp = m.infer(xd, raw=True)[:, 1].cpu().numpy()
            w[:, 1] = np.where(yp > y[:, 1], 1.0 - expectile, expectile) * 2.0
            # the network already predicts in the targets' units: no target standardisation
            m.fit(x, y, w, epochs=max(2, epochs // 2), lr=1e-3, seed=seed + 1 + r, log=log, normalize_targets=False)
    info = {"target_err": target, "err_proxy_median": float(np.median(e1)), "n_train": int(ut.shape[0]),
            "resolved_frac": float(res.mean()),
            "scale_target_median": float(np.median(s)), "scale_target_mean_log": float(np.log(s).mean())}
    if nc > 0:
        dev = torch.device("cuda", torch.cuda.current_device())
        probs = DeviceProblems(f, uc, pc, np.ascontiguousarray(tc), time_type, dev)
        ref = _solve_device(probs, alg, True, dt=dt, abstol=abstol / 64, reltol=reltol / 64)
        ur = ref.us[:, 1].double()
        nr = ur.norm(dim=1).clamp_min(1e-3)

        rplain = _solve_device(probs, alg, True, dt=dt, abstol=abstol, reltol=reltol)
        e_plain = (rplain.us[:, 1].double() - ur).norm(dim=1) / nr
        keep = e_plain <= resolved
        if int(keep.sum()) < 16:
            keep = torch.isfinite(e_plain)

        def proxy(r):
            e = (r.us[:, 1].double() - ur).norm(dim=1) / nr
            return float(torch.quantile(e[keep], target_quantile))
        q_plain = proxy(rplain)
        xc = torch.as_tensor(features(uc, pc, np.full(nc, reltol), sc_span), device=dev)
        y_raw = m.infer(xc, raw=True)
        dt0 = torch.exp(y_raw[:, 0]).clamp(*m.dt_range).contiguous()
        shift = None
        for delta in np.arange(0.0, 4.01, 0.25):
            sc = torch.exp(y_raw[:, 1] - float(delta)).clamp(*m.scale_range).contiguous()
            q = proxy(_solve_device(probs, alg, True, dt=dt, abstol=abstol, reltol=reltol, dt0=dt0, tolscale=sc))
            if q <= calib_margin * q_plain:
                shift = float(delta)
                break
        if shift is None:
            shift = 50.0  # never relax: predicted scale clamps to 1
        m.shift_log_scale(shift)
        info.update({"calib_trajectories": nc, "calib_log_scale_shift": shift, "calib_q_plain": q_plain,
                     "calib_q_learned": q if shift < 50.0 else None})
    return m, info


# ---------------------------------------------------------------------- work model
def work_order(work, stream=None):
    """Longest-first visiting order (device int32 [B]) from a per-trajectory work estimate
    (device float32 [B], e.g. predicted attempts), by degpu_work_order."""
    import torch
    st = stream or torch.cuda.current_stream(work.device)
    work = work.contiguous().float()
    order = torch.empty(work.shape[0], dtype=torch.int32, device=work.device)
    check(lib().degpu_work_order(work.data_ptr(), work.shape[0], order.data_ptr(), ctypes.c_void_p(st.cuda_stream)))
    return order


def predicted_work(model, u0_dev, p_dev, reltol, span_dev=None):
    """Predicted step attempts (device float32 [B]) of a work model on device (u0, p) and,
    for a model trained with per-trajectory tspans, the spans tf - t0 (device [B])."""
    import torch
    B = u0_dev.shape[0]
    cols = [u0_dev.float(), p_dev.float().reshape(B, -1),
            torch.full((B, 1), float(np.log10(reltol)), dtype=torch.float32, device=u0_dev.device)]
    if span_dev is not None:
        cols.append(span_dev.float().reshape(B, 1))
    x = torch.cat(cols, 1)
    if x.shape[1] != model.n_in:
        raise ValueError(f"the work model takes {model.n_in} inputs, got {x.shape[1]} (span_dev for spans?)")
    y = model.infer(x.contiguous(), raw=True)
    return torch.exp(y[:, 0]).clamp(1.0, 2.0 ** 31)


def fit_work_model(f, u0, p, tspan, time_type, alg, *, reltol, abstol, dt=0.1, step_model=None, epochs=8, seed=0,
                   holdout_frac=0.125, log=None, **solve_kw):
    """Train a work model on the step attempts of the solve it will order.

    The training solve is the plain controller, or the learned one when `step_model` is
    given (its dt0 / tolerance-scale predictions change the attempts).  Targets are
    log(naccept + nreject) of successful trajectories; the second output is unused (weight
    0).  With per-trajectory tspans ([B, 2]) the span tf - t0 is an input too.  Returns
    (model, info) with the correlation of predicted and actual log attempts on a held-out
    share of the ensemble."""
    import torch

    from .api import DeviceProblems, _solve_device
    dev = torch.device("cuda", torch.cuda.current_device())
    B = u0.shape[0]
    per_traj = np.ndim(tspan) == 2
    tsp = np.asarray(tspan) if per_traj else np.broadcast_to(np.asarray(tspan, dtype=time_type), (B, 2))
    probs = DeviceProblems(f, u0, p, tsp, time_type, dev)
    span = (tsp[:, 1].astype(np.float64) - tsp[:, 0]) if per_traj else None
    x = features(u0, p, np.full(B, reltol), span)
    kw = {}
    if step_model is not None:
        d0, sc = step_model.infer(torch.as_tensor(x, device=dev))
        kw = dict(dt0=d0.contiguous(), tolscale=sc.contiguous())
    r = _solve_device(probs, alg, True, dt=dt, abstol=abstol, reltol=reltol, **kw, **solve_kw)
    work = (r.naccept + r.nreject).cpu().numpy().astype(np.float64)
    ok = (r.retcode.cpu().numpy() == 1) & (work > 0)
    y = np.stack([np.log(np.maximum(work, 1.0)), np.zeros(B)], 1).astype(np.float32)
    w = np.stack([ok, np.zeros(B, bool)], 1).astype(np.float32)
    nh = int(B * holdout_frac)
    m = StepSizeModel(x.shape[1], seed=seed)
    m.dt_range = (1.0, 2.0 ** 31)  # exp(first output) = predicted attempts
    m.scale_range = (1.0, 1.0)
    m.fit(x[nh:], y[nh:], w[nh:], epochs=epochs, batch=2048, seed=seed, log=log)
    info = {"n_train": int(B - nh), "attempts_mean": float(work[ok].mean()) if ok.any() else None}
    if nh > 0:
        yh = m.infer(torch.as_tensor(x[:nh], device=dev), raw=True)[:, 0].cpu().numpy()
        sel = ok[:nh]
        info["holdout_corr_log_attempts"] = float(np.corrcoef(yh[sel], y[:nh, 0][sel])[0, 1]) if sel.sum() > 2 else None
    return m, info
