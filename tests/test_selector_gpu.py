"""Learned plan selector: the hand-written CUDA forward/backward/Adam kernels
against the FP64 oracle, training on method-generated data, and what the
trained network gains over the method without it."""
import importlib
import math

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sel():
    return importlib.import_module("mixed-mlx_gb300.selector")


def _rand_params(msq, seed):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal(msq.MLP_PARAMS) * 0.2).astype(np.float32)


def test_forward_matches_oracle(ctx, msq):
    import torch
    p = _rand_params(msq, 1)
    x = np.random.default_rng(2).standard_normal((37, msq.MLP_IN)).astype(np.float32)
    z = ctx.mlp_forward(torch.from_numpy(p).cuda(), torch.from_numpy(x).cuda())
    z_ref, _ = O.mlp_forward(p, x.astype(np.float64))
    np.testing.assert_allclose(z.cpu().numpy(), z_ref, rtol=1e-4, atol=1e-5)


def test_backward_gradient_matches_fp64_oracle(ctx, msq):
    import torch
    p = _rand_params(msq, 3)
    rng = np.random.default_rng(4)
    x = rng.standard_normal((300, msq.MLP_IN)).astype(np.float32)
    y = (rng.random((300, msq.MLP_OUT)) < 0.5).astype(np.float32)
    grad = torch.zeros(msq.MLP_PARAMS, device="cuda")
    loss = ctx.mlp_backward(torch.from_numpy(p).cuda(), torch.from_numpy(x).cuda(),
                            torch.from_numpy(y).cuda(), grad)
    loss_ref, grad_ref = O.mlp_loss_and_grad(p, x, y)
    assert abs(float(loss.item()) - loss_ref) < 1e-5 * max(1.0, abs(loss_ref))
    g = grad.cpu().numpy()
    np.testing.assert_allclose(g, grad_ref, rtol=2e-3, atol=2e-6 * np.abs(grad_ref).max())
    # and the oracle's analytic gradient against a central difference (FP64)
    eps = 1e-3
    for k in (0, 100, 1100, 5000):
        d = np.zeros_like(p)
        d[k] = eps
        lp, _ = O.mlp_loss_and_grad(p + d, x, y)
        lm, _ = O.mlp_loss_and_grad(p - d, x, y)
        # BF16 rounding makes the loss piecewise constant in tiny steps; only
        # check where the step moved the rounded weight
        if lp != lm:
            assert np.sign((lp - lm)) == np.sign(grad_ref[k]) or abs(grad_ref[k]) < 1e-6


def test_adam_step_matches_formula(ctx, msq):
    import torch
    p = _rand_params(msq, 5)
    g = np.random.default_rng(6).standard_normal(msq.MLP_PARAMS).astype(np.float32)
    pt = torch.from_numpy(p.copy()).cuda()
    m = torch.zeros_like(pt)
    v = torch.zeros_like(pt)
    ctx.mlp_step(pt, torch.from_numpy(g).cuda(), m, v, 1, 1e-2)
    m1, v1 = 0.1 * g, 0.001 * g * g
    expect = p - 1e-2 * (m1 / 0.1) / (np.sqrt(v1 / 0.001) + 1e-8)
    np.testing.assert_allclose(pt.cpu().numpy(), expect, rtol=1e-5, atol=1e-6)


def test_trained_selector_plans_cost_less_than_the_fp32_path(ctx, msq, sel):
    """Train on plans the method itself ran and scored, then on held-out
    matrices: every result still meets the tolerance (FP32 fallback on a
    miss), the selected plans' pass costs less GPU time than
    solving every matrix with the FP32 path the method uses without a
    selector, and with the misses' fallback the call stays close to that
    path (asserted within 15%).

    Held-out: 2048 matrices (n <= 512, condition to 1e3), enough per SM that
    a Jacobi sweep's time follows the work of the members still rotating.
    (On a batch smaller than the SMs' capacity the pass lasts as long as its
    slowest member's sweeps, and one FP32 member takes as long as the FP32
    path.)  Most of these matrices admit a low-bit plan, which saves about a
    quarter of the pass; the fallback of the misses is a small,
    latency-bound FP32 pass that gives back most of it, so end to end the
    two are within a few percent of each other (measured on GB300 over
    several runs, the network differing run to run with the order of its
    gradient sums: pass 0.76x - 0.88x, call 0.97x - 1.05x; at condition to
    1e5: 0.85x and 0.96x)."""
    import torch
    tol = 1e-5
    orders, mats = sel.generate(torch, 384, seed=11, n_hi=512, cond_hi=1e5)
    batch, flat = sel.pack(msq, torch, orders, mats)
    feats = sel.features(ctx, torch, batch, flat, tol)
    outcome = sel.score_plans(ctx, msq, torch, batch, flat, tol)
    selector = sel.Selector(msq, torch, ctx, seed=0)
    selector.cost_order = list(np.argsort(outcome.seconds))
    losses = selector.fit(feats, torch.from_numpy(outcome.accepted).cuda(), epochs=60)
    assert losses[-1] < 0.7 * losses[0]

    orders_t, mats_t = sel.generate(torch, 2048, seed=13, n_hi=512, cond_hi=1e3)
    batch_t, flat_t = sel.pack(msq, torch, orders_t, mats_t)
    feats_t = sel.features(ctx, torch, batch_t, flat_t, tol)
    choice = selector.choose(feats_t, threshold=0.9)
    plans = [msq.plan(msq.PLAN_FP32, 1, 1e-7, 15) if k < 0 else
             sel.plan_structs(msq, [int(k)])[0] for k in choice]
    fp32 = [msq.plan(msq.PLAN_FP32, 1, 1e-7, 15)] * batch_t.count
    out_sel = torch.empty_like(flat_t)
    fresh = msq.Context(0)  # timed on a context whose caches hold only this workload
    try:
        def timed(p, t, out):
            for _ in range(2):  # plan caches, then the solve's graph capture
                fresh.solve_batched(flat_t, batch_t, p, t, out=out)
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            _, res = fresh.solve_batched(flat_t, batch_t, p, t, out=out)
            e.record()
            torch.cuda.synchronize()
            return s.elapsed_time(e), res

        scratch = torch.empty_like(flat_t)
        # tolerance 1: every plan is accepted, so this times the plan pass alone
        t_pass_sel, _ = timed(plans, 1.0, scratch)
        t_pass_fp32, _ = timed(fp32, 1.0, scratch)
        t_fp32, res_fp32 = timed(fp32, tol, scratch)
        t_sel, res_sel = timed(plans, tol, out_sel)
    finally:
        fresh.close()
    # a miss is allowed only where the FP32 method without a selector (the
    # fallback) misses too: inputs whose conditioning is beyond FP32 Jacobi
    misses = [(i, int(orders_t[i]), int(choice[i]), r.final_residual, r.fallback,
               res_fp32[i].final_residual)
              for i, r in enumerate(res_sel) if not r.final_residual <= tol]
    assert all(not (m[5] <= tol) for m in misses), misses
    assert len(misses) <= 0.05 * batch_t.count, misses
    accepted = np.mean([r.accepted for r in res_sel])
    assert accepted > 0.8
    times = dict(pass_sel=t_pass_sel, pass_fp32=t_pass_fp32, sel=t_sel, fp32=t_fp32,
                 fallbacks=int(sum(r.fallback for r in res_sel)))
    assert t_pass_sel < 0.95 * t_pass_fp32, times
    assert t_sel < 1.15 * t_fp32, times
    xs = batch_t.unpack(out_sel.cpu().numpy())
    for i in range(0, batch_t.count, 16):
        a64 = mats_t[i].cpu().numpy()
        assert O.relative_residual(a64, xs[i]) <= 2 * tol
