"""The whole batched solve as one CUDA graph: from the second call with the
same layout, plans, buffers and tolerance, msq_solve_batched captures its
plan groups' launch sequence (gather, Jacobi, reconstruction, residuals,
corrections, scatter, report copies) and later calls replay it with a single
graph launch and one host synchronisation.  The replay computes the same
bits as direct launches."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def _batch(msq, orders, seed):
    import torch
    mats = [O.wishart(n, seed=seed + i) for i, n in enumerate(orders)]
    b = msq.Batch.from_orders(orders)
    return mats, b, torch.from_numpy(b.pack(mats)).cuda()


def test_steady_state_is_one_graph_launch_with_the_same_bits(ctx, msq):
    import torch
    # orders up to 256 (the batched kernels; no grid-path matrix), two plans
    orders = [40, 64, 100, 130, 200, 256] * 3
    mats, b, a = _batch(msq, orders, seed=100)
    plans = [msq.plan(msq.PLAN_BF16, 1, 1e-4) if i % 2 else msq.plan(msq.PLAN_FP8, 2, 1e-3)
             for i in range(len(orders))]
    out = torch.empty_like(a)
    ctx.set_graphs(True)
    for _ in range(4):  # launch-shape tuning, the direct run, the capture
        _, res = ctx.solve_batched(a, b, plans, 1e-5, out=out)
    assert not any(r.fallback for r in res)
    g0, l0 = ctx.graph_launches, ctx.launches
    _, res_graph = ctx.solve_batched(a, b, plans, 1e-5, out=out)
    assert ctx.graph_launches - g0 == 1
    assert ctx.launches - l0 > 20  # the replayed graph holds the whole solve
    root_graph = out.cpu().numpy().copy()
    ctx.set_graphs(False)
    try:
        _, res_direct = ctx.solve_batched(a, b, plans, 1e-5, out=out)
        root_direct = out.cpu().numpy()
    finally:
        ctx.set_graphs(True)
    assert np.array_equal(root_graph.view(np.uint32), root_direct.view(np.uint32))
    # the roots are the same bits; the reported norms are FP64 sums whose
    # per-warp atomic order may differ run to run (last-bit differences)
    for rg, rd in zip(res_graph, res_direct):
        assert rg.final_residual == pytest.approx(rd.final_residual, rel=1e-12)
        assert rg.initial_residual == pytest.approx(rd.initial_residual, rel=1e-12)
        assert rg.jacobi_sweeps == rd.jacobi_sweeps and rg.accepted == rd.accepted
    for m, x, r in zip(mats, b.unpack(root_graph), res_graph):
        assert r.final_residual <= 1e-5
        assert O.relative_residual(m, x) <= 2e-5


def test_graph_replay_with_a_fallback_and_new_inputs(ctx, msq):
    """A replay reads the buffers it was captured with: new values in the
    same input buffer give that input's roots; a miss still takes the FP32
    fallback after the replay."""
    import torch
    orders = [8, 12, 50, 90, 160]
    mats1, b, a = _batch(msq, orders, seed=7)
    mats2, _, a2 = _batch(msq, orders, seed=77)
    # a 4-bit basis without sweeps misses 1e-5 everywhere: every matrix falls back
    plans = [msq.plan(msq.PLAN_MXFP4, 1, 1e-3)] * len(orders)
    out = torch.empty_like(a)
    for _ in range(4):
        _, res = ctx.solve_batched(a, b, plans, 1e-5, out=out)
    a.copy_(a2)  # same buffer, new matrices
    g0 = ctx.graph_launches
    _, res = ctx.solve_batched(a, b, plans, 1e-5, out=out)
    assert ctx.graph_launches - g0 >= 1
    for m, x, r in zip(mats2, b.unpack(out.cpu().numpy()), res):
        assert r.final_residual <= 1e-5
        assert O.relative_residual(m, x) <= 2e-5
