"""The launch-shape autotuner: candidate CTA sizes are timed on live sweeps
and the fastest kept per size class; every candidate computes the same bits,
so results before, during and after tuning are identical."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def _solve(ctx, msq, b, a_host):
    import torch
    a = torch.from_numpy(a_host.copy()).cuda()
    v, w, sweeps, off = ctx.jacobi(a, b, 1e-7, 15)
    torch.cuda.synchronize()
    return v.cpu().numpy(), w.cpu().numpy(), sweeps.cpu().numpy()


def test_tuning_keeps_results_bit_identical(ctx, msq):
    # one matrix in each small size class and nine of order 300 (with more
    # than eight matrices above 256 these stay on the batched kernels)
    orders = [12, 30, 60, 100, 200] + [300] * 9
    mats = [O.spd_loguniform(n, 1e2, seed=i) for i, n in enumerate(orders)]
    b = msq.Batch.from_orders(orders)
    packed = b.pack(mats)
    msq.lib().msq_autotune_reset(1)
    first = _solve(ctx, msq, b, packed)      # measures candidates on sweeps 1..C
    second = _solve(ctx, msq, b, packed)
    third = _solve(ctx, msq, b, packed)      # tuned shapes
    for x, y, z in zip(first, second, third):
        assert np.array_equal(x, y) and np.array_equal(x, z)
    report = ctx.autotune_report()
    lines = [l for l in report.splitlines() if l]
    assert len(lines) == 9
    tuned = [l for l in lines if "untuned" not in l]
    # every class present in the batch (classes n <= 16 .. n <= 320) is tuned
    assert len(tuned) >= 6, report


def test_tuning_disabled_uses_defaults(ctx, msq):
    orders = [100, 200]
    mats = [O.spd_loguniform(n, 1e2, seed=n) for n in orders]
    b = msq.Batch.from_orders(orders)
    msq.lib().msq_autotune_reset(0)
    try:
        r = _solve(ctx, msq, b, b.pack(mats))
        assert "untuned" in ctx.autotune_report()
    finally:
        msq.lib().msq_autotune_reset(1)
    r2 = _solve(ctx, msq, b, b.pack(mats))
    assert np.array_equal(r[0], r2[0]) and np.array_equal(r[1], r2[1])


def test_graph_replay_matches_direct_launches(ctx, msq):
    """The batched Jacobi's captured CUDA graph (replayed from the second
    call on) gives the same bits as launching every kernel directly, with
    the internal streams on and off."""
    orders = [20, 50, 90, 150, 220] + [300] * 9
    mats = [O.spd_loguniform(n, 1e3, seed=50 + i) for i, n in enumerate(orders)]
    b = msq.Batch.from_orders(orders)
    packed = b.pack(mats)
    for _ in range(3):  # tune and capture
        _solve(ctx, msq, b, packed)
    l0 = ctx.launches
    graph = _solve(ctx, msq, b, packed)
    assert ctx.launches > l0
    ctx.set_graphs(False)
    try:
        direct = _solve(ctx, msq, b, packed)
        ctx.set_concurrency(False)
        serial = _solve(ctx, msq, b, packed)
    finally:
        ctx.set_concurrency(True)
        ctx.set_graphs(True)
    for x, y, z in zip(graph, direct, serial):
        assert np.array_equal(x, y) and np.array_equal(x, z)
