"""The bounded device waits give up, report, and leave the context usable.

No wait is made to run out by breaking anything: msq_debug_expire_waits
points the waits at a condition nothing fulfils (a shared-memory flag value
no warp writes; an mbarrier phase nothing arrives at, waited on before any
copy or MMA is issued) with a short limit.  The call's status check must
then return MSQ_ERR_DEVICE_STATUS naming the expired wait, the allocation-
free Jacobi must mark its outputs, and the next call with the injection off
must give correct results on the same context."""
import ctypes

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

FLAG, MBARRIER = 1, 2


@pytest.fixture
def injection(msq, ctx):
    ctx.set_graphs(False)
    yield lambda mode: msq.lib().msq_debug_expire_waits(mode)
    assert msq.lib().msq_debug_expire_waits(0) == 0
    ctx.set_graphs(True)
    ctx.set_jacobi_vectors(-1)


def _batch(msq, orders, seed=0):
    import torch
    mats = [O.wishart(n, seed=seed + n) for n in orders]
    b = msq.Batch.from_orders(orders)
    return mats, b, torch.from_numpy(b.pack(mats)).cuda()


@pytest.mark.parametrize("mode,orders", [
    # the two-level order (257..512) has pairs that share a super-tile, so
    # quads wait on each other's flags; the round-robin shared-tile classes
    # reload their tiles by TMA between sweeps
    # MSQ_VECTORS_BLOCKED: two-level order, FP32 replay; more than eight
    # orders above 256, so the batched kernels (not the grid path) take them
    (1, [300, 400, 512] * 4),
    (0, [64, 128, 200, 256]),  # MSQ_VECTORS_REPLAY: round-robin
])
def test_jacobi_wait_expiry_is_reported(msq, ctx, injection, mode, orders):
    import torch
    mats, b, a = _batch(msq, orders)
    ctx.set_jacobi_vectors(mode)
    assert injection(FLAG) == 0
    ctx.jacobi(a.clone(), b, 1e-7, 15)
    with pytest.raises(msq.MsqError, match="wait expired"):
        ctx.synchronize()
    assert injection(0) == 0
    _, w, _, _ = ctx.jacobi(a.clone(), b, 1e-7, 15)
    ctx.set_jacobi_vectors(-1)
    ctx.synchronize()
    got = w.cpu().numpy()
    at = 0
    for n, m in zip(orders, mats):
        ref = np.linalg.eigvalsh(m)
        np.testing.assert_allclose(np.sort(got[at:at + n]), ref, rtol=0,
                                   atol=max(5e-6, 3 * n * 2.0 ** -24) * np.abs(ref).max())
        at += n


def test_tcgen05_mbarrier_wait_expiry_is_reported(msq, ctx, injection):
    import torch
    orders = [100, 256]
    rng = np.random.default_rng(3)
    fs = [rng.standard_normal((n, n)).astype(np.float32) / np.sqrt(n) for n in orders]
    b = msq.Batch.from_orders(orders)
    f = torch.from_numpy(b.pack(fs)).cuda()
    assert injection(MBARRIER) == 0
    ctx.reconstruct_factor(msq.PLAN_BF16, f, b)
    with pytest.raises(msq.MsqError, match="mbarrier wait expired"):
        ctx.synchronize()
    assert injection(0) == 0
    x = ctx.reconstruct_factor(msq.PLAN_BF16, f, b)
    ctx.synchronize()
    for fg, xg in zip(fs, b.unpack(x.cpu().numpy())):
        fq = fg.astype(np.float64)  # F = W^T K-major: X = fq^T fq up to BF16 rounding
        x_ref = fq.T @ fq
        assert np.linalg.norm(xg - x_ref) / np.linalg.norm(x_ref) < 1e-2


def test_solve_reports_an_expired_wait_and_recovers(msq, ctx, injection):
    orders = [40, 300]
    mats, b, a = _batch(msq, orders, seed=7)
    plans = [msq.plan(msq.PLAN_BF16, 1, 1e-4)] * len(orders)
    assert injection(MBARRIER) == 0
    with pytest.raises(msq.MsqError, match="mbarrier wait expired"):
        ctx.solve_batched(a, b, plans, tolerance=1e-5)
    assert injection(0) == 0
    root, res = ctx.solve_batched(a, b, plans, tolerance=1e-5)
    ctx.synchronize()
    for m, x, r in zip(mats, b.unpack(root.cpu().numpy()), res):
        assert r.final_residual <= 1e-5
        assert O.relative_residual(m, x) <= 2e-5


def test_noalloc_marks_its_outputs_when_a_wait_expires(msq, ctx, injection):
    import torch
    n = 256
    a0 = np.asfortranarray(O.wishart(n, seed=1), np.float32).reshape(-1, order="F")
    a = torch.from_numpy(a0.copy()).cuda()
    v = torch.empty_like(a)
    w = torch.empty(n, dtype=torch.float32, device="cuda")
    sweeps = torch.zeros(1, dtype=torch.int32, device="cuda")
    off = torch.zeros(1, dtype=torch.float32, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    call = msq.lib().msq_jacobi_noalloc
    assert injection(FLAG) == 0
    assert call(a.data_ptr(), v.data_ptr(), w.data_ptr(), n, 1e-7, 15, stream,
                sweeps.data_ptr(), off.data_ptr()) == 0
    torch.cuda.synchronize()
    assert np.isnan(w.cpu().numpy()).all()
    assert int(sweeps.item()) == -1 and np.isnan(float(off.item()))
    assert injection(0) == 0
    a.copy_(torch.from_numpy(a0).cuda())
    assert call(a.data_ptr(), v.data_ptr(), w.data_ptr(), n, 1e-7, 15, stream,
                sweeps.data_ptr(), off.data_ptr()) == 0
    torch.cuda.synchronize()
    assert int(sweeps.item()) > 0
    ref = np.linalg.eigvalsh(O.wishart(n, seed=1))
    np.testing.assert_allclose(np.sort(w.cpu().numpy()), ref, rtol=0,
                               atol=3 * n * 2.0 ** -24 * np.abs(ref).max())
