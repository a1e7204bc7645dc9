"""The allocation-free Jacobi entry point (msq_jacobi_noalloc).

It exists for callers that must not allocate device memory: latency-critical
loops that must not wait on the allocator's device synchronisation, and host
applications that own all device memory.  It must agree with the regular
entry point (msq_jacobi_batched on a one-matrix batch), call after call, even
though every call reuses the same static device scratch.  This file sorts last so a
run that stops at the first failure has already run everything else.
"""
import ctypes

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def _noalloc(msq, a_np, tol=1e-7, max_sweeps=15, report=True):
    import torch
    n = a_np.shape[0]
    a = torch.from_numpy(np.asfortranarray(a_np, np.float32).reshape(-1, order="F").copy()).cuda()
    v = torch.empty_like(a)
    w = torch.empty(n, dtype=torch.float32, device="cuda")
    sweeps = torch.zeros(1, dtype=torch.int32, device="cuda")
    off = torch.zeros(1, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    status = msq.lib().msq_jacobi_noalloc(a.data_ptr(), v.data_ptr(), w.data_ptr(), n, tol,
                                          max_sweeps, ctypes.c_void_p(stream.cuda_stream),
                                          sweeps.data_ptr() if report else None,
                                          off.data_ptr() if report else None)
    assert status == 0
    torch.cuda.synchronize()
    return (v.cpu().numpy().reshape(n, n, order="F"), w.cpu().numpy(), int(sweeps.item()),
            float(off.item()))


def _batched(ctx, msq, a_np, max_sweeps=15):
    import torch
    b = msq.Batch.from_orders([a_np.shape[0]])
    a = torch.from_numpy(b.pack([a_np])).cuda()
    v, w, sweeps, off = ctx.jacobi(a, b, 1e-7, max_sweeps)
    torch.cuda.synchronize()
    return b.unpack(v.cpu().numpy())[0], w.cpu().numpy(), int(sweeps[0].item())


def _agree(msq, ctx, a):
    v_na, w_na, s_na, off_na = _noalloc(msq, a)
    v_b, w_b, s_b = _batched(ctx, msq, a)
    scale = np.abs(w_b).max()
    assert s_na == s_b and off_na <= 1e-7
    np.testing.assert_allclose(w_na, w_b, rtol=0, atol=1e-6 * scale)
    np.testing.assert_allclose(v_na, v_b, rtol=0, atol=1e-5)


@pytest.mark.parametrize("n", [5, 96, 256])
def test_noalloc_matches_batched_entry_point_twice(ctx, msq, n):
    a1 = O.spd_loguniform(n, 1e3, seed=11 * n)
    a2 = O.wishart(n, seed=n + 1)
    for a in (a1, a2):  # two calls in a row reuse the same static scratch
        v_na, w_na, s_na, off_na = _noalloc(msq, a)
        v_b, w_b, s_b = _batched(ctx, msq, a)
        scale = np.abs(w_b).max()
        assert s_na == s_b and off_na <= 1e-7
        np.testing.assert_allclose(w_na, w_b, rtol=0, atol=1e-6 * scale)
        np.testing.assert_allclose(v_na, v_b, rtol=0, atol=1e-5)
        ref = np.linalg.eigvalsh(a)
        # FP32 Jacobi: eigenvalue error of order n * u * ||A|| (u = 2^-24)
        np.testing.assert_allclose(np.sort(w_na), ref, rtol=0, atol=max(5e-6, 3 * n * 2.0**-24) * scale)


def test_noalloc_rejects_orders_beyond_its_scratch(msq):
    import torch
    n = msq.lib().msq_jacobi_noalloc  # noqa: F841  (symbol present)
    big = 257
    a = torch.zeros(big * big, device="cuda")
    status = msq.lib().msq_jacobi_noalloc(a.data_ptr(), a.data_ptr(), a.data_ptr(), big, 1e-7, 15,
                                          None, None, None)
    assert status == 1  # MSQ_ERR_INVALID_ARGUMENT, nothing launched


def test_noalloc_large_then_small_order_on_the_shared_scratch(ctx, msq):
    # the second call must not see anything the first left in the array
    _agree(msq, ctx, O.wishart(256, seed=3))
    _agree(msq, ctx, O.spd_loguniform(5, 1e2, seed=4))
    _agree(msq, ctx, O.wishart(40, seed=5))


def test_noalloc_zero_sweeps_without_report_pointers(ctx, msq):
    a = O.spd_loguniform(64, 1e3, seed=21)
    v_na, w_na, _, _ = _noalloc(msq, a, max_sweeps=0, report=False)
    v_b, w_b, s_b = _batched(ctx, msq, a, max_sweeps=0)
    assert s_b == 0
    np.testing.assert_array_equal(w_na, w_b)
    np.testing.assert_array_equal(v_na, v_b)
    # no sweep: the eigenvalues are the diagonal, the vectors the identity
    np.testing.assert_allclose(w_na, np.diag(a).astype(np.float32), rtol=0, atol=0)
    np.testing.assert_array_equal(v_na, np.eye(64, dtype=np.float32))


def test_noalloc_call_after_the_first_allocates_nothing(msq):
    import torch
    n = 200
    a0 = np.asfortranarray(O.wishart(n, seed=9), np.float32).reshape(-1, order="F")
    a_src = torch.from_numpy(a0.copy()).cuda()
    a = torch.empty_like(a_src)
    v = torch.empty_like(a)
    w = torch.empty(n, dtype=torch.float32, device="cuda")
    sweeps = torch.zeros(1, dtype=torch.int32, device="cuda")
    off = torch.zeros(1, dtype=torch.float32, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    call = msq.lib().msq_jacobi_noalloc
    a.copy_(a_src)
    assert call(a.data_ptr(), v.data_ptr(), w.data_ptr(), n, 1e-7, 15, stream,
                sweeps.data_ptr(), off.data_ptr()) == 0  # first call: set-up
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()  # cudaMemGetInfo
    for _ in range(3):
        a.copy_(a_src)  # the call overwrites its input; a device copy allocates nothing
        assert call(a.data_ptr(), v.data_ptr(), w.data_ptr(), n, 1e-7, 15, stream,
                    sweeps.data_ptr(), off.data_ptr()) == 0
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before
    assert int(sweeps.item()) > 0
