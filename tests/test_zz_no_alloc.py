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


def _noalloc(msq, a_np, tol=1e-7, max_sweeps=15):
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
                                          sweeps.data_ptr(), off.data_ptr())
    assert status == 0
    torch.cuda.synchronize()
    return (v.cpu().numpy().reshape(n, n, order="F"), w.cpu().numpy(), int(sweeps.item()),
            float(off.item()))


def _batched(ctx, msq, a_np):
    import torch
    b = msq.Batch.from_orders([a_np.shape[0]])
    a = torch.from_numpy(b.pack([a_np])).cuda()
    v, w, sweeps, off = ctx.jacobi(a, b, 1e-7, 15)
    torch.cuda.synchronize()
    return b.unpack(v.cpu().numpy())[0], w.cpu().numpy(), int(sweeps[0].item())


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
