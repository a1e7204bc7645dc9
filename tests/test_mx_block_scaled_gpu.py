"""Block-scaled MMA (tcgen05.mma kind::mxf4 / kind::mxf8f6f4 .block_scale)
for MX factors: X0 = Q(W) Q(W)^T with E2M1 or E4M3 codes and one UE8M0
scale per 32 consecutive K of a row, the scale factors applied inside the
tensor core.  Checked against the FP64 product of the oracle's decoded
factor (the reference's MX codec restated), so only the FP32 accumulation
error remains: relative Frobenius error below 2e-6."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

ACC = 2e-6  # FP32 accumulation of an n-long sum of exact products


def _dev(x):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x, np.float32)).cuda()


def _factor(n, seed):
    """F = W^T (K-major: column i of the column-major storage is row i of W)
    from a random orthonormal V and lambda log-uniform on [1e-3, 1]."""
    rng = np.random.default_rng(seed)
    v = np.linalg.qr(rng.standard_normal((n, n)))[0]
    lam = np.exp(rng.uniform(np.log(1e-3), 0.0, n))
    return (v * lam ** 0.25).T.astype(np.float32)


def _per_row_decoded(fmt, f):
    """The oracle's codec applied to each K-major row of W on its own (blocks
    of 32 start at every row), decoded; rows as the columns of the result."""
    n = f.shape[0]
    cols = []
    for i in range(n):
        col = np.ascontiguousarray(f[:, i], np.float32)
        v, s = O.encode(fmt, col)
        cols.append(O.decode(fmt, v, s, n))
    return np.stack(cols, axis=1).astype(np.float64)


@pytest.mark.parametrize("orders", [[256], [1, 31, 100, 129, 257, 300, 512], [64, 96, 128]])
def test_mxfp4_plan_reconstruction_from_the_factor(ctx, msq, orders):
    """The solver's MXFP4 stage at any order (ragged last block per row)."""
    import torch
    b = msq.Batch.from_orders(orders)
    fs = [_factor(n, seed=n) for n in orders]
    f = _dev(b.pack(fs))
    x = ctx.reconstruct_factor(msq.PLAN_MXFP4, f, b)
    torch.cuda.synchronize()
    for n, fg, xg in zip(orders, fs, b.unpack(x.cpu().numpy())):
        fq = _per_row_decoded(msq.MXFP4_E2M1, fg)
        x_ref = fq.T @ fq
        err = np.linalg.norm(xg - x_ref) / np.linalg.norm(x_ref)
        assert err < ACC, (n, err)


@pytest.mark.parametrize("fmt_name", ["MXFP4_E2M1", "MXFP8_E4M3FN"])
@pytest.mark.parametrize("n", [32, 128, 256, 512])
def test_mx_codes_reconstruction(ctx, msq, fmt_name, n):
    """msq_reconstruct straight from the flat codec's codes and scale bytes
    (order divisible by 32: the flat blocks are row blocks)."""
    import torch
    fmt = getattr(msq, fmt_name)
    f = _factor(n, seed=3 * n + 1)
    single = msq.Batch.from_orders([n])
    flat = np.ascontiguousarray(f.reshape(-1, order="F"))
    vals, scl = ctx.copy_to_storage(fmt, _dev(flat))
    ov, os_ = O.encode(fmt, flat)
    assert np.array_equal(vals.cpu().numpy(), ov) and np.array_equal(scl.cpu().numpy(), os_)
    x = ctx.reconstruct(fmt, vals, scl, single)
    torch.cuda.synchronize()
    fq = O.decode(fmt, ov, os_, n * n).reshape(n, n, order="F").astype(np.float64)
    x_ref = fq.T @ fq
    xg = single.unpack(x.cpu().numpy())[0]
    err = np.linalg.norm(xg - x_ref) / np.linalg.norm(x_ref)
    assert err < ACC, err


def test_mx_block_scaled_agrees_with_exact_bf16_decode(ctx, msq):
    """Ragged flat MXFP4 codes (order 100: blocks straddle rows) take the
    exact BF16 decode with kind::f16; the same codes re-laid per row take
    kind::mxf4.  Both equal the oracle's decoded product."""
    import torch
    n = 100
    f = _factor(n, seed=5)
    single = msq.Batch.from_orders([n])
    flat = np.ascontiguousarray(f.reshape(-1, order="F"))
    vals, scl = ctx.copy_to_storage(msq.MXFP4_E2M1, _dev(flat))
    x = ctx.reconstruct(msq.MXFP4_E2M1, vals, scl, single)
    torch.cuda.synchronize()
    ov, os_ = O.encode(msq.MXFP4_E2M1, flat)
    fq = O.decode(msq.MXFP4_E2M1, ov, os_, n * n).reshape(n, n, order="F").astype(np.float64)
    x_ref = fq.T @ fq
    xg = single.unpack(x.cpu().numpy())[0]
    assert np.linalg.norm(xg - x_ref) / np.linalg.norm(x_ref) < ACC


def test_mxfp8_ragged_order_is_reported_unsupported(ctx, msq):
    import torch
    n = 100
    single = msq.Batch.from_orders([n])
    vals, scl = ctx.copy_to_storage(msq.MXFP8_E4M3FN, torch.ones(n * n, device="cuda"))
    with pytest.raises(msq.MsqError):
        ctx.reconstruct(msq.MXFP8_E4M3FN, vals, scl, single)


def test_mxfp4_reconstruction_order_8192(ctx, msq):
    """n = 8192 (the MXFP4 single-matrix case): the kind::mxf4 product of the
    per-row-quantized factor against the FP64 product of the oracle's decode."""
    import torch
    n = 8192
    rng = np.random.default_rng(8192)
    # a random factor with the spread of an eigenbasis scaled by lambda^(1/4)
    f = (rng.standard_normal((n, n)) / np.sqrt(n) *
         np.exp(rng.uniform(np.log(1e-1), 0.0, n))[None, :]).astype(np.float32)
    b = msq.Batch.from_orders([n])
    x = ctx.reconstruct_factor(msq.PLAN_MXFP4, _dev(b.pack([f])), b)
    torch.cuda.synchronize()
    xg = b.unpack(x.cpu().numpy())[0]
    del x
    # per-row blocks of 32 with n divisible by 32: the flat codec of the
    # K-major storage has the same blocks
    flat = np.ascontiguousarray(f.reshape(-1, order="F"))
    ov, os_ = O.encode(msq.MXFP4_E2M1, flat)
    fq = O.decode(msq.MXFP4_E2M1, ov, os_, n * n).reshape(n, n, order="F").astype(np.float64)
    x_ref = fq.T @ fq
    err = np.linalg.norm(xg - x_ref) / np.linalg.norm(x_ref)
    assert err < ACC, err
