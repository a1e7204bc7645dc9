"""GPU codec parity: the CUDA encoders/decoders, called through the C ABI,
must reproduce the reference host codec bit for bit (golden vectors from the
reference's compiled copyToStorage/storageValueAt, and the oracle restatement
on seeded tensors)."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

ALL = list(range(9))


def _gpu_roundtrip(ctx, fmt, x, row_length=0):
    import torch
    t = torch.from_numpy(np.ascontiguousarray(x, np.float32)).cuda()
    v, s = ctx.copy_to_storage(fmt, t, row_length)
    d = ctx.storage_values(fmt, v, s, x.size, row_length)
    torch.cuda.synchronize()
    return (v.cpu().numpy()[:ctx_storage(fmt, x.size)], None if s is None else s.cpu().numpy(),
            d.cpu().numpy())


def ctx_storage(fmt, n):
    import importlib
    return importlib.import_module("mixed-mlx_gb300").storage_bytes(fmt, n)


@pytest.mark.parametrize("fmt", range(8))
def test_golden_vectors_bit_exact(ctx, golden_codecs, fmt):
    x = golden_codecs["x"]
    v, s, d = _gpu_roundtrip(ctx, fmt, x)
    np.testing.assert_array_equal(v, golden_codecs[f"values_{fmt}"])
    if golden_codecs[f"scales_{fmt}"].size:
        np.testing.assert_array_equal(s, golden_codecs[f"scales_{fmt}"])
    np.testing.assert_array_equal(d.view(np.uint32), golden_codecs[f"decoded_bits_{fmt}"])


@pytest.mark.parametrize("fmt", range(8))
@pytest.mark.parametrize("size", [0, 1, 7, 31, 32, 33, 63, 1000, 4097])
def test_ragged_sizes_bit_exact(ctx, fmt, size):
    rng = np.random.default_rng(size * 10 + fmt)
    x = (rng.standard_normal(size) * 2.0 ** rng.integers(-12, 12, size)).astype(np.float32)
    if size == 0:
        return
    v, s, d = _gpu_roundtrip(ctx, fmt, x)
    ov, os_ = O.encode(fmt, x)
    np.testing.assert_array_equal(v, ov)
    if os_ is not None:
        np.testing.assert_array_equal(s, os_)
    np.testing.assert_array_equal(d.view(np.uint32), O.decode(fmt, ov, os_, size).view(np.uint32))


@pytest.mark.parametrize("fmt", range(8))
@pytest.mark.parametrize("dist", ["normal", "student_t3", "wide"])
def test_seeded_tensors_2p20_bit_exact(ctx, fmt, dist):
    """N(0,1) / Student-t(3) / sign*2^U(-30,30) tensors of 2^20 elements.
    (2^20 keeps the linear-scan oracle fast; larger sizes are checked through
    size-independent properties below.)"""
    rng = np.random.default_rng(fmt * 10 + ["normal", "student_t3", "wide"].index(dist))
    n = 1 << 20
    if dist == "normal":
        x = rng.standard_normal(n)
    elif dist == "student_t3":
        x = rng.standard_t(3, n)
    else:
        x = np.sign(rng.standard_normal(n)) * 2.0 ** rng.uniform(-30, 30, n)
    x = x.astype(np.float32)
    if fmt in (2, 3, 4, 5):
        idx = rng.choice(n, 1 << 16, replace=False)  # linear-scan oracle is slow
    else:
        idx = None
    v, s, d = _gpu_roundtrip(ctx, fmt, x)
    if idx is None:
        ov, os_ = O.encode(fmt, x)
        np.testing.assert_array_equal(v, ov)
        if os_ is not None:
            np.testing.assert_array_equal(s, os_)
        np.testing.assert_array_equal(d.view(np.uint32), O.decode(fmt, ov, os_, n).view(np.uint32))
    else:
        # check whole 32-blocks around the sampled indices
        blocks = np.unique(idx // 32)
        sel = (blocks[:, None] * 32 + np.arange(32)).reshape(-1)
        ov, os_ = O.encode(fmt, x[sel])
        np.testing.assert_array_equal(v[sel] if fmt != 1 else v.view(np.uint16)[sel].view(np.uint8), ov)
        if os_ is not None:
            np.testing.assert_array_equal(s[blocks], os_)
        np.testing.assert_array_equal(d[sel].view(np.uint32), O.decode(fmt, ov, os_, sel.size).view(np.uint32))


@pytest.mark.parametrize("row_length", [1, 5, 64, 1000])
def test_rowscale_bit_exact(ctx, row_length):
    rng = np.random.default_rng(row_length)
    rows = 37
    x = (rng.standard_normal(rows * row_length) * 10.0 ** rng.uniform(-3, 3)).astype(np.float32)
    x[:row_length] = 0.0  # an all-zero row takes scale 1
    v, s, d = _gpu_roundtrip(ctx, 8, x, row_length)
    ov, os_ = O.encode(8, x, row_length)
    np.testing.assert_array_equal(v, ov)
    np.testing.assert_array_equal(s, os_)
    np.testing.assert_array_equal(d.view(np.uint32), O.decode(8, ov, os_, x.size, row_length).view(np.uint32))


@pytest.mark.parametrize("fmt", [1, 2, 3, 4, 5, 6, 7])
def test_large_2p26_roundtrip_properties(ctx, fmt):
    """2^26 elements: decode(encode(x)) is idempotent under re-encoding, and
    the GPU decode of a block agrees with the oracle on sampled blocks."""
    import torch
    n = 1 << 26
    g = torch.Generator(device="cuda").manual_seed(fmt)
    x = torch.randn(n, device="cuda", generator=g)
    v, s = ctx.copy_to_storage(fmt, x)
    d = ctx.storage_values(fmt, v, s, n)
    v2, s2 = ctx.copy_to_storage(fmt, d)
    assert torch.equal(v, v2)
    if s is not None:
        assert torch.equal(s, s2)
    rng = np.random.default_rng(fmt)
    blocks = rng.integers(0, n // 32, 512)
    sel = torch.from_numpy((blocks[:, None] * 32 + np.arange(32)).reshape(-1)).cuda()
    xs = x[sel].cpu().numpy()
    ov, os_ = O.encode(fmt, xs)
    od = O.decode(fmt, ov, os_, xs.size)
    np.testing.assert_array_equal(d[sel].cpu().numpy().view(np.uint32), od.view(np.uint32))


@pytest.mark.parametrize("dist", ["normal", "student_t3"])
def test_mxfp4_2p26_full_tensor_bit_exact(ctx, dist):
    """The MXFP4 round trip at 2^26 elements (E2M1 codes, one E8M0 scale per
    32): every code, scale and decoded value equals the oracle's, for N(0,1)
    and heavy-tailed Student-t(3) tensors."""
    import torch
    n = 1 << 26
    rng = np.random.default_rng(26 + (dist == "student_t3"))
    x = (rng.standard_normal(n) if dist == "normal" else rng.standard_t(3, n)).astype(np.float32)
    fmt = 7  # MXFP4_E2M1
    t = torch.from_numpy(x).cuda()
    v, s = ctx.copy_to_storage(fmt, t)
    d = ctx.storage_values(fmt, v, s, n)
    torch.cuda.synchronize()
    ov, os_ = O.encode(fmt, x)
    np.testing.assert_array_equal(v.cpu().numpy()[:ov.size], ov)
    np.testing.assert_array_equal(s.cpu().numpy()[:os_.size], os_)
    od = O.decode(fmt, ov, os_, n)
    np.testing.assert_array_equal(d.cpu().numpy().view(np.uint32), od.view(np.uint32))


def test_misaligned_pointers_fall_back_to_scalar_path(ctx):
    import torch
    x = torch.randn(1001, device="cuda")
    xs = x[1:]  # 4-byte offset: not 16-byte aligned
    for fmt in (1, 2, 7):
        v, s = ctx.copy_to_storage(fmt, xs)
        ov, os_ = O.encode(fmt, xs.cpu().numpy())
        np.testing.assert_array_equal(v.cpu().numpy()[:ov.size], ov)
