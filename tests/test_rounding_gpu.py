"""Stochastic rounding and log-spectrum storage on the GPU (through the C ABI)
against the oracle (tests/test_rounding_oracle.py pins the oracle against the
reference).

Stochastic codes are compared bit for bit: the hash is integer arithmetic,
the sample is an exact 24-bit fraction and the round-up probability is an
exact quotient (adjacent codes differ by a power of two).  Log-spectrum
storage goes through log2 / exp2, which neither the GPU nor the C library
rounds correctly, so metadata and decoded values are compared within a few
ulps and codes must agree except where a value sits on a rounding boundary.
"""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

SEED = 0x2545F491
STREAM = 0x53520000


def _inputs(n: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    x = (rng.standard_normal(n) * np.exp2(rng.uniform(-12, 12, n))).astype(np.float32)
    specials = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 448.0, 500.0, -6.0, 7.0, 57344.0,
                         1e-40, -3e-39, 0.3, -0.3, 1.0, 1.25, -np.nan], dtype=np.float32)
    k = min(n, specials.size)
    x[:k] = specials[:k]
    return x


def _gpu_encode(ctx, fmt, x, seed, stream, row_length=0):
    import torch
    v, s = ctx.copy_to_storage_stochastic(fmt, torch.from_numpy(x).cuda(), seed, stream, row_length)
    torch.cuda.synchronize()
    vb = v.cpu().numpy()[:O.olib().msqo_storage_bytes(fmt, x.size)]
    return vb, (s.cpu().numpy() if s is not None else None)


@pytest.mark.parametrize("fmt", [1, 2, 3, 4, 5, 6, 7])
@pytest.mark.parametrize("n", [1, 31, 33, 1000, 65543])
def test_stochastic_codes_equal_the_oracle(ctx, msq, fmt, n):
    x = _inputs(n, 10 * fmt + n)
    for seed, stream in [(SEED, STREAM), (0, 0), (0xFFFFFFFF, 12345)]:
        v, s = _gpu_encode(ctx, fmt, x, seed, stream)
        ov, os_ = O.encode_stochastic(fmt, x, seed, stream)
        assert np.array_equal(v, ov), (fmt, n, seed, stream)
        if os_ is not None:
            assert np.array_equal(s[:os_.size], os_)


@pytest.mark.parametrize("row_length", [32, 100])
def test_stochastic_row_scaled_equals_the_oracle(ctx, msq, row_length):
    x = _inputs(row_length * 37, row_length)
    v, s = _gpu_encode(ctx, 8, x, SEED, STREAM, row_length)
    ov, os_ = O.encode_stochastic(8, x, SEED, STREAM, row_length)
    assert np.array_equal(v, ov)
    assert np.array_equal(s.view(np.uint8)[:os_.size], os_)


@pytest.mark.parametrize("fmt", [1, 2, 3, 4, 5, 6, 7])
def test_stochastic_passes_the_reference_check_on_the_gpu(ctx, msq, fmt):
    """checkStochasticQuantization (src/metal_checks.cpp:409-504): the same
    seed and stream reproduce the codes, another stream changes them, and
    the sample mean of decode - source stays within the reference's bound."""
    import torch
    x = np.full(65536, 0.3, dtype=np.float32)
    x[32768:] = -0.3
    xd = torch.from_numpy(x).cuda()
    v1, s1 = ctx.copy_to_storage_stochastic(fmt, xd, SEED, STREAM)
    v2, _ = ctx.copy_to_storage_stochastic(fmt, xd, SEED, STREAM)
    v3, _ = ctx.copy_to_storage_stochastic(fmt, xd, SEED, STREAM + 1)
    d = ctx.storage_values(fmt, v1, s1, x.size)
    torch.cuda.synchronize()
    assert torch.equal(v1, v2) and not torch.equal(v1, v3)
    d = d.cpu().numpy().astype(np.float64)
    err = max(abs(np.mean(d[:32768] - 0.3)), abs(np.mean(d[32768:] + 0.3)))
    tol = 5e-5 if fmt == 1 else (1e-2 if fmt in (6, 7) else 1e-3)
    assert err <= tol, err


def _spectra():
    rng = np.random.default_rng(77)
    wide = np.exp2(rng.uniform(-20, 20, 1001)).astype(np.float32)
    wide[8:16] = 3.0
    check = np.array([1.0, 1.5, 2.0, 3.0, 10.0, 31.622776, 100.0, 1000.0], dtype=np.float32)
    idx = np.arange(65536)
    pos = np.power((idx % 8) / np.float32(7.0), np.float32(1.3)).astype(np.float32)
    pattern = np.exp2(np.float32(-2.0) + np.float32(4.0) * pos).astype(np.float32)
    return {"wide": wide, "check": check, "pattern": pattern, "one": np.array([5.0], np.float32)}


@pytest.mark.parametrize("rounding", [0, 1])
@pytest.mark.parametrize("fmt", [2, 6])
def test_log_spectrum_matches_the_oracle(ctx, msq, fmt, rounding):
    import torch
    for name, s in _spectra().items():
        v, m = ctx.copy_spectrum_to_storage(fmt, torch.from_numpy(s).cuda(), rounding, SEED, STREAM)
        d = ctx.spectrum_values(fmt, v, m, s.size)
        ctx.synchronize()
        v = v.cpu().numpy()[:O.olib().msqo_storage_bytes(fmt, s.size)]
        m = m.cpu().numpy()[:O.spectrum_metadata_floats(s.size)]
        d = d.cpu().numpy()
        ov, om = O.spectrum_encode(fmt, s, bool(rounding), SEED, STREAM)
        # log2 on the GPU and in the C library may differ by an ulp
        np.testing.assert_allclose(m[0::2], om[0::2], rtol=0, atol=4e-6 * np.abs(om[0::2]).max() + 1e-30)
        np.testing.assert_allclose(m[1::2], om[1::2], rtol=0, atol=8e-6 * np.abs(om[0::2]).max() + 1e-30)
        codes = (np.stack([v & 15, v >> 4], 1).reshape(-1)[:s.size] if fmt == 6 else v)
        ocodes = (np.stack([ov & 15, ov >> 4], 1).reshape(-1)[:s.size] if fmt == 6 else ov)
        assert np.mean(codes == ocodes) >= 0.995, name
        assert np.all(np.abs(codes.astype(int) - ocodes.astype(int)) <= 1), name
        # the GPU decoder against the oracle's on the GPU's codes and metadata
        np.testing.assert_allclose(d, O.spectrum_decode(fmt, v, m, s.size), rtol=4e-6, atol=0)
        if name == "check":
            assert np.max(np.abs(d.astype(np.float64) / s - 1.0)) < (0.5 if fmt == 2 else 4.0)


def test_log_spectrum_rejects_non_positive_input(ctx, msq):
    """A zero or negative root eigenvalue sets the device status (the
    reference host codec fails on it); the context reports it and recovers."""
    import torch
    s = torch.tensor([1.0, 0.0, 2.0], device="cuda")
    ctx.copy_spectrum_to_storage(2, s)
    with pytest.raises(RuntimeError, match="log-spectrum"):
        ctx.synchronize()
    v, m = ctx.copy_spectrum_to_storage(2, torch.tensor([1.0, 2.0], device="cuda"))
    ctx.synchronize()


@pytest.mark.parametrize("fmt", [0, 1, 2, 3, 4, 5, 6, 7, 8])
@pytest.mark.parametrize("n", [1, 7, 33, 64])
def test_native_correction_equals_the_oracle(ctx, msq, fmt, n):
    """msq_native_sylvester_sweep from X = 0 leaves (E + E^T) / 2 with E the
    oracle's native correction, bit for bit (same quantizer, same FMA
    chains, same divisions)."""
    import torch
    rng = np.random.default_rng(100 * fmt + n)
    q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    v = q.astype(np.float32)
    rl = n if fmt == 8 else 0
    def stored(m):
        if fmt == 0:
            return np.asfortranarray(m, np.float32)
        flat = np.asfortranarray(m, np.float32).reshape(-1, order="F")
        return O.decode(fmt, *O.encode(fmt, flat, rl), flat.size, rl).reshape(n, n, order="F")
    vq, vtq = stored(v), stored(v.T)
    s = np.exp(rng.uniform(-1, 1, n)).astype(np.float32)
    r = (1e-3 * rng.standard_normal((n, n))).astype(np.float32)
    r = np.asfortranarray(0.5 * (r + r.T))
    e = O.native_correction(fmt, vq, vtq, s, r)
    b = msq.Batch.from_orders([n])
    col = lambda m: torch.from_numpy(b.pack([np.asfortranarray(m, np.float32)])).cuda()
    x_hi = torch.zeros(b.total, dtype=torch.float32, device="cuda")
    x_lo = torch.zeros_like(x_hi)
    ctx.native_sylvester_sweep(fmt, col(vq), col(vtq), torch.from_numpy(s).cuda(), col(r), b,
                               x_hi, x_lo)
    ctx.synchronize()
    got = b.unpack(x_hi.cpu().numpy(), dtype=np.float32)[0]
    # the float-float add starts from x = +0: +0 + corr turns a -0 into +0
    want = (np.float32(0.5) * (e + e.T) + np.float32(0.0)).astype(np.float32)
    assert np.array_equal(np.ascontiguousarray(got).view(np.uint32),
                          np.ascontiguousarray(want).view(np.uint32))


@pytest.mark.parametrize("fmt", [0, 1, 3, 5, 7, 8])
def test_native_correction_batched_equals_the_oracle(ctx, msq, fmt):
    """A batch of uneven orders in one call (each step one launch over the
    batch; MX blocks and scale rows within each matrix): every matrix equals
    the oracle's native correction of that matrix alone, bit for bit."""
    import torch
    orders = [1, 7, 33, 64, 100, 5]
    rng = np.random.default_rng(900 + fmt)
    rl = lambda n: n if fmt == 8 else 0

    def stored(m, n):
        if fmt == 0:
            return np.asfortranarray(m, np.float32)
        flat = np.asfortranarray(m, np.float32).reshape(-1, order="F")
        return O.decode(fmt, *O.encode(fmt, flat, rl(n)), flat.size, rl(n)).reshape(n, n, order="F")

    vqs, vtqs, ss, rs, want = [], [], [], [], []
    for n in orders:
        q, _ = np.linalg.qr(rng.standard_normal((n, n)))
        v = q.astype(np.float32)
        vq, vtq = stored(v, n), stored(v.T, n)
        s = np.exp(rng.uniform(-1, 1, n)).astype(np.float32)
        r = (1e-3 * rng.standard_normal((n, n))).astype(np.float32)
        r = np.asfortranarray(0.5 * (r + r.T))
        e = O.native_correction(fmt, vq, vtq, s, r)
        vqs.append(vq); vtqs.append(vtq); ss.append(s); rs.append(r)
        want.append((np.float32(0.5) * (e + e.T) + np.float32(0.0)).astype(np.float32))
    b = msq.Batch.from_orders(orders)
    col = lambda ms: torch.from_numpy(b.pack([np.asfortranarray(m, np.float32) for m in ms])).cuda()
    x_hi = torch.zeros(b.total, dtype=torch.float32, device="cuda")
    x_lo = torch.zeros_like(x_hi)
    l0 = ctx.launches
    ctx.native_sylvester_sweep(fmt, col(vqs), col(vtqs), torch.from_numpy(np.concatenate(ss)).cuda(),
                               col(rs), b, x_hi, x_lo)
    ctx.synchronize()
    assert ctx.launches - l0 <= 13  # one launch per step, whatever the batch size
    for n, got, w in zip(orders, b.unpack(x_hi.cpu().numpy(), dtype=np.float32), want):
        assert np.array_equal(np.ascontiguousarray(got).view(np.uint32),
                              np.ascontiguousarray(w).view(np.uint32)), n
