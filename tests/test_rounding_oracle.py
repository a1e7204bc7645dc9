"""The oracle's stochastic rounding and log-spectrum storage, pinned by the
reference.

* Log-spectrum storage: codes, (min, span) metadata and decoded values against
  the reference host codec's own outputs (copySpectrumToStorage /
  spectrumValueAt, src/storage_codecs.cpp:387-460, recorded in
  tests/golden/spectrum.npz by tests/golden/make_golden.py).  The oracle
  restates the device form (metal_mixed_sqrt.metal:1689-1804), whose span
  is one ulp lower when min + span rounds above the block maximum and whose
  decode evaluates (span * code) / max instead of span * (code / max).
* Stochastic rounding exists only in the reference's shaders
  (metal_mixed_sqrt.metal:394-405, 462-484, 545-568, 740-763, 1888-1907):
  the oracle is checked with the reference's own test of it
  (checkStochasticQuantization, src/metal_checks.cpp:409-504) and with its
  definition (a code is the nearest one or the neighbour on the value's other
  side).
"""
import os

import numpy as np
import pytest

import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FORMATS = [1, 2, 3, 4, 5, 6, 7, 8]
SEED = 0x2545F491
STREAM = 0x53520000  # the stream of checkStochasticQuantization


def check_source(elements: int = 65536, fmt: int = 2) -> np.ndarray:
    """checkStochasticQuantization's input for the linear formats.  The
    row-scaled format (no reference counterpart) would map a constant row
    onto its largest code exactly, so each of its rows gets one element of
    magnitude 0.5."""
    x = np.full(elements, 0.3, dtype=np.float32)
    x[elements // 2:] = -0.3
    if fmt == 8:
        x[::256] *= np.float32(0.5 / 0.3)
    return x


def bias_tolerance(fmt: int) -> float:
    return 5e-5 if fmt == 1 else (1e-2 if fmt in (6, 7) else 1e-3)


def row_length(fmt: int) -> int:
    return 256 if fmt == 8 else 0


@pytest.mark.parametrize("fmt", FORMATS)
def test_stochastic_passes_the_reference_check(fmt):
    x = check_source(fmt=fmt)
    rl = row_length(fmt)
    v1, s1 = O.encode_stochastic(fmt, x, SEED, STREAM, rl)
    v2, s2 = O.encode_stochastic(fmt, x, SEED, STREAM, rl)
    assert np.array_equal(v1, v2)                      # reproducible
    v3, _ = O.encode_stochastic(fmt, x, SEED, STREAM + 1, rl)
    assert not np.array_equal(v1, v3)                  # the stream matters
    d = O.decode(fmt, v1, s1, x.size, rl).astype(np.float64)
    half = x.size // 2
    err = max(abs(np.mean(d[:half] - x[:half])), abs(np.mean(d[half:] - x[half:])))
    assert err <= bias_tolerance(fmt), err


def _inputs(n: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    x = (rng.standard_normal(n) * np.exp2(rng.uniform(-12, 12, n))).astype(np.float32)
    specials = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 448.0, 500.0, -6.0, 7.0, 57344.0,
                         1e-40, -3e-39, 0.3, -0.3, 1.0, 1.25], dtype=np.float32)
    x[:specials.size] = specials
    return x


@pytest.mark.parametrize("fmt", [1, 2, 3, 6])
def test_stochastic_codes_are_the_bracketing_codes(fmt):
    """A stochastic code is the nearest code or the adjacent code on the
    other side of the value; exact values and specials keep the nearest."""
    x = _inputs(20000, fmt)
    vn, _ = O.encode(fmt, x)
    vs, _ = O.encode_stochastic(fmt, x, SEED, 7)
    dn = O.decode(fmt, vn, None, x.size).astype(np.float64)
    ds = O.decode(fmt, vs, None, x.size).astype(np.float64)
    if fmt == 1:
        cn, cs = vn.view(np.uint16).astype(np.int64), vs.view(np.uint16).astype(np.int64)
        mag = 0x7FFF
    elif fmt == 6:
        cn = np.stack([vn & 15, vn >> 4], 1).reshape(-1)[:x.size].astype(np.int64)
        cs = np.stack([vs & 15, vs >> 4], 1).reshape(-1)[:x.size].astype(np.int64)
        mag = 0x7
    else:
        cn, cs = vn.astype(np.int64), vs.astype(np.int64)
        mag = 0x7F
    same = (dn == ds) | (np.isnan(dn) & np.isnan(ds))
    differ = ~same
    # adjacent magnitude codes of the same sign
    assert np.all(np.abs((cs & mag) - (cn & mag))[differ] == 1)
    xs = x.astype(np.float64)[differ]
    lo, hi = np.minimum(dn[differ], ds[differ]), np.maximum(dn[differ], ds[differ])
    assert np.all((lo < xs) & (xs < hi))
    # values that are codes, and the specials, do not move
    exact = dn == x.astype(np.float64)
    assert np.all(same[exact])
    top = {1: 3.3895e38, 2: 448.0, 3: 57344.0, 6: 6.0}[fmt]
    between = np.isfinite(x) & (np.abs(x) > 0) & (np.abs(x) < top) & ~exact
    assert differ.sum() > 0.05 * between.sum()  # the random path is exercised


def test_stochastic_hash_is_the_shader_hash():
    """stochastic_hash (metal_mixed_sqrt.metal:394-398) on a few words,
    evaluated here with Python integers."""
    def h(i, seed, stream):
        m = 0xFFFFFFFF
        state = (i * 747796405 + seed + stream * 2891336453) & m
        word = (((state >> ((state >> 28) + 4)) ^ state) * 277803737) & m
        return (word >> 22) ^ word
    for i, seed, stream in [(0, 0, 0), (1, 2, 3), (65535, SEED, STREAM), (2**31 + 5, 7, 2**32 - 1)]:
        assert O.olib().msqo_stochastic_hash(i, seed, stream) == h(i, seed, stream)


@pytest.fixture(scope="module")
def golden_spectrum():
    return np.load(os.path.join(GOLDEN, "spectrum.npz"))


@pytest.mark.parametrize("case", ["check", "pattern", "wide"])
@pytest.mark.parametrize("fmt", [2, 6])
def test_log_spectrum_matches_the_reference_host_codec(golden_spectrum, case, fmt):
    s = golden_spectrum[f"{case}_input"]
    ref_v = golden_spectrum[f"{case}_values_{fmt}"]
    ref_m = golden_spectrum[f"{case}_meta_{fmt}"]
    ref_d = golden_spectrum[f"{case}_decoded_{fmt}"]
    v, m = O.spectrum_encode(fmt, s)
    assert np.array_equal(m[0::2], ref_m[0::2])                       # block minima
    span, ref_span = m[1::2], ref_m[1::2]
    assert np.all((span == ref_span) | (span == np.nextafter(ref_span, np.float32(0))))
    assert np.array_equal(v, ref_v)                                   # codes
    d = O.spectrum_decode(fmt, v, m, s.size)
    # the device form's one-ulp span and (span * code) / max ordering move the
    # log-domain argument (|min| up to 20 here) by a few ulps: exp2 of it by
    # a few 1e-6 relative
    np.testing.assert_allclose(d, ref_d, rtol=1e-5, atol=0)


@pytest.mark.parametrize("fmt,bound", [(2, 0.5), (6, 4.0)])
def test_log_spectrum_passes_the_reference_check(golden_spectrum, fmt, bound):
    """checkLogSpectrumStorage (src/metal_checks.cpp:506-534)."""
    s = golden_spectrum["check_input"]
    v, m = O.spectrum_encode(fmt, s)
    d = O.spectrum_decode(fmt, v, m, s.size).astype(np.float64)
    assert np.all(np.isfinite(d) & (d > 0))
    assert np.max(np.abs(d / s - 1.0)) < bound


@pytest.mark.parametrize("fmt", [2, 6])
def test_log_spectrum_stochastic_is_unbiased_in_log2(golden_spectrum, fmt):
    """checkStochasticQuantization's log-spectrum leg: the sample mean of
    log2(decoded) - log2(s) over 65536 values."""
    idx = np.arange(65536)
    pos = np.power((idx % 8) / np.float32(7.0), np.float32(1.3)).astype(np.float32)
    s = np.exp2(np.float32(-2.0) + np.float32(4.0) * pos).astype(np.float32)
    v, m = O.spectrum_encode(fmt, s, True, SEED, STREAM)
    v2, _ = O.spectrum_encode(fmt, s, True, SEED, STREAM + 1)
    assert not np.array_equal(v, v2)
    d = O.spectrum_decode(fmt, v, m, s.size).astype(np.float64)
    err = abs(np.mean(np.log2(d) - np.log2(s.astype(np.float64))))
    assert err <= (1e-2 if fmt == 6 else 1e-3), err


def test_log_spectrum_rejects_non_positive_input():
    for bad in ([1.0, 0.0], [1.0, -2.0], [np.inf, 1.0], [np.nan]):
        with pytest.raises(ValueError):
            O.spectrum_encode(2, np.array(bad, dtype=np.float32))


def _near_root_case(n: int, seed: int):
    rng = np.random.default_rng(seed)
    q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    s = np.exp(rng.uniform(-1.0, 1.0, n))
    a = (q * s ** 2) @ q.T
    x0 = (q * s) @ q.T + 1e-3 * rng.standard_normal((n, n))
    x0 = 0.5 * (x0 + x0.T)
    return q, s, a, x0, a - x0 @ x0


def test_native_correction_in_fp32_is_the_sylvester_correction():
    """With FP32 storage the native correction is E = V ((V^T R V) o H) V^T
    (refineNativeStaged with no quantizer)."""
    q, s, a, x0, r = _near_root_case(24, 1)
    f = lambda m: m.astype(np.float32)
    e = O.native_correction(0, f(q), f(q.T), f(s), f(r))
    e64 = q @ ((q.T @ r @ q) / (s[:, None] + s[None, :])) @ q.T
    assert np.abs(e - e64).max() <= 1e-5 * np.abs(e64).max()


@pytest.mark.parametrize("fmt,gain", [(0, 1e-2), (1, 1e-1), (8, 0.5), (7, 0.5)])
def test_native_correction_reduces_the_residual(fmt, gain):
    q, s, a, x0, r = _near_root_case(24, 2)
    f = lambda m: m.astype(np.float32)
    vq = O.decode(fmt, *O.encode(fmt, f(q).reshape(-1, order="F"), 24 if fmt == 8 else 0),
                  24 * 24, 24 if fmt == 8 else 0).reshape(24, 24, order="F") if fmt else f(q)
    vtq = O.decode(fmt, *O.encode(fmt, f(q.T).reshape(-1, order="F"), 24 if fmt == 8 else 0),
                   24 * 24, 24 if fmt == 8 else 0).reshape(24, 24, order="F") if fmt else f(q.T)
    e = O.native_correction(fmt, vq, vtq, f(s), f(r))
    x1 = x0 + 0.5 * (e + e.T)
    before = np.linalg.norm(a - x0 @ x0) / np.linalg.norm(a)
    after = np.linalg.norm(a - x1 @ x1) / np.linalg.norm(a)
    assert after < gain * before, (before, after)
