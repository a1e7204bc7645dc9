"""CPU tests: the oracle restatement pinned against the reference's own
outputs (tests/golden, produced by the reference's compiled CPU code)."""
import os

import numpy as np
import pytest

import oracle as O


@pytest.mark.parametrize("fmt", range(8))
def test_codec_restatement_matches_reference_vectors(golden_codecs, fmt):
    x = golden_codecs["x"]
    v, s = O.encode(fmt, x)
    np.testing.assert_array_equal(v, golden_codecs[f"values_{fmt}"])
    if golden_codecs[f"scales_{fmt}"].size:
        np.testing.assert_array_equal(s, golden_codecs[f"scales_{fmt}"])
    d = O.decode(fmt, golden_codecs[f"values_{fmt}"],
                 golden_codecs[f"scales_{fmt}"] if golden_codecs[f"scales_{fmt}"].size else None,
                 x.size)
    np.testing.assert_array_equal(d.view(np.uint32), golden_codecs[f"decoded_bits_{fmt}"])


def test_reference_known_answers():
    """checkLowPrecisionCodecs (src/storage_codecs.cpp:200-247)."""
    e4m3 = lambda v: O.encode(2, np.array([v], np.float32))[0][0]
    assert e4m3(448.0) == 0x7E
    assert np.isnan(O.decode(2, np.array([e4m3(np.nan)], np.uint8), None, 1)[0])
    assert O.encode(3, np.array([np.inf], np.float32))[0][0] == 0x7C
    assert e4m3(1.0625) == 0x38 and e4m3(1.1875) == 0x3A
    x = np.zeros(33, np.float32); x[0] = 6.1
    v, s = O.encode(7, x)
    assert list(s) == [127, 127] and (v[0] & 0xF) == 0x7
    x = np.zeros(33, np.float32); x[0] = 512.0
    v, s = O.encode(4, x)
    assert list(s) == [128, 127]
    assert O.decode(4, v, s, 33)[0] == 512.0
    v, s = O.encode(5, np.ones(32, np.float32))
    assert s[0] == 112 and O.decode(5, v, s, 32)[0] == 1.0


def test_rowscale_format_definition():
    rng = np.random.default_rng(3)
    x = rng.standard_normal((8, 40)).astype(np.float32)
    x[3] = 0.0
    v, s = O.encode(8, x.reshape(-1), row_length=40)
    scales = s.view(np.float32)
    ref_scale = np.where(np.abs(x).max(1) == 0, 1.0, np.abs(x).max(1) / np.float32(448)).astype(np.float32)
    np.testing.assert_array_equal(scales, ref_scale)
    codes = np.array([O.encode(2, np.array([xi / sc], np.float32))[0][0]
                      for xi, sc in zip(x.reshape(-1), np.repeat(scales, 40))], np.uint8)
    np.testing.assert_array_equal(v, codes)


def _reference_schedule(order):
    """makeJacobiSchedule (src/metal_solver.cpp:50-79), restated step by step."""
    m = order + order % 2
    participants = list(range(m))
    rounds = []
    for _ in range(m - 1):
        rounds.append([(min(participants[k], participants[m - 1 - k]),
                        max(participants[k], participants[m - 1 - k])) for k in range(m // 2)])
        participants = [participants[0], participants[-1]] + participants[1:-1]
    return rounds


@pytest.mark.parametrize("order", [2, 3, 4, 7, 16, 33])
def test_round_robin_closed_form_matches_schedule(order):
    sched = _reference_schedule(order)
    for r, pairs in enumerate(sched):
        assert [O.jacobi_pair(order, r, k) for k in range(len(pairs))] == pairs
    m = order + order % 2
    seen = {p for pairs in sched for p in pairs}
    assert len(seen) == m * (m - 1) // 2  # every pair exactly once per sweep


@pytest.mark.parametrize("n", [2, 5, 16, 33])
def test_oracle_jacobi_against_fp64_eigh(n):
    a = O.spd_loguniform(n, 1e3, seed=n)
    w, v, sweeps, off = O.jacobi(a, tol=1e-7, max_sweeps=20)
    assert off <= 1e-7 and sweeps <= 12
    ref = np.linalg.eigvalsh(a)
    np.testing.assert_allclose(np.sort(w), ref, rtol=0, atol=1e-6 * np.abs(ref).max())
    np.testing.assert_allclose(v.T.astype(np.float64) @ v, np.eye(n), atol=2e-6)


@pytest.mark.parametrize("key", ["n16", "n64", "n96"])
def test_generators_and_fp64_oracle_match_reference(golden_numerics, key):
    n = int(key[1:])
    a_ref = golden_numerics[f"{key}_a"].reshape(n, n, order="F")
    cond = float(golden_numerics[f"{key}_cond"][0])
    # FP64 restatements: agreement to a few ulps of the matrix scale
    np.testing.assert_allclose(O.controlled(n, cond), a_ref, rtol=0,
                               atol=1e-13 * np.abs(a_ref).max())
    root = O.reference_root(a_ref)
    root_ref = golden_numerics[f"{key}_root"].reshape(n, n, order="F")
    np.testing.assert_allclose(root, root_ref, rtol=0, atol=1e-12 * np.abs(root_ref).max())


@pytest.mark.parametrize("key", ["n16", "n64", "n96"])
def test_plain_method_port_matches_reference(golden_numerics, key):
    """runAccelerateCase: same iteration count, residuals <= 1e-12."""
    n = int(key[1:])
    a = golden_numerics[f"{key}_a"].reshape(n, n, order="F")
    summary = golden_numerics[f"{key}_summary"]
    root, hist = O.plain_method(a, 12, 1e-12)
    assert len(hist) - 1 == int(summary[2])
    assert hist[-1] <= 1e-12 and summary[0] <= 1e-12
    ref_hist = golden_numerics[f"{key}_history"][0::2]
    # first residual: FP32 eigensolver, LAPACK-dependent bits; same order
    assert 0.1 < hist[0] / ref_hist[0] < 10
    assert O.relative_error(root, O.reference_root(a)) < 1e-13


def test_ff_residual_matches_fp64():
    rng = np.random.default_rng(5)
    a = O.spd_loguniform(24, 1e2, 7).astype(np.float32)
    x = O.reference_root(a.astype(np.float64)).astype(np.float32)
    rel, r = O.ff_residual(a, x)
    r64 = a.astype(np.float64) - x.astype(np.float64) @ x.astype(np.float64)
    assert abs(rel - np.linalg.norm(r64) / np.linalg.norm(a.astype(np.float64))) < 1e-12


@pytest.mark.parametrize("test_set", [5, 6, 7])
@pytest.mark.parametrize("n", [32, 64])
def test_paper_sets_match_the_reference(test_set, n):
    """preparePaperMatrix (src/accelerate_backend.cpp:690-801) for the
    symmetric paper sets against the reference's own matrices
    (tests/golden/paper.npz).  The shift of V and VI comes from FP64
    extreme eigenvalues (numpy's LAPACK here, the reference's there), so the
    diagonals agree to rounding of that eigenvalue."""
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "paper.npz"))
    ref = g[f"set{test_set}_n{n}"].reshape(n, n, order="F")
    ref_shift, ref_cond = g[f"set{test_set}_n{n}_shift_condition"]
    a, shift, cond, seed = O.paper_matrix(test_set, n)
    off = ~np.eye(n, dtype=bool)
    assert np.array_equal(a[off], ref[off])             # the generator, bit for bit
    np.testing.assert_allclose(np.diag(a), np.diag(ref), rtol=1e-13, atol=0)
    assert abs(shift - ref_shift) <= 1e-12 * max(1.0, ref_shift)
    assert abs(cond - ref_cond) <= 1e-6 * ref_cond
    if test_set != 7:
        assert seed == (0x243F6A8885A308D3 ^ (0x9E3779B97F4A7C15 * test_set)) & (2**64 - 1)
