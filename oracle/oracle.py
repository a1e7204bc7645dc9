"""CPU oracle for the SPD square-root hot path — TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module, and only as the checker (or as the timed CPU baseline).  The
product (libmsq_cuda.so and its Python host layer) never imports it.

Parts
  * libmsq_oracle.so (msq_oracle.c, built by build_oracle()): the reference
    host codecs restated with their linear nearest-code scan, the
    parallel-order Jacobi and the float-float residual.
  * numpy restatements of the reference's FP64 oracle and definitions
    (src/numerics.cpp, src/accelerate_backend.cpp:555-607) and of its CPU
    plain method runAccelerateCase (src/accelerate_backend.cpp:803-1091).
  * seeded generators for the workload families (Gaussian-QR, Wishart,
    clustered, power-law) and the reference's controlled family
    (makeSpdMatrix, src/numerics.cpp:141-195).
  * ref(): the reference's own compiled CPU code (oracle/_ref/libmsq_ref.so,
    built from the reference sources where they exist), used to pin the
    restatements; absent where the reference tree is absent.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(HERE, "libmsq_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libmsq_ref.so")

_P = ctypes.c_void_p


def build_oracle() -> str:
    src = os.path.join(HERE, "msq_oracle.c")
    if (not os.path.exists(ORACLE_LIB) or
            os.path.getmtime(ORACLE_LIB) < os.path.getmtime(src)):
        subprocess.run(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off",
                        src, "-o", ORACLE_LIB, "-lm"], check=True)
    return ORACLE_LIB


_ORACLE = None


def olib() -> ctypes.CDLL:
    global _ORACLE
    if _ORACLE is None:
        build_oracle()
        lib = ctypes.CDLL(ORACLE_LIB)
        lib.msqo_encode.argtypes = [ctypes.c_int, _P, ctypes.c_size_t, ctypes.c_size_t, _P, _P]
        lib.msqo_decode.argtypes = [ctypes.c_int, _P, _P, ctypes.c_size_t, ctypes.c_size_t, _P]
        lib.msqo_storage_bytes.argtypes = [ctypes.c_int, ctypes.c_size_t]
        lib.msqo_storage_bytes.restype = ctypes.c_size_t
        lib.msqo_jacobi.argtypes = [_P, _P, _P, ctypes.c_uint, ctypes.c_double, ctypes.c_int,
                                    ctypes.POINTER(ctypes.c_double)]
        lib.msqo_jacobi_blocked.argtypes = [_P, _P, _P, _P, ctypes.c_uint, ctypes.c_double,
                                            ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
        lib.msqo_jacobi_blocked_order.argtypes = [_P, _P, _P, _P, ctypes.c_uint, ctypes.c_double,
                                                  ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                                  ctypes.c_int]
        lib.msqo_two_level_rounds.argtypes = [ctypes.c_uint]
        lib.msqo_two_level_schedule.argtypes = [ctypes.c_uint, _P]
        lib.msqo_jacobi_pair.argtypes = [ctypes.c_uint, ctypes.c_uint, ctypes.c_uint,
                                         ctypes.POINTER(ctypes.c_uint), ctypes.POINTER(ctypes.c_uint)]
        lib.msqo_ff_residual.argtypes = [_P, _P, _P, ctypes.c_uint, _P]
        lib.msqo_ff_residual.restype = ctypes.c_double
        lib.msqo_stochastic_hash.argtypes = [ctypes.c_uint32] * 3
        lib.msqo_stochastic_hash.restype = ctypes.c_uint32
        lib.msqo_encode_stochastic.argtypes = [ctypes.c_int, _P, ctypes.c_size_t, ctypes.c_size_t,
                                               ctypes.c_uint32, ctypes.c_uint32, _P, _P]
        lib.msqo_spectrum_encode.argtypes = [ctypes.c_int, _P, ctypes.c_size_t, ctypes.c_int,
                                             ctypes.c_uint32, ctypes.c_uint32, _P, _P]
        lib.msqo_spectrum_decode.argtypes = [ctypes.c_int, _P, _P, ctypes.c_size_t, _P]
        lib.msqo_native_correction.argtypes = [ctypes.c_int, _P, _P, _P, _P, ctypes.c_uint, _P]
        lib.msqo_paper_matrix.argtypes = [ctypes.c_int, ctypes.c_uint, _P,
                                          ctypes.POINTER(ctypes.c_uint64)]
        _ORACLE = lib
    return _ORACLE


def scale_bytes(fmt: int, elements: int, row_length: int = 0) -> int:
    if fmt in (4, 5, 7):
        return (elements + 31) // 32
    if fmt == 8:
        return (elements // row_length) * 4
    return 0


def encode(fmt: int, x: np.ndarray, row_length: int = 0):
    """copyToStorage restated: returns (values uint8, scales uint8 | None)."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    n = x.size
    values = np.zeros(max(olib().msqo_storage_bytes(fmt, n), 1), dtype=np.uint8)
    sb = scale_bytes(fmt, n, row_length)
    scales = np.zeros(max(sb, 1), dtype=np.uint8)
    rc = olib().msqo_encode(fmt, x.ctypes.data, n, row_length, values.ctypes.data,
                            scales.ctypes.data)
    if rc:
        raise ValueError("oracle encode failed")
    return values[:olib().msqo_storage_bytes(fmt, n)], (scales[:sb] if sb else None)


def decode(fmt: int, values: np.ndarray, scales, elements: int, row_length: int = 0):
    """storageValueAt restated for every index."""
    out = np.zeros(elements, dtype=np.float32)
    values = np.ascontiguousarray(values, dtype=np.uint8)
    sc = np.ascontiguousarray(scales, dtype=np.uint8) if scales is not None else np.zeros(1, np.uint8)
    rc = olib().msqo_decode(fmt, values.ctypes.data, sc.ctypes.data, elements, row_length,
                            out.ctypes.data)
    if rc:
        raise ValueError("oracle decode failed")
    return out


def encode_stochastic(fmt: int, x: np.ndarray, seed: int, stream: int, row_length: int = 0):
    """The device quantizers' stochastic rounding restated: (values, scales | None)."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    n = x.size
    values = np.zeros(max(olib().msqo_storage_bytes(fmt, n), 1), dtype=np.uint8)
    sb = scale_bytes(fmt, n, row_length)
    scales = np.zeros(max(sb, 1), dtype=np.uint8)
    rc = olib().msqo_encode_stochastic(fmt, x.ctypes.data, n, row_length, seed & 0xffffffff,
                                       stream & 0xffffffff, values.ctypes.data, scales.ctypes.data)
    if rc:
        raise ValueError("oracle stochastic encode failed")
    return values[:olib().msqo_storage_bytes(fmt, n)], (scales[:sb] if sb else None)


def spectrum_metadata_floats(elements: int) -> int:
    """Two floats (min, span of log2 s) per block of 8 root eigenvalues."""
    return 2 * ((elements + 7) // 8)


def spectrum_encode(fmt: int, s: np.ndarray, stochastic: bool = False, seed: int = 0,
                    stream: int = 0):
    """Log-spectrum storage (device form): returns (codes, metadata)."""
    s = np.ascontiguousarray(s, dtype=np.float32)
    n = s.size
    values = np.zeros(max(olib().msqo_storage_bytes(fmt, n), 1), dtype=np.uint8)
    meta = np.zeros(max(spectrum_metadata_floats(n), 1), dtype=np.float32)
    rc = olib().msqo_spectrum_encode(fmt, s.ctypes.data, n, int(stochastic), seed & 0xffffffff,
                                     stream & 0xffffffff, values.ctypes.data, meta.ctypes.data)
    if rc:
        raise ValueError("oracle spectrum encode failed (format or non-positive input)")
    return values[:olib().msqo_storage_bytes(fmt, n)], meta[:spectrum_metadata_floats(n)]


def spectrum_decode(fmt: int, values: np.ndarray, meta: np.ndarray, elements: int):
    out = np.zeros(elements, dtype=np.float32)
    values = np.ascontiguousarray(values, dtype=np.uint8)
    meta = np.ascontiguousarray(meta, dtype=np.float32)
    if olib().msqo_spectrum_decode(fmt, values.ctypes.data, meta.ctypes.data, elements,
                                   out.ctypes.data):
        raise ValueError("oracle spectrum decode failed")
    return out


def native_correction(fmt: int, v: np.ndarray, vt: np.ndarray, s: np.ndarray, r: np.ndarray):
    """One native-quantized correction E (refineNativeStaged restated); all
    matrices n x n FP32 column-major, s the n root eigenvalues."""
    n = v.shape[0]
    f = lambda m: np.asfortranarray(m, dtype=np.float32)
    V, VT, R = f(v), f(vt), f(r)
    S = np.ascontiguousarray(s, dtype=np.float32)
    E = np.zeros((n, n), dtype=np.float32, order="F")
    if olib().msqo_native_correction(fmt, V.ctypes.data, VT.ctypes.data, S.ctypes.data,
                                     R.ctypes.data, n, E.ctypes.data):
        raise ValueError("oracle native correction failed")
    return E


PAPER_ORDERS = {5: 4096, 6: 4096, 7: 1024}  # paperTestSetOrder (src/configuration.cpp:255-271)


def paper_matrix(test_set: int, n: int):
    """preparePaperMatrix (src/accelerate_backend.cpp:690-801) for the
    symmetric sets V, VI, VII: (matrix, diagonal_shift, condition, rng_seed).
    Sets V and VI are shifted so that the smallest eigenvalue is
    max(1, 0.01 ||A||_inf) (FP64 eigenvalues, numpy's LAPACK)."""
    a = np.zeros((n, n), dtype=np.float64, order="F")
    seed = ctypes.c_uint64(0)
    if olib().msqo_paper_matrix(test_set, n, a.ctypes.data, ctypes.byref(seed)):
        raise ValueError("paper sets V, VI and VII only")
    lam = np.linalg.eigvalsh(a)
    if test_set == 7:
        return a, 1e-6, float(lam[-1] / lam[0]), 0
    separation = max(1.0, 0.01 * np.abs(a).sum(axis=1).max())
    shift = max(0.0, separation - lam[0])
    a[np.diag_indices(n)] += shift
    return a, shift, float((lam[-1] + shift) / (lam[0] + shift)), int(seed.value)


def jacobi_pair(order: int, rnd: int, pair: int) -> tuple[int, int]:
    p, q = ctypes.c_uint(), ctypes.c_uint()
    olib().msqo_jacobi_pair(order, rnd, pair, ctypes.byref(p), ctypes.byref(q))
    return p.value, q.value


def jacobi(a: np.ndarray, tol: float = 1e-7, max_sweeps: int = 15):
    """Parallel-order two-sided Jacobi (FP32 storage, FP64 angles)."""
    n = a.shape[0]
    A = np.asfortranarray(a, dtype=np.float32).copy(order="F")
    V = np.zeros((n, n), dtype=np.float32, order="F")
    w = np.zeros(n, dtype=np.float32)
    ratio = ctypes.c_double()
    sweeps = olib().msqo_jacobi(A.ctypes.data, V.ctypes.data, w.ctypes.data, n, tol, max_sweeps,
                                ctypes.byref(ratio))
    return w, V, sweeps, ratio.value


def two_level_schedule(blocks: int) -> np.ndarray:
    """The two-level pair table for `blocks` 4-index blocks: (rounds, blocks/2,
    2) int32 pairs (I, J), J = -1 - J for an identity pair."""
    rounds = olib().msqo_two_level_rounds(blocks)
    out = np.zeros(rounds * blocks, dtype=np.int32)
    olib().msqo_two_level_schedule(blocks, out.ctypes.data)
    return out.reshape(rounds, blocks // 2, 2)


def jacobi_blocked(a: np.ndarray, tol: float = 1e-7, max_sweeps: int = 15, with_matrix=False,
                   two_level=False):
    """The same rotations in the blocked order the CUDA eigensolver uses, with
    the same FP32 roundings: after the same number of sweeps the CUDA kernels
    return the same eigenvalues, eigenvectors and rotated matrix bit for bit.
    two_level: the two-level pairing the solver uses for orders 257..512 in
    its blocked and tensor-core eigenvector modes.
    Returns (w, V, sweeps, off_ratio[, final matrix])."""
    n = a.shape[0]
    A = np.asfortranarray(a, dtype=np.float32)
    out = np.zeros((n, n), dtype=np.float32, order="F")
    V = np.zeros((n, n), dtype=np.float32, order="F")
    w = np.zeros(n, dtype=np.float32)
    ratio = ctypes.c_double()
    sweeps = olib().msqo_jacobi_blocked_order(A.ctypes.data, out.ctypes.data, V.ctypes.data,
                                              w.ctypes.data, n, tol, max_sweeps,
                                              ctypes.byref(ratio), int(bool(two_level)))
    if with_matrix:
        return w, V, sweeps, ratio.value, out
    return w, V, sweeps, ratio.value


def ff_residual(a: np.ndarray, x_hi: np.ndarray, x_lo=None):
    """float-float residual R = A - X X; returns (relative norm, R)."""
    n = a.shape[0]
    A = np.asfortranarray(a, dtype=np.float32)
    H = np.asfortranarray(x_hi, dtype=np.float32)
    L = np.asfortranarray(x_lo, dtype=np.float32) if x_lo is not None else None
    R = np.zeros((n, n), dtype=np.float32, order="F")
    rel = olib().msqo_ff_residual(A.ctypes.data, H.ctypes.data,
                                  L.ctypes.data if L is not None else None, n, R.ctypes.data)
    return rel, R


# ---------------------------------------------------------------- FP64 oracle

def reference_root(a: np.ndarray) -> np.ndarray:
    """symmetricReferenceRoot (src/accelerate_backend.cpp:594-607): FP64
    eigendecomposition, V diag(sqrt(lambda)) V^T, symmetrised."""
    a = np.asarray(a, dtype=np.float64)
    w, v = np.linalg.eigh(a)
    if not np.all(w > 0):
        raise ValueError("The FP64 reference has a nonpositive eigenvalue.")
    root = (v * np.sqrt(w)) @ v.T
    return 0.5 * (root + root.T)


def relative_residual(a: np.ndarray, x: np.ndarray) -> float:
    """relativeResidual (src/numerics.cpp:213-228): ||A - X X^T||_F/||A||_F."""
    a = np.asarray(a, dtype=np.float64)
    x = np.asarray(x, dtype=np.float64)
    return float(np.linalg.norm(a - x @ x.T) / np.linalg.norm(a))


def relative_error(x: np.ndarray, ref: np.ndarray) -> float:
    """relativeError (src/numerics.cpp:230-240)."""
    x = np.asarray(x, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    return float(np.linalg.norm(x - ref) / np.linalg.norm(ref))


# ---------------------------------------------------------------- generators

def _orthogonal(n: int, rng: np.random.Generator) -> np.ndarray:
    g = rng.standard_normal((n, n))
    q, r = np.linalg.qr(g)
    return q * np.sign(np.diag(r))


def spd_from_spectrum(lam: np.ndarray, rng: np.random.Generator) -> np.ndarray:
    q = _orthogonal(lam.size, rng)
    a = (q * lam) @ q.T
    return 0.5 * (a + a.T)


def loguniform_spectrum(n: int, cond: float, rng: np.random.Generator) -> np.ndarray:
    lam = np.exp(rng.uniform(np.log(1.0 / cond), 0.0, n))
    if n >= 2:
        lam[0], lam[-1] = 1.0 / cond, 1.0
    return lam


def spd_loguniform(n: int, cond: float, seed: int) -> np.ndarray:
    """A = Q diag(lambda) Q^T, Q from QR of a seeded N(0,1) matrix (sign-fixed),
    lambda log-uniform on [1/cond, 1]."""
    rng = np.random.default_rng(seed)
    return spd_from_spectrum(loguniform_spectrum(n, cond, rng), rng)


def spd_clustered(n: int, cond: float, seed: int) -> np.ndarray:
    """90% of lambda in [0.9, 1.1], 10% log-uniform down to 1/cond."""
    rng = np.random.default_rng(seed)
    k = max(1, n // 10)
    lam = np.concatenate([rng.uniform(0.9, 1.1, n - k),
                          np.exp(rng.uniform(np.log(1.0 / cond), np.log(0.9), k))])
    lam[-1] = 1.0 / cond
    return spd_from_spectrum(lam, rng)


def spd_power_law(n: int, seed: int) -> np.ndarray:
    """lambda_i proportional to i^-2."""
    rng = np.random.default_rng(seed)
    lam = 1.0 / np.arange(1, n + 1, dtype=np.float64) ** 2
    return spd_from_spectrum(lam, rng)


def wishart(n: int, seed: int, ratio: int = 2, shift: float = 1e-6) -> np.ndarray:
    """A = X^T X / m + shift I, X ~ N(0,1) of shape m x n, m = ratio * n."""
    rng = np.random.default_rng(seed)
    m = ratio * n
    x = rng.standard_normal((m, n))
    a = x.T @ x / m + shift * np.eye(n)
    return 0.5 * (a + a.T)


def wishart_orders(count: int, lo: int, hi: int, seed: int) -> np.ndarray:
    """n log-uniform integer in [lo, hi]."""
    rng = np.random.default_rng(seed)
    n = np.floor(np.exp(rng.uniform(np.log(lo), np.log(hi + 1), count))).astype(np.int32)
    return np.clip(n, lo, hi)


def controlled(n: int, cond: float) -> np.ndarray:
    """makeSpdMatrix (src/numerics.cpp:141-195): deterministic sin/cos basis,
    Gram-Schmidt, geometric eigenvalues cond^(k/(n-1))."""
    rows = np.arange(n, dtype=np.float64)[:, None]
    cols = np.arange(n, dtype=np.float64)[None, :]
    v = np.sin(0.173 * (rows + 1) * (cols + 2)) + np.cos(0.117 * (rows + 3) * (cols + 1))
    for c in range(n):
        for p in range(c):
            v[:, c] -= (v[:, p] @ v[:, c]) * v[:, p]
        v[:, c] /= np.linalg.norm(v[:, c])
    lam = np.exp(np.log(cond) * np.arange(n) / max(1, n - 1))
    return (v * lam) @ v.T


# ---------------------------------------- stage-3 precision plans (restated)

# FactorFormat (3_spectral/spectral.hpp) -> codec id of encode/decode; FP16
# is numpy's IEEE binary16 (round to nearest even).
SPECTRAL_FORMATS = {"fp32": None, "fp16": "fp16", "bf16": 1, "fp8_e4m3": 2, "fp8_e5m2": 3,
                    "mxfp8_e4m3": 4, "mxfp4_e2m1": 7}
# precision_plans() (3_spectral/spectral.cpp:769-786)
SPECTRAL_PLANS = [("fp32_baseline", "fp32", "fp32"), ("spectrum_fp16", "fp32", "fp16"),
                  ("spectrum_bf16", "fp32", "bf16"), ("spectrum_e4m3", "fp32", "fp8_e4m3"),
                  ("spectrum_e5m2", "fp32", "fp8_e5m2"), ("spectrum_mxfp8", "fp32", "mxfp8_e4m3"),
                  ("spectrum_mxfp4", "fp32", "mxfp4_e2m1"), ("basis_fp16", "fp16", "fp32"),
                  ("basis_bf16", "bf16", "fp32"), ("basis_e4m3", "fp8_e4m3", "fp32"),
                  ("basis_e5m2", "fp8_e5m2", "fp32"), ("basis_mxfp8", "mxfp8_e4m3", "fp32"),
                  ("basis_mxfp4", "mxfp4_e2m1", "fp32"), ("fp16_mxfp8", "fp16", "mxfp8_e4m3"),
                  ("bf16_mxfp8", "bf16", "mxfp8_e4m3"), ("e4m3_mxfp4", "fp8_e4m3", "mxfp4_e2m1")]


def _spectral_quantize(fmt: str, x: np.ndarray) -> np.ndarray:
    """Nearest quantize + decode of a flat FP32 array (column-major order)."""
    x = np.ascontiguousarray(x, np.float32).reshape(-1)
    if fmt == "fp32":
        return x.copy()
    if fmt == "fp16":
        return x.astype(np.float16).astype(np.float32)
    codec = SPECTRAL_FORMATS[fmt]
    vals, scl = encode(codec, x)
    return decode(codec, vals, scl, x.size)


def spectral_plan(a: np.ndarray, basis_fmt: str, spectrum_fmt: str, condition: float,
                  max_corrections: int = 30, tol: float = 1e-12, reference=None) -> dict:
    """run_spectral (3_spectral/spectral.cpp:787-1385) restated with FP64
    products on the same operands: FP32 eigenbasis (the blocked Jacobi the
    CUDA solver runs, bit for bit), root spectrum sqrt(lambda); basis and
    spectrum quantized; Vinv = Q(V)^T, or for an FP16 basis the FP16 image of
    the FP32 basis's inverse (invert_basis :600-637, rejected at 1-norm
    condition >= 1e4); X0 = (Q(V) diag(Q(s))) Vinv; corrections
    E = V ((Vinv R V) o H) Vinv, H_ij = 1/(s_i + s_j), with every operand
    re-quantized to the basis format while a low-bit basis (E4M3, E5M2,
    MXFP8, MXFP4) of a matrix below condition 1000 is above residual 1e-3
    and has not stalled twice (no 2x drop); stop at tol, the budget, or
    divergence (residual >= max(1, 1e4 initial))."""
    n = a.shape[0]
    a64 = np.asarray(a, np.float64)
    a32 = a64.astype(np.float32)
    w, v, _, _ = jacobi_blocked(a32.astype(np.float64), 1e-7, 20)
    if not np.all(w > 0):
        raise ValueError("The FP32 factor has an invalid spectrum.")
    s = np.sqrt(w.astype(np.float32))
    out = {"accepted": False, "reason": "", "basis_condition": float("nan")}
    fp16_basis = basis_fmt == "fp16"
    low = basis_fmt in ("fp8_e4m3", "fp8_e5m2", "mxfp8_e4m3", "mxfp4_e2m1") and condition < 1000.0
    v32 = np.asarray(v, np.float32)
    inverse = None
    if fp16_basis:
        vd = v32.astype(np.float64)
        inverse = np.linalg.inv(vd)
        cond = np.abs(vd).sum(0).max() * np.abs(inverse).sum(0).max()
        out["basis_condition"] = float(cond)
        if not cond < 1e4:
            out["reason"] = "ill_conditioned_basis"
            return out
    else:
        out["basis_condition"] = 1.0
    vq = _spectral_quantize(basis_fmt, v32.reshape(-1, order="F")).reshape(n, n, order="F")
    sq = _spectral_quantize(spectrum_fmt, s)
    out["basis_error"] = float(np.linalg.norm(vq.astype(np.float64) - v32) / np.linalg.norm(v32.astype(np.float64)))
    out["spectrum_error"] = float(np.linalg.norm(sq.astype(np.float64) - s) / np.linalg.norm(s.astype(np.float64)))
    if not (np.all(sq > 0) and np.all(np.isfinite(sq))):
        out["reason"] = "invalid_spectrum"
        return out
    if fp16_basis:
        vinv = inverse.astype(np.float32).astype(np.float16).astype(np.float32)
        if not np.all(np.isfinite(vinv)):
            out["reason"] = "ill_conditioned_basis"
            return out
    else:
        vinv = vq.T.copy()
    out["accepted"] = True

    def q(x):  # an operand re-encoded to the basis format (flat column-major)
        return _spectral_quantize(basis_fmt, np.asarray(x, np.float32).reshape(-1, order="F")
                                  ).reshape(n, n, order="F").astype(np.float64)

    vs = (vq * sq[None, :]).astype(np.float32)
    vs_op = q(vs) if low else (vs.astype(np.float16).astype(np.float64) if fp16_basis
                               else vs.astype(np.float64))
    vinv_op = q(vinv) if low else vinv.astype(np.float64)
    V, Vinv = vq.astype(np.float64), vinv.astype(np.float64)
    H = 1.0 / (sq.astype(np.float64)[:, None] + sq.astype(np.float64)[None, :])
    x = vs_op @ vinv_op
    norm_a = np.linalg.norm(a64)

    def residual(x):
        r = a64 - x @ x
        return r, float(np.linalg.norm(r) / norm_a)

    r, measured = residual(x)
    history = [measured]
    limit = max(1.0, 1e4 * measured)
    low_on, low_prev, stalls, low_count = True, measured, 0, 0
    it = 0
    while measured > tol and it < max_corrections and measured < limit:
        use_low = low and low_on and measured > 1e-3
        if use_low:
            wk = q(vinv_op @ q(r))
            c = q((wk @ V) * H)
            e = q(V @ c) @ vinv_op
            low_count += 1
        else:
            c = ((Vinv @ r) @ V) * H
            e = (V @ c) @ Vinv
        x = x + e
        r, measured = residual(x)
        history.append(measured)
        it += 1
        if low and low_on and measured > tol:
            stalls = stalls + 1 if measured > low_prev * 0.5 else 0
            low_prev = measured
            low_on = stalls < 2
    out.update(iterations=it, residuals=history, final_residual=history[-1],
               low_product_corrections=low_count, converged=history[-1] <= tol)
    out["reason"] = ("converged" if history[-1] <= tol else "nonfinite_residual"
                     if not np.isfinite(history[-1]) else "divergent" if history[-1] >= limit
                     else "correction_limit")
    if reference is not None:
        out["final_error"] = relative_error(x, reference)
    return out


# ------------------------------------------------- CPU plain method (port)

def plain_method(a: np.ndarray, max_corrections: int = 12, tol: float = 1e-12):
    """runAccelerateCase, symmetric branch (src/accelerate_backend.cpp:803-1091):
    FP32 ssyevd -> X0 = (V diag s) V^T in FP32 -> FP64 residual -> frozen-basis
    corrections C = (V^T R V) o 1/(s_i+s_j), E = V C V^T until residual <= tol.
    Returns (root FP64, residual history)."""
    import scipy.linalg as sla
    a = np.asarray(a, dtype=np.float64)
    n = a.shape[0]
    w, v = sla.eigh(a.astype(np.float32), driver="evd", overwrite_a=False, check_finite=False)
    if not np.all(w > 0):
        raise ValueError("Accelerate ssyevd returned a nonpositive eigenvalue.")
    s = np.sqrt(w).astype(np.float32)
    v = v.astype(np.float32)
    x0 = (v * s) @ v.T
    root = x0.astype(np.float64)
    root = 0.5 * (root + root.T)
    denom = (s[:, None] + s[None, :]).astype(np.float32)
    anorm = np.linalg.norm(a)

    def residual(x):
        r = a - x @ x.T
        return r, float(np.linalg.norm(r) / anorm)

    r, res = residual(root)
    history = [res]
    it = 0
    while res > tol and it < max_corrections and np.isfinite(res):
        r32 = r.astype(np.float32)
        c = v.T @ (r32 @ v)
        c = (0.5 * (c + c.T)) / denom
        e = (v @ c) @ v.T
        root = root + e.astype(np.float64)
        root = 0.5 * (root + root.T)
        it += 1
        r, res = residual(root)
        history.append(res)
    return root, history


# --------------------------------------------------- plan-selector MLP

MLP_SHAPES = ((64, 16), (64, 64), (8, 64))


def _mlp_unpack(params: np.ndarray):
    """FP32 master parameters -> BF16-rounded FP64 (W1, b1, W2, b2, W3, b3),
    the layout of msq_mlp.cu.  BF16 rounding is the reference codec's RNE."""
    v, _ = encode(1, np.asarray(params, np.float32))
    p = decode(1, v, None, params.size).astype(np.float64)
    out, off = [], 0
    for rows, cols in MLP_SHAPES:
        out.append(p[off:off + rows * cols].reshape(rows, cols))
        off += rows * cols
        out.append(p[off:off + rows])
        off += rows
    return out


def mlp_forward(params: np.ndarray, x: np.ndarray):
    W1, b1, W2, b2, W3, b3 = _mlp_unpack(params)
    h1 = np.maximum(x @ W1.T + b1, 0.0)
    h2 = np.maximum(h1 @ W2.T + b2, 0.0)
    return h2 @ W3.T + b3, (h1, h2)


def mlp_loss_and_grad(params: np.ndarray, x: np.ndarray, y: np.ndarray):
    """Mean sigmoid cross-entropy over rows and outputs and its gradient with
    respect to the FP32 masters (BF16 rounding as a straight-through
    identity), in FP64."""
    W1, b1, W2, b2, W3, b3 = _mlp_unpack(params)
    x = np.asarray(x, np.float64)
    z, (h1, h2) = mlp_forward(params, x)
    scale = 1.0 / z.size
    loss = np.sum(np.maximum(z, 0) + np.log1p(np.exp(-np.abs(z))) - y * z) * scale
    dz = (1.0 / (1.0 + np.exp(-z)) - y) * scale
    gW3, gb3 = dz.T @ h2, dz.sum(0)
    dh2 = (dz @ W3) * (h2 > 0)
    gW2, gb2 = dh2.T @ h1, dh2.sum(0)
    dh1 = (dh2 @ W2) * (h1 > 0)
    gW1, gb1 = dh1.T @ x, dh1.sum(0)
    grad = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss, grad


# ------------------------------------------- the reference's own CPU code

_REF = None


def ref_available() -> bool:
    return os.path.exists(REF_LIB)


def ref() -> ctypes.CDLL:
    """The reference's CPU path compiled from its own sources (x86 build
    container only)."""
    global _REF
    if _REF is None:
        lib = ctypes.CDLL(REF_LIB)
        lib.ref_last_error.restype = ctypes.c_char_p
        lib.ref_storage_bytes.argtypes = [ctypes.c_int, ctypes.c_size_t]
        lib.ref_storage_bytes.restype = ctypes.c_size_t
        lib.ref_scale_bytes.argtypes = [ctypes.c_int, ctypes.c_size_t]
        lib.ref_scale_bytes.restype = ctypes.c_size_t
        lib.ref_encode.argtypes = [ctypes.c_int, _P, ctypes.c_size_t, _P, _P]
        lib.ref_decode.argtypes = [ctypes.c_int, _P, _P, ctypes.c_size_t, _P]
        lib.ref_make_spd.argtypes = [ctypes.c_size_t, ctypes.c_double, _P]
        lib.ref_reference_root.argtypes = [_P, ctypes.c_size_t, _P]
        lib.ref_relative_residual.argtypes = [_P, _P, ctypes.c_size_t]
        lib.ref_relative_residual.restype = ctypes.c_double
        lib.ref_relative_error.argtypes = [_P, _P, ctypes.c_size_t]
        lib.ref_relative_error.restype = ctypes.c_double
        lib.ref_run_accelerate.argtypes = [_P, ctypes.c_size_t, ctypes.c_double, ctypes.c_size_t,
                                           ctypes.c_double, _P, _P, ctypes.c_size_t]
        lib.ref_spectrum_encode.argtypes = [ctypes.c_int, _P, ctypes.c_size_t, _P, _P]
        lib.ref_spectrum_decode.argtypes = [ctypes.c_int, _P, _P, ctypes.c_size_t, _P]
        _REF = lib
    return _REF


def ref_encode(fmt: int, x: np.ndarray):
    lib = ref()
    x = np.ascontiguousarray(x, dtype=np.float32)
    n = x.size
    values = np.zeros(max(lib.ref_storage_bytes(fmt, n), 1), dtype=np.uint8)
    sb = lib.ref_scale_bytes(fmt, n)
    scales = np.zeros(max(sb, 1), dtype=np.uint8)
    if lib.ref_encode(fmt, x.ctypes.data, n, values.ctypes.data, scales.ctypes.data if sb else None):
        raise ValueError(lib.ref_last_error().decode())
    return values[:lib.ref_storage_bytes(fmt, n)], (scales[:sb] if sb else None)


def ref_decode(fmt: int, values: np.ndarray, scales, elements: int):
    lib = ref()
    out = np.zeros(elements, dtype=np.float32)
    values = np.ascontiguousarray(values, dtype=np.uint8)
    sc = np.ascontiguousarray(scales, dtype=np.uint8) if scales is not None else None
    if lib.ref_decode(fmt, values.ctypes.data, sc.ctypes.data if sc is not None else None,
                      elements, out.ctypes.data):
        raise ValueError(lib.ref_last_error().decode())
    return out


def ref_spectrum_encode(fmt: int, s: np.ndarray):
    """copySpectrumToStorage of the reference (host form): (codes, metadata)."""
    lib = ref()
    s = np.ascontiguousarray(s, dtype=np.float32)
    n = s.size
    values = np.zeros(max(lib.ref_storage_bytes(fmt, n), 1), dtype=np.uint8)
    meta = np.zeros(max(spectrum_metadata_floats(n), 1), dtype=np.float32)
    if lib.ref_spectrum_encode(fmt, s.ctypes.data, n, values.ctypes.data, meta.ctypes.data):
        raise ValueError(lib.ref_last_error().decode())
    return values[:lib.ref_storage_bytes(fmt, n)], meta[:spectrum_metadata_floats(n)]


def ref_spectrum_decode(fmt: int, values: np.ndarray, meta: np.ndarray, elements: int):
    lib = ref()
    out = np.zeros(elements, dtype=np.float32)
    values = np.ascontiguousarray(values, dtype=np.uint8)
    meta = np.ascontiguousarray(meta, dtype=np.float32)
    if lib.ref_spectrum_decode(fmt, values.ctypes.data, meta.ctypes.data, elements,
                               out.ctypes.data):
        raise ValueError(lib.ref_last_error().decode())
    return out
