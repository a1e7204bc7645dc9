"""Generate tests/golden/*.npz from the reference's own CPU code.

Runs only where the reference sources are present: oracle/Makefile compiles
them (src/storage_codecs.cpp, src/numerics.cpp, src/accelerate_backend.cpp,
...) into oracle/_ref/libmsq_ref.so, and this script records their outputs:

  codecs.npz     inputs (specials, boundary values, the fixture rule of
                 tests/matrix_codec.cpp:39-78, N(0,1), Student-t(3), wide
                 sign*2^U(-30,30), midpoints of every code pair and their
                 float neighbours) with the reference's encoded values,
                 scale planes and decoded FP32 bits for codecs 0..7.
  numerics.npz   makeSpdMatrix(n, cond) outputs, symmetricReferenceRoot of
                 them, and runAccelerateCase (src/accelerate_backend.cpp:
                 803-1091) residual/forward-error histories.
  paper.npz      preparePaperMatrix (src/accelerate_backend.cpp:690-801)
                 for the symmetric paper sets V, VI, VII at orders 32 and 64:
                 the matrices, diagonal shifts and conditions.
  csv_headers.txt  writeSummaryHeader and writeIterationsHeader
                 (src/reporting.cpp:124-166, 305-327): the reference's CSV
                 schema, one header line each.
  spectrum.npz   copySpectrumToStorage / spectrumValueAt (src/storage_codecs.
                 cpp:387-460) codes, (min, span) metadata and decoded values
                 of the log-spectrum precisions (FP8-E4M3FN and FP4-E2M1
                 codes) for the roots of checkLogSpectrumStorage, the
                 spectrum of checkStochasticQuantization and log-uniform
                 spectra with equal-valued blocks and a ragged tail.

Usage: make -C oracle REF=<reference checkout> && python tests/golden/make_golden.py [csv | paper | spectrum]
(each option writes the files listed up to and including its own: csv_headers.txt,
then paper.npz, then spectrum.npz)
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
import oracle as O  # noqa: E402

F32 = np.float32


def fixture_matrix(order: int) -> np.ndarray:
    """The boundary fixture rule of tests/matrix_codec.cpp:39-78 (restated)."""
    values = np.array([0.0, -0.0, 0.125, 0.25, 0.375, 0.5, 0.625, 0.75, 0.875, 1.0,
                       1.00048828125, 1.00146484375, 1.0625, 1.1875, 1.25, 1.375, 1.75,
                       1.875, 2.0, 2.125, 2.5, 2.75, 3.0, 3.5, 4.0, 4.5, 5.0, 5.5, 6.0, 6.5,
                       7.0, 7.5], dtype=F32)
    src = np.zeros(order * order, dtype=F32)
    for col in range(1, order):
        for row in range(1, order):
            e = (row % 7) - 3 + 2 * (col // 32) + (col % 3) - 1
            v = np.ldexp(values[(13 * row + 7 * col) % 32], e).astype(F32)
            if (row + col) % 2:
                v = -v
            src[row + col * order] = v
    bounds = [-0.0, 2.0 ** -25, 3 * 2.0 ** -25, 2.0 ** -17, 3 * 2.0 ** -17, 2.0 ** -10,
              3 * 2.0 ** -10, 448.0, 464.0, -464.0, 57344.0, 61440.0, 65504.0, 65520.0]
    for i, b in enumerate(bounds):
        src[(i + 1) + (i + 2) * order] = F32(b)
    return src


def codec_inputs() -> np.ndarray:
    rng = np.random.default_rng(20261203)
    f = np.finfo(F32)
    specials = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, -np.nan, f.max, -f.max, f.tiny,
                         -f.tiny, 2.0 ** -149, -2.0 ** -149, 2.0 ** -133, 1.0, -1.0, 6.1, 512.0,
                         1.0625, 1.1875], dtype=F32)
    parts = [specials, fixture_matrix(96)]
    for fmt in (2, 3):
        v = O.decode(fmt, np.arange(256, dtype=np.uint8), None, 256).astype(np.float64)
        v = np.unique(np.abs(v[np.isfinite(v)]))
        mid = ((v[1:] + v[:-1]) / 2).astype(F32)
        parts += [mid, np.nextafter(mid, F32(np.inf)), np.nextafter(mid, F32(-np.inf)), -mid]
    v4 = np.array([0, 0.5, 1, 1.5, 2, 3, 4, 6], dtype=np.float64)
    mid = ((v4[1:] + v4[:-1]) / 2).astype(F32)
    parts += [mid, np.nextafter(mid, F32(np.inf)), np.nextafter(mid, F32(-np.inf)), -mid]
    parts += [rng.standard_normal(4096).astype(F32), rng.standard_t(3, 4096).astype(F32),
              (np.sign(rng.standard_normal(4096)) * 2.0 ** rng.uniform(-30, 30, 4096)).astype(F32)]
    x = np.concatenate(parts).astype(F32)
    # pad to a multiple of 32 plus a ragged tail of 7 (exercise partial blocks)
    pad = (-x.size) % 32 + 7
    return np.concatenate([x, rng.standard_normal(pad).astype(F32)])


def spectrum_inputs() -> dict:
    """Finite positive spectra: the roots checkLogSpectrumStorage uses
    (src/metal_checks.cpp:507-509), 1024 values of the spectrum
    checkStochasticQuantization builds (:425-431), and 2^U(-20, 20) values
    with two equal-valued blocks (span 0) and a ragged tail (1001 values)."""
    check = np.array([1.0, 1.5, 2.0, 3.0, 10.0, 31.622776, 100.0, 1000.0], dtype=F32)
    idx = np.arange(1024)
    pos = np.power((idx % 8) / F32(7.0), F32(1.3)).astype(F32)
    pattern = np.exp2(F32(-2.0) + F32(4.0) * pos).astype(F32)
    rng = np.random.default_rng(2024)
    wide = np.exp2(rng.uniform(-20.0, 20.0, 1001)).astype(F32)
    wide[8:16] = F32(3.0)
    wide[16:24] = F32(1e-3)
    return {"check": check, "pattern": pattern, "wide": wide}


def write_spectrum() -> None:
    out = {}
    for name, s in spectrum_inputs().items():
        out[f"{name}_input"] = s
        for fmt in (2, 6):
            v, m = O.ref_spectrum_encode(fmt, s)
            out[f"{name}_values_{fmt}"] = v
            out[f"{name}_meta_{fmt}"] = m
            out[f"{name}_decoded_{fmt}"] = O.ref_spectrum_decode(fmt, v, m, s.size)
    np.savez_compressed(os.path.join(HERE, "spectrum.npz"), **out)
    print("wrote", os.path.join(HERE, "spectrum.npz"))


def write_csv_headers() -> None:
    import tempfile
    lib = O.ref()
    lib.ref_csv_headers.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
    with tempfile.TemporaryDirectory() as tmp:
        a, b = os.path.join(tmp, "s.csv"), os.path.join(tmp, "i.csv")
        assert lib.ref_csv_headers(a.encode(), b.encode()) == 0, lib.ref_last_error()
        lines = [open(a).read().strip(), open(b).read().strip()]
    with open(os.path.join(HERE, "csv_headers.txt"), "w") as f:
        f.write("\n".join(lines) + "\n")
    print("wrote", os.path.join(HERE, "csv_headers.txt"))


def write_paper() -> None:
    lib = O.ref()
    lib.ref_paper_matrix.argtypes = [ctypes.c_int, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_void_p]
    out = {}
    for test_set in (5, 6, 7):
        for n in (32, 64):
            a, meta = np.zeros(n * n), np.zeros(3)
            assert lib.ref_paper_matrix(test_set, n, a.ctypes.data, meta.ctypes.data) == 0, \
                lib.ref_last_error()
            out[f"set{test_set}_n{n}"] = a
            out[f"set{test_set}_n{n}_shift_condition"] = meta[:2]
    np.savez_compressed(os.path.join(HERE, "paper.npz"), **out)
    print("wrote", os.path.join(HERE, "paper.npz"))


def main() -> None:
    if not O.ref_available():
        raise SystemExit("oracle/_ref/libmsq_ref.so missing: run `make -C oracle REF=<reference checkout>` first")
    write_csv_headers()
    if sys.argv[1:] == ["csv"]:
        return
    write_paper()
    if sys.argv[1:] == ["paper"]:
        return
    write_spectrum()
    if sys.argv[1:] == ["spectrum"]:
        return
    lib = O.ref()
    assert lib.ref_check_codecs() == 0, lib.ref_last_error()
    x = codec_inputs()
    out = {"x": x}
    for fmt in range(8):
        v, s = O.ref_encode(fmt, x)
        d = O.ref_decode(fmt, v, s, x.size)
        out[f"values_{fmt}"] = v
        out[f"scales_{fmt}"] = s if s is not None else np.zeros(0, np.uint8)
        out[f"decoded_bits_{fmt}"] = d.view(np.uint32)
    np.savez_compressed(os.path.join(HERE, "codecs.npz"), **out)

    num = {}
    for n, cond in [(16, 10.0), (64, 1e3), (96, 1e2)]:
        a = np.zeros(n * n)
        assert lib.ref_make_spd(n, cond, a.ctypes.data) == 0
        root = np.zeros(n * n)
        assert lib.ref_reference_root(a.ctypes.data, n, root.ctypes.data) == 0
        summary = np.zeros(8)
        hist = np.zeros(2 * 16)
        assert lib.ref_run_accelerate(a.ctypes.data, n, cond, 12, 1e-12, summary.ctypes.data,
                                      hist.ctypes.data, 16) == 0, lib.ref_last_error()
        key = f"n{n}"
        num[f"{key}_a"] = a
        num[f"{key}_root"] = root
        num[f"{key}_summary"] = summary
        num[f"{key}_history"] = hist[:2 * (int(summary[2]) + 1)]
        num[f"{key}_cond"] = np.array([cond])
    np.savez_compressed(os.path.join(HERE, "numerics.npz"), **num)
    print("wrote", os.path.join(HERE, "codecs.npz"), os.path.join(HERE, "numerics.npz"))


if __name__ == "__main__":
    main()
