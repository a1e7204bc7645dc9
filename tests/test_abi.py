"""CPU checks of the C ABI boundary: the shared library loads (no GPU call is
made) and exports every entry point include/*.h declares."""
import glob
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "mixed-mlx_gb300", "libmsq_cuda.so")


def declared_symbols():
    names = set()
    for header in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(header).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:[a-z_]+\s+\**)+\**(msq_[a-z0-9_]+)\s*\(", text, re.M):
            names.add(m.group(1))
    return names


@pytest.fixture(scope="module")
def lib_path():
    if not os.path.exists(LIB):
        import importlib.util
        spec = importlib.util.spec_from_file_location(
            "msq_build", os.path.join(ROOT, "mixed-mlx_gb300", "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
    return LIB


def test_header_declares_the_boundary():
    names = declared_symbols()
    for must in ("msq_create", "msq_encode", "msq_decode", "msq_jacobi_batched",
                 "msq_reconstruct", "msq_residual", "msq_sylvester_sweep", "msq_solve_batched",
                 "msq_mlp_forward", "msq_mlp_backward", "msq_mlp_step", "msq_jacobi_noalloc",
                 "msq_encode_stochastic", "msq_spectrum_encode", "msq_spectrum_decode",
                 "msq_spectrum_metadata_bytes", "msq_native_sylvester_sweep"):
        assert must in names


def test_library_exports_every_declared_symbol(lib_path):
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True,
                         text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = declared_symbols() - exported
    assert not missing, missing


def test_library_loads_without_gpu(lib_path):
    import ctypes
    lib = ctypes.CDLL(lib_path)
    lib.msq_storage_bytes.restype = ctypes.c_size_t
    lib.msq_storage_bytes.argtypes = [ctypes.c_int, ctypes.c_size_t]
    lib.msq_scale_bytes.restype = ctypes.c_size_t
    lib.msq_scale_bytes.argtypes = [ctypes.c_int, ctypes.c_size_t, ctypes.c_size_t]
    # storageBytes / scaleBytes (src/configuration.cpp:188-213), host-only
    assert lib.msq_storage_bytes(7, 33) == 17 and lib.msq_scale_bytes(7, 33, 0) == 2
    lib.msq_spectrum_metadata_bytes.restype = ctypes.c_size_t
    lib.msq_spectrum_metadata_bytes.argtypes = [ctypes.c_size_t]
    # two floats (min, span of log2 s) per block of 8 root eigenvalues
    assert lib.msq_spectrum_metadata_bytes(17) == 24
    assert lib.msq_storage_bytes(1, 10) == 20 and lib.msq_scale_bytes(1, 10, 0) == 0
    assert lib.msq_scale_bytes(8, 64, 16) == 16


def test_python_host_layer_refuses_without_gpu():
    import importlib
    import torch
    msq = importlib.import_module("mixed-mlx_gb300")
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    with pytest.raises(msq.MsqError):
        msq.Context(0)


def test_csv_schema_is_the_references(lib_path):
    """msq_csv_headers (the C++ mirror's writers) against the header lines
    the reference's own writeSummaryHeader / writeIterationsHeader wrote
    (tests/golden/csv_headers.txt)."""
    import ctypes
    lib = ctypes.CDLL(lib_path)
    a, b = ctypes.create_string_buffer(8192), ctypes.create_string_buffer(8192)
    assert lib.msq_csv_headers(a, 8192, b, 8192) == 0
    golden = open(os.path.join(ROOT, "tests", "golden", "csv_headers.txt")).read().split("\n")
    assert a.value.decode().rstrip("\n") == golden[0]
    assert b.value.decode().rstrip("\n") == golden[1]
    assert lib.msq_csv_headers(a, 16, b, 8192) != 0   # too small a buffer
