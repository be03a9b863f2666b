"""The uneven batches' border rows (near-toeplitz-applications_gb300/csrc/
ntk_batch_borders.h) on the CPU: the header's own code, built with g++ by
tests/batch_borders_check.cpp, on the window layouts of both batch kernels
(the paired-chunk / chunked windows and the FP64 windows) for the benchmark
batch's lengths and edge cases.  Every central row that a window of another
CTA reads must go through the work array (a border row): the last window of
a system starts at n - 512 and can reach back past its neighbour, which a
rule against the immediate neighbours alone misses."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "near-toeplitz-applications_gb300", "csrc")


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    out = tmp_path_factory.mktemp("borders") / "libborders.so"
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I", CSRC, "-o", str(out),
           os.path.join(ROOT, "tests", "batch_borders_check.cpp")]
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert res.returncode == 0, res.stdout
    lib = ctypes.CDLL(str(out))
    lib.batch_borders_check.restype = ctypes.c_longlong
    lib.batch_borders_check.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                                        ctypes.c_int, ctypes.POINTER(ctypes.c_longlong)]
    return lib


def _check(lib, layout, lengths, H, per_cta):
    n = np.ascontiguousarray(lengths, dtype=np.int32)
    nb = ctypes.c_longlong()
    bad = lib.batch_borders_check(layout, len(n), n.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), H, per_cta,
                                  ctypes.byref(nb))
    return bad, nb.value


@pytest.mark.parametrize("layout", [0, 1])
@pytest.mark.parametrize("per_cta", [1, 4, 8])
def test_benchmark_batch_borders(lib, layout, per_cta):
    from ntk.workloads import uneven_batch

    lengths, _ = uneven_batch(1024, seed=0)
    bad, nb = _check(lib, layout, lengths, 38, per_cta)
    assert bad == 0
    assert nb > 0


@pytest.mark.parametrize("layout", [0, 1])
def test_last_window_reaching_two_back(lib, layout):
    # n just above a window boundary: the last window (start n - 512) reads
    # rows of the window two before it
    H, L = 38, 512 - 76
    lengths = [512 + L * k - H + d for k in range(1, 6) for d in (1, 2, 5, 20, 37)] + [3, 100, 512, 513, 8192]
    for per_cta in (2, 3, 4):
        bad, _ = _check(lib, layout, lengths, H, per_cta)
        assert bad == 0
