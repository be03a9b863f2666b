"""Shared fixtures.  Tests marked `gpu` need a CUDA device and the built
libntk.so; everything else runs on the CPU."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(ROOT, "near-toeplitz-applications_gb300")
ORACLE_DIR = os.path.join(ROOT, "oracle")
for p in (PKG_DIR, ORACLE_DIR, ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden", "reference_golden.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libntk.so")


@pytest.fixture(scope="session")
def golden():
    return np.load(GOLDEN)


@pytest.fixture(scope="session")
def oracle():
    import oracle as O

    O.lib()
    return O


@pytest.fixture(scope="session")
def ntk_lib():
    """libntk built in-tree (nvcc cross-compiles without a GPU)."""
    import __graft_entry__ as g

    g._path()
    from importlib import util

    spec = util.spec_from_file_location("_ntk_build", os.path.join(PKG_DIR, "ntk", "build.py"))
    mod = util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build()
    import ntk

    return ntk.load()


@pytest.fixture(scope="session")
def cuda(ntk_lib):
    import torch

    if not torch.cuda.is_available():
        raise RuntimeError("GPU test run without a CUDA device: there is no CPU path to fall back to")
    return torch.device("cuda:0")


@pytest.fixture(scope="session")
def r2emu(tmp_path_factory):
    """The host emulation of the paired-chunk solve (tests/r2_emul.cpp),
    built with g++ from the product's own arithmetic header."""
    import ctypes
    import subprocess

    out = tmp_path_factory.mktemp("r2emu") / "libr2emu.so"
    cuda_inc = os.environ.get("CUDA_HOME", "/usr/local/cuda") + "/include"
    cmd = ["g++", "-O2", "-ffp-contract=off", "-std=c++17", "-fPIC", "-shared",
           "-I", os.path.join(PKG_DIR, "csrc"), "-I", cuda_inc, "-o", str(out),
           os.path.join(ROOT, "tests", "r2_emul.cpp")]
    res = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if res.returncode != 0:
        raise RuntimeError("building the host emulation failed:\n" + res.stdout)
    lib = ctypes.CDLL(str(out))
    P = ctypes.POINTER
    d = ctypes.c_double
    lib.r2emu_solve.argtypes = [ctypes.c_int, ctypes.c_int, P(d), P(d), d, d, d, ctypes.c_int, d, ctypes.c_int,
                                ctypes.c_longlong, P(d), P(d), ctypes.c_char_p, ctypes.c_int]
    lib.r2emu_solve_general.argtypes = [ctypes.c_int, ctypes.c_int, P(d), P(d), d, d, d, d, d, ctypes.c_int,
                                        ctypes.c_longlong, P(d), P(d), ctypes.c_char_p, ctypes.c_int]
    lib.r2emu_split.argtypes = [P(d), ctypes.c_longlong, P(ctypes.c_float), P(ctypes.c_float)]
    lib.r2emu_dw.argtypes = [P(ctypes.c_float), P(ctypes.c_float), ctypes.c_longlong, P(d)]
    return lib


def r2emu_solve(lib, lines, compact=True, sweeps=1, coeffs=(1., 2., .25, 1., .25, 2., 1.), h=1.0 / 511,
                head=None, tail=None):
    """Runs the emulation on `lines` (systems x 512); returns (status, x)."""
    import ctypes

    P = ctypes.POINTER(ctypes.c_double)
    f = np.ascontiguousarray(lines, dtype=np.float64)
    out = np.zeros_like(f)
    b1, c1, ai, bi, ci, an, bn = [float(c) for c in coeffs]
    nh = nt = 1
    if head is None:
        head = [0., b1, c1, 0., 1., 0.]
    else:
        nh = 2
    if tail is None:
        tail = [an, bn, 0., 0., 1., 0.]
    else:
        nt = 2
    hd = np.ascontiguousarray(head, dtype=np.float64)
    tl = np.ascontiguousarray(tail, dtype=np.float64)
    why = ctypes.create_string_buffer(256)
    rc = lib.r2emu_solve(nh, nt, hd.ctypes.data_as(P), tl.ctypes.data_as(P), ai, bi, ci, int(compact), float(h),
                         int(sweeps), f.shape[0], f.ctypes.data_as(P), out.ctypes.data_as(P), why, 256)
    return rc, out
