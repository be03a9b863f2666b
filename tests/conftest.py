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
