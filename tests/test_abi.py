"""The C ABI: libntk.so loads, exports every entry point include/ntk.h
declares, and rejects bad arguments with a status and a message before it
touches the GPU.  No compute calls here (this runs without a GPU)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "ntk.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ntk_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for required in ["ntk_plan_create", "ntk_plan_destroy", "ntk_solve", "ntk_solve_strided", "ntk_compact_deriv",
                     "ntk_compact_rhs", "ntk_permute3d", "ntk_adi_rhs", "ntk_transpose2d", "ntk_last_error"]:
        assert required in names


def test_every_declared_symbol_is_exported(ntk_lib):
    missing = [n for n in declared_functions() if not hasattr(ntk_lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_header(ntk_lib):
    from ntk import _lib

    bound = {name for name, _, _ in _lib.SIGNATURES}
    assert set(declared_functions()) <= bound | set(), set(declared_functions()) - bound


def test_version(ntk_lib):
    v = ntk_lib.ntk_version().decode()
    assert "ntk" in v and "sm_103a" in v


def _create(lib, n, nrhs, coeffs, prec, sweeps):
    h = ctypes.c_void_p()
    co = (ctypes.c_double * 7)(*coeffs)
    rc = lib.ntk_plan_create(ctypes.byref(h), n, nrhs, co, prec, sweeps)
    return rc, h


@pytest.mark.parametrize("n,nrhs,prec,sweeps", [(2, 1, 0, 1), (1, 1, 0, 1), (8, -1, 0, 1), (8, 1, 7, 1),
                                                (8, 1, 2, 0), (8, 1, 2, 9)])
def test_plan_create_rejects_bad_arguments(ntk_lib, n, nrhs, prec, sweeps):
    from ntk import _lib

    rc, h = _create(ntk_lib, n, nrhs, (1, 2, .25, 1, .25, 2, 1), prec, sweeps)
    assert rc == _lib.NTK_ERR_INVALID
    assert not h.value
    assert _lib.last_error()


def test_plan_create_rejects_non_finite(ntk_lib):
    from ntk import _lib

    rc, _ = _create(ntk_lib, 8, 1, (1, 2, float("nan"), 1, .25, 2, 1), 0, 1)
    assert rc == _lib.NTK_ERR_INVALID
    assert "finite" in _lib.last_error()


def test_null_arguments_rejected(ntk_lib):
    from ntk import _lib

    assert ntk_lib.ntk_solve(None, None, None) == _lib.NTK_ERR_INVALID
    assert ntk_lib.ntk_compact_rhs(None, None, 8, 8, 8, 0.1, None) == _lib.NTK_ERR_INVALID
    assert ntk_lib.ntk_transpose2d(None, None, 8, None) == _lib.NTK_ERR_INVALID
    assert ntk_lib.ntk_plan_destroy(None) == _lib.NTK_OK


def test_last_error_truncates(ntk_lib):
    ntk_lib.ntk_solve(None, None, None)
    buf = ctypes.create_string_buffer(8)
    full = ntk_lib.ntk_last_error(buf, 8)
    assert full > 7 and len(buf.value) == 7


def test_no_cpu_fallback_for_host_tensors(ntk_lib):
    import torch

    import ntk

    with pytest.raises(ValueError, match="CUDA"):
        ntk.device_ptr(torch.zeros(4, dtype=torch.float64))


def test_missing_library_fails_loudly(tmp_path):
    from ntk import _lib

    with pytest.raises(RuntimeError, match="libntk.so not found"):
        _lib.load(str(tmp_path / "libntk.so"))


def test_tuning_keys_validated(ntk_lib):
    from ntk import _lib

    v = ctypes.c_int()
    assert ntk_lib.ntk_plan_set_tuning(None, 1, 0) == _lib.NTK_ERR_INVALID
    assert ntk_lib.ntk_plan_get_tuning(None, 1, ctypes.byref(v)) == _lib.NTK_ERR_INVALID
