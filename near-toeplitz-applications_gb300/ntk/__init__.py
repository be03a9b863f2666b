"""ntk -- GB300-native batched near-Toeplitz tridiagonal solvers.

Python face of libntk.so (C ABI in include/ntk.h).  Device buffers are
accepted as torch CUDA tensors, objects with ``data_ptr()``, objects with a
``gpudata`` device address (PyCUDA GPUArrays, as the reference passes), or
objects exposing ``__cuda_array_interface__``; all hold float64.

    Plan(n, nrhs, coeffs, precision="fp64"|"fp32"|"fp32_refine", refine_sweeps=1)
        .solve(d)                      in place, nrhs contiguous systems
        .solve_strided(d, out, ...)    strided batches (y/z sweeps without permutes)
        .compact_deriv(f, out, axis, h)  fused compact RHS + solve on a 3D field
    compact_rhs, permute3d, adi_rhs, transpose2d   the reference's free functions

The reference-shaped modules next to this package (neato.py, compact/, adi/)
re-export these under the reference's own names.
"""
import ctypes

from . import _lib
from ._lib import NtkError, PRECISIONS, check, load  # noqa: F401

__all__ = ["Plan", "Adi", "AdiVar", "UnevenBatch", "compact_rhs", "permute3d", "adi_rhs", "transpose2d", "NtkError", "device_ptr",
           "current_stream", "version"]

COMPACT_COEFFS = (1., 2., 1. / 4, 1., 1. / 4, 2., 1.)  # experiments/run-compact.py:48


def version():
    return load().ntk_version().decode()


def _is_torch(x):
    return type(x).__module__.startswith("torch")


def device_ptr(x, need_f64=True):
    """Device address of a buffer (see module docstring)."""
    if _is_torch(x):
        import torch

        if not x.is_cuda:
            raise ValueError("ntk: tensor must live on a CUDA device (there is no CPU path)")
        if need_f64 and x.dtype != torch.float64:
            raise ValueError("ntk: tensor must be float64, got %s" % x.dtype)
        return int(x.data_ptr())
    if hasattr(x, "__cuda_array_interface__"):
        cai = x.__cuda_array_interface__
        if need_f64 and cai.get("typestr") not in ("<f8", "=f8"):
            raise ValueError("ntk: buffer must be float64")
        return int(cai["data"][0])
    if hasattr(x, "gpudata"):
        return int(x.gpudata)
    if hasattr(x, "data_ptr"):
        return int(x.data_ptr())
    if isinstance(x, int):
        return x
    raise TypeError("ntk: cannot take a device pointer of %r" % type(x))


def current_stream(x=None):
    """cudaStream_t to launch on: torch's current stream for torch tensors,
    else the legacy default stream (the reference's, neato.py:181)."""
    if x is None or _is_torch(x):
        try:
            import torch

            if torch.cuda.is_available():
                return int(torch.cuda.current_stream().cuda_stream)
        except Exception:  # pragma: no cover - torch absent
            pass
    return 0


def _stream(stream, x):
    if stream is None:
        return current_stream(x)
    if hasattr(stream, "cuda_stream"):
        return int(stream.cuda_stream)
    if hasattr(stream, "handle"):
        return int(stream.handle)
    return int(stream)


def _available(x):
    """float64 values addressable from x's start to the end of its storage
    (pointer-offset views such as d[1, 0] reach past their own extent, as in
    experiments/run-adi.py:65), or None when unknown."""
    if _is_torch(x):
        try:
            return x.untyped_storage().nbytes() // 8 - x.storage_offset()
        except Exception:
            return x.numel()
    if hasattr(x, "size") and isinstance(getattr(x, "size"), int):
        return int(x.size)
    return None


class Plan:
    """Solver for batches of one near-Toeplitz tridiagonal matrix.

    coeffs = (b1, c1, ai, bi, ci, an, bn) as in the reference (neato.py:136-138).
    """

    def __init__(self, n, nrhs, coeffs, precision="fp64", refine_sweeps=1):
        lib = load()
        if isinstance(precision, str):
            if precision not in PRECISIONS:
                raise ValueError("precision must be one of %s" % sorted(PRECISIONS))
            prec = PRECISIONS[precision]
        else:
            prec = int(precision)
        co = (ctypes.c_double * 7)(*[float(c) for c in coeffs])
        h = ctypes.c_void_p()
        check(lib.ntk_plan_create(ctypes.byref(h), int(n), int(nrhs), co, prec, int(refine_sweeps)))
        self._h = h
        self.n = int(n)
        self.nrhs = int(nrhs)
        self.coeffs = tuple(float(c) for c in coeffs)
        self.precision = precision
        self.refine_sweeps = int(refine_sweeps)

    @property
    def handle(self):
        if self._h is None:
            raise ValueError("ntk: plan is closed")
        return self._h

    def close(self):
        if getattr(self, "_h", None) is not None:
            try:
                load().ntk_plan_destroy(self._h)
            finally:
                self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_tuning(self, **kw):
        """Set launch parameters (ntk_plan_set_tuning): f64_x_variant,
        f64_threads, refine_w, refine_spw, refine_kernel, refine_prefetch,
        refine_tps."""
        for k, v in kw.items():
            if k not in _lib.TUNE_KEYS:
                raise ValueError("unknown tuning key %r" % k)
            check(load().ntk_plan_set_tuning(self.handle, _lib.TUNE_KEYS[k], int(v)))

    def get_tuning(self):
        out = {}
        for k, key in _lib.TUNE_KEYS.items():
            v = ctypes.c_int()
            check(load().ntk_plan_get_tuning(self.handle, key, ctypes.byref(v)))
            out[k] = v.value
        return out


    def status(self, stream=None, raise_on_error=True):
        """Reads and clears the device status of the FP32 / FP32+refine
        solves issued so far (synchronous on the stream): returns the
        NTK_STATUS_* bits; with raise_on_error, an input outside the
        double-word range (|x| >= 2^128, inf, nan) raises NtkError with
        status NTK_ERR_RANGE."""
        flags = ctypes.c_int()
        rc = load().ntk_plan_status(self._h, ctypes.byref(flags), _stream(stream, None))
        if rc != _lib.NTK_ERR_RANGE or raise_on_error:
            check(rc)
        return flags.value

    def solve(self, d, stream=None):
        """In-place solve of nrhs contiguous systems starting at d (neato.py:168-197)."""
        ne = _available(d)
        if ne is not None and ne < self.n * self.nrhs:
            raise ValueError("ntk: buffer holds %d values, need nrhs*n = %d" % (ne, self.n * self.nrhs))
        check(load().ntk_solve(self.handle, device_ptr(d), _stream(stream, d)))

    def solve_strided(self, d_in, d_out, nsys, ni, is_, os_, es, stream=None):
        check(load().ntk_solve_strided(self.handle, device_ptr(d_in), device_ptr(d_out), int(nsys), int(ni),
                                       int(is_), int(os_), int(es), _stream(stream, d_in)))

    def compact_deriv(self, f, out, axis, h, shape=None, stream=None):
        """Compact 4th-order derivative of the [nz][ny][nx] field f along axis
        (0=z, 1=y, 2=x) into out; one fused pass, no permutes."""
        if shape is None:
            shape = tuple(f.shape)
        if len(shape) == 2:
            shape = (1,) + tuple(shape)
            axis = axis + 1 if axis >= 0 else axis
        nz, ny, nx = [int(v) for v in shape]
        if axis < 0:
            axis += 3
        if _is_torch(f) and not f.is_contiguous():
            raise ValueError("ntk: f must be C-contiguous")
        if _is_torch(out) and not out.is_contiguous():
            raise ValueError("ntk: out must be C-contiguous")
        check(load().ntk_compact_deriv(self.handle, device_ptr(f), device_ptr(out), nz, ny, nx, int(axis),
                                       float(h), _stream(stream, f)))


    def compact_grad(self, f, dfdx, dfdy, dfdz, h, stream=None):
        """dfdx, dfdy, dfdz of the n x n x n field f (experiments/run-compact.py:47-90
        in one call; one kernel launch for n = 512 on the FP32 paths)."""
        for t in (f, dfdx, dfdy, dfdz):
            if _is_torch(t) and not t.is_contiguous():
                raise ValueError("ntk: arrays must be C-contiguous")
        nz, ny, nx = [int(v) for v in f.shape]
        check(load().ntk_compact_grad(self.handle, device_ptr(f), device_ptr(dfdx), device_ptr(dfdy),
                                      device_ptr(dfdz), nz, ny, nx, float(h), _stream(stream, f)))


class Adi:
    """Peaceman-Rachford ADI stepper for N x N fields (experiments/run-adi.py).

    step(u, d_x, d_y) / run(u, d_x, d_y, steps, graph=True) operate on device
    arrays with the reference's meaning (see ntk_adi_step in include/ntk.h).
    """

    def __init__(self, N, dx, dt, precision="fp64"):
        lib = load()
        prec = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        h = ctypes.c_void_p()
        check(lib.ntk_adi_create(ctypes.byref(h), int(N), float(dx), float(dt), prec))
        self._h = h
        self.N, self.dx, self.dt = int(N), float(dx), float(dt)

    @property
    def segments(self):
        L, H, P = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(load().ntk_adi_segments(self._h, ctypes.byref(L), ctypes.byref(H), ctypes.byref(P)))
        return L.value, H.value, P.value


    def status(self, stream=None, raise_on_error=True):
        """Reads and clears the device status of the FP32 / FP32+refine
        solves issued so far (synchronous on the stream): returns the
        NTK_STATUS_* bits; with raise_on_error, an input outside the
        double-word range (|x| >= 2^128, inf, nan) raises NtkError with
        status NTK_ERR_RANGE."""
        flags = ctypes.c_int()
        rc = load().ntk_adi_status(self._h, ctypes.byref(flags), _stream(stream, None))
        if rc != _lib.NTK_ERR_RANGE or raise_on_error:
            check(rc)
        return flags.value

    def step(self, u, d_x, d_y, stream=None):
        check(load().ntk_adi_step(self._h, device_ptr(u), device_ptr(d_x), device_ptr(d_y), _stream(stream, u)))

    def run(self, u, d_x, d_y, steps, graph=True, stream=None):
        check(load().ntk_adi_run(self._h, device_ptr(u), device_ptr(d_x), device_ptr(d_y), int(steps),
                                 1 if graph else 0, _stream(stream, u)))

    def close(self):
        if getattr(self, "_h", None) is not None:
            try:
                load().ntk_adi_destroy(self._h)
            finally:
                self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class AdiVar:
    """ADI with per-line coefficients (ntk_adi_var_* in include/ntk.h):
    u_t = kx(y) u_xx + ky(x) u_yy, kx[j] on row j, ky[i] on column i
    (float64 arrays of length N; kx = ky = 1 is Adi's step).

    step(u, d_x, d_y) runs one Peaceman-Rachford step as run-adi.py:59-71
    does: afterwards d_x holds the x half step, d_y the y half step and
    u = d_y^T."""

    def __init__(self, N, dx, dt, kx, ky, precision="fp64"):
        import numpy as np

        lib = load()
        prec = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        kxa = np.ascontiguousarray(kx, dtype=np.float64)
        kya = np.ascontiguousarray(ky, dtype=np.float64)
        if kxa.size != int(N) or kya.size != int(N):
            raise ValueError("ntk: kx and ky need N values each")
        h = ctypes.c_void_p()
        check(lib.ntk_adi_var_create(ctypes.byref(h), int(N), float(dx), float(dt), kxa.ctypes.data,
                                     kya.ctypes.data, prec))
        self._h = h
        self.N = int(N)

    def step(self, u, d_x, d_y, stream=None):
        check(load().ntk_adi_var_step(self._h, device_ptr(u), device_ptr(d_x), device_ptr(d_y), _stream(stream, u)))

    def status(self, stream=None, raise_on_error=True):
        flags = ctypes.c_int()
        rc = load().ntk_adi_var_status(self._h, ctypes.byref(flags), _stream(stream, None))
        if rc != _lib.NTK_ERR_RANGE or raise_on_error:
            check(rc)
        return flags.value

    def close(self):
        if getattr(self, "_h", None) is not None:
            try:
                load().ntk_adi_var_destroy(self._h)
            finally:
                self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class UnevenBatch:
    """Many near-Toeplitz systems of different lengths/coefficients in one
    buffer, solved in place by one persistent launch (see ntk_batch_create).

    lengths: int array (nsys,), offsets: int64 array (nsys,) or None (packed),
    interior: (nsys, 3) (a, b, c), head: (nsys, 2, 3) rows 0 and 1,
    tail: (nsys, 2, 3) rows n-2 and n-1.
    """

    def __init__(self, lengths, interior, head, tail, offsets=None, precision="fp64"):
        import numpy as np

        lib = load()
        n = np.ascontiguousarray(lengths, dtype=np.int32)
        if offsets is None:
            offsets = np.concatenate([[0], np.cumsum(n.astype(np.int64))[:-1]]) if len(n) else np.zeros(0)
        off = np.ascontiguousarray(offsets, dtype=np.int64)
        inter = np.ascontiguousarray(interior, dtype=np.float64).reshape(-1)
        hd = np.ascontiguousarray(head, dtype=np.float64).reshape(-1)
        tl = np.ascontiguousarray(tail, dtype=np.float64).reshape(-1)
        if not (len(off) == len(n) and inter.size == 3 * len(n) and hd.size == 6 * len(n) and tl.size == 6 * len(n)):
            raise ValueError("ntk: descriptor arrays do not match the number of systems")
        prec = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        h = ctypes.c_void_p()
        check(lib.ntk_batch_create(ctypes.byref(h), len(n), n.ctypes.data, off.ctypes.data, inter.ctypes.data,
                                   hd.ctypes.data, tl.ctypes.data, prec))
        self._h = h
        self.lengths = n
        self.offsets = off
        self.elements = int((off + n).max()) if len(n) else 0

    def status(self, stream=None, raise_on_error=True):
        """Reads and clears the device status of the FP32 / FP32+refine
        solves issued so far (synchronous on the stream): returns the
        NTK_STATUS_* bits; with raise_on_error, an input outside the
        double-word range (|x| >= 2^128, inf, nan) raises NtkError with
        status NTK_ERR_RANGE."""
        flags = ctypes.c_int()
        rc = load().ntk_batch_status(self._h, ctypes.byref(flags), _stream(stream, None))
        if rc != _lib.NTK_ERR_RANGE or raise_on_error:
            check(rc)
        return flags.value

    def info(self):
        a, b, c = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_longlong()
        check(load().ntk_batch_info(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return {"max_n": a.value, "segmented": b.value, "elements": c.value}

    def windows(self):
        """{"windows": 512-row windows solved, "paired": how many of them on
        the paired-chunk FP32 solve (FP32 / FP32 + refinement batches).}"""
        w, p = ctypes.c_longlong(), ctypes.c_longlong()
        check(load().ntk_batch_windows(self._h, ctypes.byref(w), ctypes.byref(p)))
        return {"windows": w.value, "paired": p.value}

    def solve(self, d, stream=None):
        ne = _available(d)
        if ne is not None and ne < self.elements:
            raise ValueError("ntk: buffer holds %d values, the batch spans %d" % (ne, self.elements))
        check(load().ntk_batch_solve(self._h, device_ptr(d), _stream(stream, d)))

    def close(self):
        if getattr(self, "_h", None) is not None:
            try:
                load().ntk_batch_destroy(self._h)
            finally:
                self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def compact_rhs(f, rhs, dx, stream=None):
    """compute_rhs(f, rhs, dx) of compact/rhs.py:47-53 (last axis of a 3D field)."""
    shape = tuple(f.shape)
    if len(shape) == 2:
        shape = (1,) + shape
    nz, ny, nx = shape
    check(load().ntk_compact_rhs(device_ptr(f), device_ptr(rhs), nz, ny, nx, float(dx), _stream(stream, f)))


def permute3d(a, b, permutation, stream=None):
    """permute(a_d, b_d, permutation) of compact/permute.py:32-52: b = a.transpose(permutation)."""
    if _is_torch(a):
        st = [int(s) for s in a.stride()]
    else:
        st = [int(s) // 8 for s in a.strides]
    s = [st[p] for p in permutation]
    oshape = [int(a.shape[p]) for p in permutation]
    check(load().ntk_permute3d(device_ptr(a), device_ptr(b), oshape[0], oshape[1], oshape[2], s[0], s[1], s[2],
                               _stream(stream, a)))


def adi_rhs(u, d, dx, dt, N, stream=None):
    """compute_rhs(u, d, dx, dt, N) of adi/rhs.py:35-55 (interior points only)."""
    check(load().ntk_adi_rhs(device_ptr(u), device_ptr(d), int(N), float(dx), float(dt), _stream(stream, u)))


def transpose2d(a, b, N, stream=None):
    """transpose(a, b, N) of adi/transpose.py:40-50: b = a^T."""
    check(load().ntk_transpose2d(device_ptr(a), device_ptr(b), int(N), _stream(stream, a)))
