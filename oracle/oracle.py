"""Python face of the parity checker (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and the CPU-baseline legs of bench.py
may import this module.  It wraps

  * libntk_oracle.so -- the C restatement of the reference (ntk_oracle.c),
  * oracle/_ref/libntkref_cpu.so -- the reference's own kernels run on the
    CPU (ref_cpu.cpp), when it was built,
  * oracle/_ref/libntkref_gpu.so -- the reference's own kernels on the GPU
    (ref_gpu.cu), when it was built,

and restates the reference's CPU path with NumPy/SciPy:

  tridiagonal_solve      experiments/run-compact.py:14-28 (solve_banded)
  banded_compact_deriv   RHS of compact/rhs.py:21-36 + the banded solve, any axis
  adi_step_banded        experiments/run-adi.py:59-71 with the banded solve
  thomas_ld / exact_solve / adi_step_exact   the same in long double: the
                         accuracy reference for badly scaled (ADI) matrices
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

_c_double_p = ctypes.POINTER(ctypes.c_double)
_lib = None
_ref_cpu = None
_ref_gpu = None


def _ptr(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_c_double_p)


def lib():
    """The C restatement, built on first use."""
    global _lib
    if _lib is None:
        from importlib import util

        spec = util.spec_from_file_location("_ntk_oracle_build", os.path.join(HERE, "build.py"))
        mod = util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        path = mod.build_oracle()
        L = ctypes.CDLL(path)
        L.ntko_precompute.restype = ctypes.c_int
        L.ntko_precompute.argtypes = [ctypes.c_int, _c_double_p] + [_c_double_p] * 8
        L.ntko_cr_solve.restype = ctypes.c_int
        L.ntko_cr_solve.argtypes = [ctypes.c_int, ctypes.c_long, _c_double_p, _c_double_p]
        L.ntko_thomas.restype = ctypes.c_int
        L.ntko_thomas.argtypes = [ctypes.c_int] + [_c_double_p] * 5
        L.ntko_thomas_ld.restype = ctypes.c_int
        L.ntko_thomas_ld.argtypes = [ctypes.c_int, ctypes.c_long] + [_c_double_p] * 5
        L.ntko_compact_rhs.restype = None
        L.ntko_compact_rhs.argtypes = [_c_double_p, _c_double_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_double]
        L.ntko_permute.restype = None
        L.ntko_permute.argtypes = [_c_double_p, _c_double_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_long, ctypes.c_long, ctypes.c_long]
        L.ntko_adi_rhs.restype = None
        L.ntko_adi_rhs.argtypes = [_c_double_p, _c_double_p, ctypes.c_int, ctypes.c_double, ctypes.c_double]
        L.ntko_transpose.restype = None
        L.ntko_transpose.argtypes = [_c_double_p, _c_double_p, ctypes.c_int]
        L.ntko_adi_step.restype = ctypes.c_int
        L.ntko_adi_step.argtypes = [_c_double_p, _c_double_p, _c_double_p, ctypes.c_int, ctypes.c_double,
                                    ctypes.c_double]
        _lib = L
    return _lib


def ref_cpu():
    """The reference's own kernels executed on the CPU, or None."""
    global _ref_cpu
    if _ref_cpu is None:
        path = os.path.join(HERE, "_ref", "libntkref_cpu.so")
        if not os.path.exists(path):
            from importlib import util

            spec = util.spec_from_file_location("_ntk_oracle_build", os.path.join(HERE, "build.py"))
            mod = util.module_from_spec(spec)
            spec.loader.exec_module(mod)
            try:
                path = mod.build_ref_cpu()
            except RuntimeError:
                path = None
            if not path:
                return None
        L = ctypes.CDLL(path)
        L.ntkref_cpu_cr.restype = ctypes.c_int
        L.ntkref_cpu_cr.argtypes = ([ctypes.c_int, ctypes.c_long] + [_c_double_p] * 8 + [ctypes.c_double] * 5
                                    + [_c_double_p])
        L.ntkref_cpu_compact_rhs.restype = ctypes.c_int
        L.ntkref_cpu_compact_rhs.argtypes = [_c_double_p, _c_double_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_double]
        L.ntkref_cpu_permute.restype = ctypes.c_int
        L.ntkref_cpu_permute.argtypes = [_c_double_p, _c_double_p] + [ctypes.c_int] * 6
        L.ntkref_cpu_adi_rhs.restype = ctypes.c_int
        L.ntkref_cpu_adi_rhs.argtypes = [_c_double_p, _c_double_p, ctypes.c_int, ctypes.c_double, ctypes.c_double]
        L.ntkref_cpu_transpose.restype = ctypes.c_int
        L.ntkref_cpu_transpose.argtypes = [_c_double_p, _c_double_p, ctypes.c_int]
        _ref_cpu = L
    return _ref_cpu


def ref_gpu():
    """The reference's own kernels compiled for the GPU, or None."""
    global _ref_gpu
    if _ref_gpu is None:
        path = os.path.join(HERE, "_ref", "libntkref_gpu.so")
        if not os.path.exists(path):
            return None
        L = ctypes.CDLL(path)
        vp = ctypes.c_void_p
        L.ntkref_gpu_cr.restype = ctypes.c_int
        L.ntkref_gpu_cr.argtypes = [ctypes.c_int, ctypes.c_long] + [vp] * 8 + [ctypes.c_double] * 5 + [vp, vp]
        L.ntkref_gpu_compact_rhs.restype = ctypes.c_int
        L.ntkref_gpu_compact_rhs.argtypes = [vp, vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, vp]
        L.ntkref_gpu_permute.restype = ctypes.c_int
        L.ntkref_gpu_permute.argtypes = [vp, vp] + [ctypes.c_int] * 6 + [vp]
        L.ntkref_gpu_adi_rhs.restype = ctypes.c_int
        L.ntkref_gpu_adi_rhs.argtypes = [vp, vp, ctypes.c_int, ctypes.c_double, ctypes.c_double, vp]
        L.ntkref_gpu_transpose.restype = ctypes.c_int
        L.ntkref_gpu_transpose.argtypes = [vp, vp, ctypes.c_int, vp]
        _ref_gpu = L
    return _ref_gpu


# --------------------------------------------------------------------------
# C restatement wrappers
# --------------------------------------------------------------------------

def precompute(n, coeffs):
    """neato.py:199-274 -> (a, b, c, k1, k2, b_first, k1_first, k1_last)."""
    L = int(np.log2(n))
    arrs = [np.zeros(max(L, 1)) for _ in range(8)]
    co = np.ascontiguousarray(coeffs, dtype=np.float64)
    rc = lib().ntko_precompute(n, _ptr(co), *[_ptr(a) for a in arrs])
    if rc:
        raise ValueError("n must be a power of two >= 4")
    return tuple(arrs)


def cr_solve(d, n, coeffs):
    """NearToeplitzSolver(n, nrhs, coeffs).solve on a copy of d (neato.py:168-197)."""
    out = np.array(d, dtype=np.float64, order="C", copy=True)
    nrhs = out.size // n
    co = np.ascontiguousarray(coeffs, dtype=np.float64)
    if lib().ntko_cr_solve(n, nrhs, _ptr(co), _ptr(out)):
        raise ValueError("n must be a power of two >= 4")
    return out


def thomas(a, b, c, d):
    n = len(b)
    x = np.empty(n)
    rc = lib().ntko_thomas(n, *[_ptr(np.ascontiguousarray(v, dtype=np.float64)) for v in (a, b, c, d)], _ptr(x))
    if rc:
        raise ValueError("bad system")
    return x


def thomas_ld(a, b, c, d):
    """Thomas in long double for the rows of d (..., n); returns float64."""
    d = np.ascontiguousarray(d, dtype=np.float64)
    n = d.shape[-1]
    out = np.empty_like(d)
    vecs = [np.ascontiguousarray(v, dtype=np.float64) for v in (a, b, c)]
    if lib().ntko_thomas_ld(n, d.size // n, *[_ptr(v) for v in vecs], _ptr(d), _ptr(out)):
        raise ValueError("bad system")
    return out


def exact_solve(d, n, coeffs):
    """High-precision solve of NearToeplitzSolver's systems (rows of d)."""
    a, b, c = near_toeplitz_bands(n, coeffs)
    return thomas_ld(a, b, c, np.asarray(d).reshape(-1, n)).reshape(np.shape(d))


def compact_rhs(f, dx):
    """compact/rhs.py:9-37: derivative RHS along the last axis of a 3D field."""
    f = np.ascontiguousarray(f, dtype=np.float64)
    nz, ny, nx = f.shape
    out = np.empty_like(f)
    lib().ntko_compact_rhs(_ptr(f), _ptr(out), nz, ny, nx, dx)
    return out


def permute(a, permutation):
    """compact/permute.py:32-52 == numpy.transpose(a, permutation)."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    st = np.array(a.strides) // a.itemsize
    s = st[list(permutation)]
    shape = [a.shape[p] for p in permutation]
    out = np.empty(shape)
    lib().ntko_permute(_ptr(a), _ptr(out), shape[0], shape[1], shape[2], int(s[0]), int(s[1]), int(s[2]))
    return out


def adi_rhs(u, d, dx, dt):
    """adi/rhs.py:35-55 applied in place to d (interior points only)."""
    N = u.shape[0]
    lib().ntko_adi_rhs(_ptr(u), _ptr(d), N, dx, dt)


def transpose(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.empty_like(a)
    lib().ntko_transpose(_ptr(a), _ptr(b), a.shape[0])
    return b


def adi_step(u, d_x, d_y, dx, dt):
    """experiments/run-adi.py:59-71, in place on u, d_x, d_y."""
    if lib().ntko_adi_step(_ptr(u), _ptr(d_x), _ptr(d_y), u.shape[0], dx, dt):
        raise ValueError("bad ADI size")


# --------------------------------------------------------------------------
# the reference's CPU path (SciPy banded solve)
# --------------------------------------------------------------------------

def tridiagonal_solve(a, b, c, rhs):
    """experiments/run-compact.py:14-28: banded LAPACK solve.

    a: sub-diagonal (first entry ignored), b: diagonal, c: super-diagonal
    (last entry ignored); rhs may be n x K (K right-hand sides)."""
    from scipy.linalg import solve_banded

    ab = np.vstack([np.append(0, c[:-1]), b, np.append(a[1:], 0)])
    return solve_banded((1, 1), ab, rhs)


def near_toeplitz_bands(n, coeffs):
    """Full diagonals of NearToeplitzSolver's matrix (neato.py:136-138)."""
    b1, c1, ai, bi, ci, an, bn = [float(v) for v in coeffs]
    a = np.full(n, ai)
    b = np.full(n, bi)
    c = np.full(n, ci)
    b[0], c[0] = b1, c1
    a[-1], b[-1] = an, bn
    a[0] = 0.0
    c[-1] = 0.0
    return a, b, c


def near_toeplitz_bands_general(n, interior, head, tail):
    """Diagonals of one system of an uneven batch (ntk_batch_create's model,
    which generalises neato.py:136-138 to two special rows per end): rows 0
    and 1 from head, rows n-2 and n-1 from tail, interior (a, b, c) between;
    for n = 3 the shared middle row is head's second row."""
    a = np.full(n, float(interior[0]))
    b = np.full(n, float(interior[1]))
    c = np.full(n, float(interior[2]))
    for r in range(2):
        if n - 2 + r >= 2:
            a[n - 2 + r], b[n - 2 + r], c[n - 2 + r] = tail[r]
    for r in range(2):
        a[r], b[r], c[r] = head[r]
    a[0] = 0.0
    c[-1] = 0.0
    return a, b, c


def compact_rhs_numpy(f, h, axis):
    """compact/rhs.py:21-36 along `axis`, vectorised NumPy."""
    f = np.moveaxis(np.asarray(f, dtype=np.float64), axis, -1)
    d = np.empty_like(f)
    d[..., 1:-1] = (3. / (4 * h)) * (f[..., 2:] - f[..., :-2])
    d[..., 0] = (1. / (2 * h)) * (-5 * f[..., 0] + 4 * f[..., 1] + f[..., 2])
    d[..., -1] = -(1. / (2 * h)) * (-5 * f[..., -1] + 4 * f[..., -2] + f[..., -3])
    return np.moveaxis(d, -1, axis)


COMPACT_COEFFS = (1., 2., 1. / 4, 1., 1. / 4, 2., 1.)  # experiments/run-compact.py:48


def banded_compact_deriv(f, h, axis, coeffs=COMPACT_COEFFS):
    """The reference's CPU path for one derivative: RHS + one banded solve
    with all systems as right-hand-side columns."""
    d = compact_rhs_numpy(f, h, axis)
    dm = np.moveaxis(d, axis, 0)
    n = dm.shape[0]
    shp = dm.shape
    a, b, c = near_toeplitz_bands(n, coeffs)
    x = tridiagonal_solve(a, b, c, dm.reshape(n, -1))
    return np.moveaxis(x.reshape(shp), 0, axis)


def adi_coeffs(dx, dt):
    """experiments/run-adi.py:50-53."""
    return (1., 0., 1. / (dx * dx), -2. * (1. / dt + 1. / (dx * dx)), 1. / (dx * dx), 0., 1.)


def adi_step_banded(u, d_x, d_y, dx, dt):
    """experiments/run-adi.py:59-71 with the CPU banded solve in place of the
    reference CR: stencil (adi/rhs.py:21-24,46-49), solve rows 1..N-2,
    transpose, twice.  In place on u, d_x, d_y (NumPy arrays)."""
    N = u.shape[0]
    bottom = -1. / (dx * dx)
    top = -1. / (dx * dx)
    center = 2 * (-1. / dt + 1. / (dx * dx))
    a, b, c = near_toeplitz_bands(N, adi_coeffs(dx, dt))
    for d in (d_x, d_y):
        d[1:-1, 1:-1] = bottom * u[:-2, 1:-1] + center * u[1:-1, 1:-1] + top * u[2:, 1:-1]
        d[1:-1, :] = tridiagonal_solve(a, b, c, d[1:-1, :].T).T
        u[:, :] = d.T


def adi_step_exact(u, d_x, d_y, dx, dt):
    """experiments/run-adi.py:59-71 with the long-double Thomas solve."""
    N = u.shape[0]
    bottom = -1. / (dx * dx)
    top = -1. / (dx * dx)
    center = 2 * (-1. / dt + 1. / (dx * dx))
    a, b, c = near_toeplitz_bands(N, adi_coeffs(dx, dt))
    for d in (d_x, d_y):
        d[1:-1, 1:-1] = bottom * u[:-2, 1:-1] + center * u[1:-1, 1:-1] + top * u[2:, 1:-1]
        d[1:-1, :] = thomas_ld(a, b, c, d[1:-1, :])
        u[:, :] = d.T


def adi_step_var_exact(u, d_x, d_y, dx, dt, kx, ky):
    """experiments/run-adi.py:59-71 with per-line coefficients (the model of
    ntk_adi_var_step: kx[j] on row j of the x operator, ky[i] on column i of
    the y operator) and the long-double Thomas solve.  In place."""
    N = u.shape[0]
    kx = np.asarray(kx, dtype=np.float64)
    ky = np.asarray(ky, dtype=np.float64)
    rdx2 = 1. / (dx * dx)
    for d, kst, kmat in ((d_x, ky, kx), (d_y, kx, ky)):
        beta = kst * rdx2
        bt = -beta
        cen = 2 * (-1. / dt + beta)
        d[1:-1, 1:-1] = bt[None, 1:-1] * u[:-2, 1:-1] + cen[None, 1:-1] * u[1:-1, 1:-1] + bt[None, 1:-1] * u[2:, 1:-1]
        for j in range(1, N - 1):
            c = kmat[j] * rdx2
            a, b, cc = near_toeplitz_bands(N, (1., 0., c, -2. * (1. / dt + c), c, 0., 1.))
            d[j, :] = thomas_ld(a, b, cc, d[j, :])
        u[:, :] = d.T


def rel_err(x, ref):
    """max |x - ref| / max |ref| (normwise relative error)."""
    x = np.asarray(x, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    den = np.max(np.abs(ref))
    num = np.max(np.abs(x - ref))
    return float(num / den) if den > 0 else float(num)
