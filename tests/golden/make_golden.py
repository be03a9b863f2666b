"""Generate the golden vectors in tests/golden/ from the reference itself.

Run where the reference tree exists (it is not needed afterwards):

    python tests/golden/make_golden.py [REFERENCE_ROOT]

Sources of truth, all the reference's own code:
  * coefficients: the reference's _precompute_coefficients (neato.py:199-274),
    taken out of neato.py with `ast` and executed as is;
  * kernel outputs: the reference's CUDA kernels (neato.py:8-124,
    compact/rhs.py:9-37, compact/permute.py:7-20, adi/rhs.py:10-25,
    adi/transpose.py:9-27) rendered exactly as the reference renders them and
    executed on the CPU by oracle/ref_cpu.cpp (one OS thread per CUDA thread,
    __syncthreads as a barrier, strict IEEE double arithmetic without
    contraction).
Inputs are seeded (numpy.random.default_rng), sizes small enough that the
fixtures total a few hundred KB.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))

import oracle as O  # noqa: E402
import render_ref  # noqa: E402

COMPACT = (1., 2., 1. / 4, 1., 1. / 4, 2., 1.)  # experiments/run-compact.py:48


def adi_coeffs(dx, dt):  # experiments/run-adi.py:50-53
    return (1., 0., 1. / (dx * dx), -2. * (1. / dt + 1. / (dx * dx)), 1. / (dx * dx), 0., 1.)


COEFF_SETS = {
    "compact": COMPACT,
    "adi256": adi_coeffs(1.0 / 255, 0.1),            # run-adi.py:37-39 defaults (N=256)
    "adi2048_r05": adi_coeffs(1.0 / 2047, (1.0 / 2047) ** 2),  # r = dt / (2 dx^2) = 0.5
    "dominant": (2.5, 0.7, 0.3, 1.9, 0.45, -0.6, 3.1),
}


def main(ref_root):
    pre = render_ref.precompute_coefficients_from_reference(ref_root)
    R = O.ref_cpu()
    if R is None:
        raise SystemExit("oracle/_ref/libntkref_cpu.so could not be built")
    rng = np.random.default_rng(20240601)
    out = {}
    # 1. coefficient arrays for n = 4 .. 2048
    for cname, co in COEFF_SETS.items():
        for L in range(2, 12):
            n = 1 << L
            arrs = pre(n, co)
            out["coef_%s_n%d" % (cname, n)] = np.stack(arrs)
    # 2. reference CR solves (the kernel itself), n = 4 .. 1024
    for cname, co in COEFF_SETS.items():
        for L in range(2, 11 if cname == "compact" else 9):
            n = 1 << L
            nrhs = 3 if n <= 64 else (2 if n <= 256 else 1)
            d = rng.normal(size=(nrhs, n))
            arrs = [np.ascontiguousarray(a) for a in pre(n, co)]
            x = d.copy()
            rc = R.ntkref_cpu_cr(n, nrhs, *[O._ptr(a) for a in arrs], co[0], co[1], co[2], co[3], co[4], O._ptr(x))
            assert rc == 0
            out["cr_%s_n%d_in" % (cname, n)] = d
            out["cr_%s_n%d_out" % (cname, n)] = x
    # 3. compact RHS on an [8][8][16] field
    f = rng.normal(size=(8, 8, 16))
    rhs = np.empty_like(f)
    assert R.ntkref_cpu_compact_rhs(O._ptr(f), O._ptr(rhs), 8, 8, 16, 0.05) == 0
    out["rhs_in"], out["rhs_out"], out["rhs_dx"] = f, rhs, np.array(0.05)
    # 4. permutes of an 8^3 cube, the three the drivers use (run-compact.py:70-86)
    a = rng.normal(size=(8, 8, 8))
    out["perm_in"] = a
    for perm in [(0, 2, 1), (1, 2, 0), (2, 0, 1)]:
        st = np.array(a.strides) // 8
        s = st[list(perm)]
        b = np.empty_like(a)
        assert R.ntkref_cpu_permute(O._ptr(a), O._ptr(b), 8, 8, 8, int(s[0]), int(s[1]), int(s[2])) == 0
        out["perm_%d%d%d" % perm] = b
    # 5. ADI explicit stencil and transpose, N = 32
    u = rng.normal(size=(32, 32))
    d = rng.normal(size=(32, 32))
    d_ref = d.copy()
    assert R.ntkref_cpu_adi_rhs(O._ptr(u), O._ptr(d_ref), 32, 1.0 / 31, 0.01) == 0
    out["adi_rhs_u"], out["adi_rhs_d"], out["adi_rhs_out"] = u, d, d_ref
    t = np.empty_like(u)
    assert R.ntkref_cpu_transpose(O._ptr(u), O._ptr(t), 32) == 0
    out["transpose_in"], out["transpose_out"] = u, t
    # 6. three ADI steps, N = 32, as run-adi.py:59-71 with the reference's own kernels
    N = 32
    dx, dt = 1.0 / (N - 1), 0.1
    co = adi_coeffs(dx, dt)
    arrs = [np.ascontiguousarray(v) for v in pre(N, co)]
    u = np.zeros((N, N))
    u[:, :] = 0.5
    u[:, 0] = 1.0  # run-adi.py:42-44
    d_x = u.copy()
    d_y = u.transpose().copy()
    out["adi_step_u0"] = u.copy()
    for _ in range(3):
        assert R.ntkref_cpu_adi_rhs(O._ptr(u), O._ptr(d_x), N, dx, dt) == 0
        v = d_x[1:].copy()
        assert R.ntkref_cpu_cr(N, N - 2, *[O._ptr(q) for q in arrs], co[0], co[1], co[2], co[3], co[4], O._ptr(v)) == 0
        d_x[1:N - 1] = v[:N - 2]
        assert R.ntkref_cpu_transpose(O._ptr(d_x), O._ptr(u), N) == 0
        assert R.ntkref_cpu_adi_rhs(O._ptr(u), O._ptr(d_y), N, dx, dt) == 0
        v = d_y[1:].copy()
        assert R.ntkref_cpu_cr(N, N - 2, *[O._ptr(q) for q in arrs], co[0], co[1], co[2], co[3], co[4], O._ptr(v)) == 0
        d_y[1:N - 1] = v[:N - 2]
        assert R.ntkref_cpu_transpose(O._ptr(d_y), O._ptr(u), N) == 0
    out["adi_step_u3"] = u
    out["adi_step_dx"], out["adi_step_dt"] = np.array(dx), np.array(dt)
    # 7. compact derivative end to end on an 8^3 field: rhs + CR (x), and
    #    permute + rhs + CR + permute (y), as run-compact.py:57-76
    n = 8
    h = 2 * np.pi / (n - 1)
    f = rng.normal(size=(n, n, n))
    arrs = [np.ascontiguousarray(v) for v in pre(n, COMPACT)]
    dfdx = np.empty_like(f)
    assert R.ntkref_cpu_compact_rhs(O._ptr(f), O._ptr(dfdx), n, n, n, h) == 0
    assert R.ntkref_cpu_cr(n, n * n, *[O._ptr(q) for q in arrs], *COMPACT[:5], O._ptr(dfdx)) == 0
    fy = np.empty_like(f)
    tmp = np.empty_like(f)
    dfdy = np.empty_like(f)
    st = np.array(f.strides) // 8
    s = st[[0, 2, 1]]
    assert R.ntkref_cpu_permute(O._ptr(f), O._ptr(fy), n, n, n, int(s[0]), int(s[1]), int(s[2])) == 0
    assert R.ntkref_cpu_compact_rhs(O._ptr(fy), O._ptr(tmp), n, n, n, h) == 0
    assert R.ntkref_cpu_cr(n, n * n, *[O._ptr(q) for q in arrs], *COMPACT[:5], O._ptr(tmp)) == 0
    st = np.array(tmp.strides) // 8
    s = st[[0, 2, 1]]
    assert R.ntkref_cpu_permute(O._ptr(tmp), O._ptr(dfdy), n, n, n, int(s[0]), int(s[1]), int(s[2])) == 0
    out["deriv_f"], out["deriv_h"], out["deriv_dfdx"], out["deriv_dfdy"] = f, np.array(h), dfdx, dfdy
    path = os.path.join(HERE, "reference_golden.npz")
    np.savez_compressed(path, **out)
    print("wrote %s (%d arrays, %.0f KB)" % (path, len(out), os.path.getsize(path) / 1024))


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("NTK_REFERENCE_ROOT", "")
    if not root:
        print("usage: make_golden.py REFERENCE_ROOT (or set NTK_REFERENCE_ROOT)")
        sys.exit(2)
    main(root)
