"""Fused compact 4th-order derivative (compute_rhs + solve, with strided
addressing instead of permutes for y and z) against the oracle.

FP64: within 1e-13 relative of the reference pipeline (RHS + CR + permutes,
restated in oracle/ntk_oracle.c); FP32+refine: within 1e-12 of the FP64
banded solve."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

COMPACT = (1., 2., 1. / 4, 1., 1. / 4, 2., 1.)
FP64_TOL = 1e-13
REFINE_TOL = 1e-12


def fourier_field(shape, seed=0, modes=8, kmax=16):
    """Seeded sum of sine/cosine modes, N(0,1) amplitudes, integer wavenumbers."""
    rng = np.random.default_rng(seed)
    grids = np.meshgrid(*[np.linspace(0, 1, s) for s in shape], indexing="ij")
    f = np.zeros(shape)
    for _ in range(modes):
        k = rng.integers(1, kmax + 1, size=len(shape))
        ph = rng.random()
        f += rng.normal() * np.sin(2 * np.pi * (sum(kk * g for kk, g in zip(k, grids)) + ph))
    return f


def reference_pipeline(oracle, f, h, axis):
    """run-compact.py:57-90 restated: permute -> RHS -> CR -> permute back."""
    perm = {2: (0, 1, 2), 1: (0, 2, 1), 0: (1, 2, 0)}[axis]
    back = {2: (0, 1, 2), 1: (0, 2, 1), 0: (2, 0, 1)}[axis]
    g = oracle.permute(f, perm) if axis != 2 else f
    n = g.shape[-1]
    x = oracle.cr_solve(oracle.compact_rhs(g, h), n, COMPACT)
    return oracle.permute(x, back) if axis != 2 else x


@pytest.mark.parametrize("axis", [0, 1, 2])
@pytest.mark.parametrize("shape", [(16, 16, 16), (32, 64, 128), (64, 32, 16)])
def test_fp64_matches_reference_pipeline(cuda, oracle, axis, shape):
    import ntk

    n = shape[axis]
    h = 1.0 / (n - 1)
    f = fourier_field(shape, seed=axis)
    t = torch.from_numpy(f).to(cuda)
    out = torch.empty_like(t)
    with ntk.Plan(n, 0, COMPACT) as p:
        p.compact_deriv(t, out, axis=axis, h=h)
        torch.cuda.synchronize()
    got = out.cpu().numpy()
    if all(s == shape[0] for s in shape):
        ref = reference_pipeline(oracle, f, h, axis)
    else:
        ref = oracle.banded_compact_deriv(f, h, axis)
    assert oracle.rel_err(got, ref) < FP64_TOL


@pytest.mark.parametrize("axis", [0, 1, 2])
@pytest.mark.parametrize("n", [32, 128, 512])
def test_refine_matches_fp64_oracle(cuda, oracle, axis, n):
    import ntk

    shape = [8, 8, 8]
    shape[axis] = n
    shape = tuple(shape)
    h = 1.0 / (n - 1)
    f = fourier_field(shape, seed=n + axis)
    t = torch.from_numpy(f).to(cuda)
    ref = oracle.banded_compact_deriv(f, h, axis)
    for prec, tol in (("fp32_refine", REFINE_TOL), ("fp32", 2e-5)):
        out = torch.empty_like(t)
        with ntk.Plan(n, 0, COMPACT, precision=prec) as p:
            p.compact_deriv(t, out, axis=axis, h=h)
            torch.cuda.synchronize()
        assert oracle.rel_err(out.cpu().numpy(), ref) < tol, prec


def test_golden_derivatives(cuda, oracle, golden):
    import ntk

    f = golden["deriv_f"]
    h = float(golden["deriv_h"])
    n = f.shape[0]
    t = torch.from_numpy(f).to(cuda)
    for axis, key in ((2, "deriv_dfdx"), (1, "deriv_dfdy")):
        for prec, tol in (("fp64", FP64_TOL), ("fp32_refine", REFINE_TOL)):
            out = torch.empty_like(t)
            with ntk.Plan(n, 0, COMPACT, precision=prec) as p:
                p.compact_deriv(t, out, axis=axis, h=h)
                torch.cuda.synchronize()
            assert oracle.rel_err(out.cpu().numpy(), golden[key]) < tol, (axis, prec)


def test_in_place_derivative(cuda, oracle):
    import ntk

    shape = (4, 8, 256)
    f = fourier_field(shape, seed=9)
    t = torch.from_numpy(f).to(cuda)
    with ntk.Plan(256, 0, COMPACT) as p:
        p.compact_deriv(t, t, axis=2, h=1.0 / 255)
        torch.cuda.synchronize()
    assert oracle.rel_err(t.cpu().numpy(), oracle.banded_compact_deriv(f, 1.0 / 255, 2)) < FP64_TOL


def test_linear_field_exact(cuda):
    """f = xyz: the compact scheme's derivative is exact
    (experiments/run-parallel-compact.py:44,90)."""
    import ntk

    n = 64
    x = np.linspace(0, 1, n)
    z, y, xx = np.meshgrid(x, x, x, indexing="ij")
    f = xx * y * z
    t = torch.from_numpy(f).to(cuda)
    for prec in ("fp64", "fp32_refine"):
        for axis, truth in ((2, y * z), (1, xx * z), (0, xx * y)):
            out = torch.empty_like(t)
            with ntk.Plan(n, 0, COMPACT, precision=prec) as p:
                p.compact_deriv(t, out, axis=axis, h=1.0 / (n - 1))
                torch.cuda.synchronize()
            np.testing.assert_allclose(out.cpu().numpy(), truth, rtol=0, atol=1e-12)


def test_analytic_derivative_of_sines(cuda):
    """experiments/run-compact.py:30-31,92-102: f = sin x + 2 sin y + 3 sin z
    on [0, 2pi]^3 -> cos x, 2 cos y, 3 cos z (the reference checks rtol 1e-1;
    the 4th-order scheme is far closer)."""
    import ntk

    n = 64
    L = 2 * np.pi
    g = np.linspace(0, L, n)
    z, y, x = np.meshgrid(g, g, g, indexing="ij")
    f = np.sin(x) + 2 * np.sin(y) + 3 * np.sin(z)
    t = torch.from_numpy(f).to(cuda)
    with ntk.Plan(n, 0, COMPACT) as p:
        for axis, truth in ((2, np.cos(x)), (1, 2 * np.cos(y)), (0, 3 * np.cos(z))):
            out = torch.empty_like(t)
            p.compact_deriv(t, out, axis=axis, h=L / (n - 1))
            torch.cuda.synchronize()
            assert np.abs(out.cpu().numpy() - truth).max() < 1e-4 * np.abs(truth).max()


def test_convergence_order(cuda):
    """experiments/run-compact-errors.py: f = sin(x)/x^3 on [2, 6]; the
    interior error falls ~16x per doubling (4th order), the boundary ~8x."""
    import ntk

    errs_mid, errs_bnd = [], []
    for n in (32, 64, 128, 256):
        x = np.linspace(2.0, 6.0, n)
        f = np.tile(np.sin(x) / x ** 3, (2, 2, 1))
        truth = (x * np.cos(x) - 3 * np.sin(x)) / x ** 4
        t = torch.from_numpy(np.ascontiguousarray(f)).to(cuda)
        out = torch.empty_like(t)
        with ntk.Plan(n, 0, COMPACT) as p:
            p.compact_deriv(t, out, axis=2, h=4.0 / (n - 1))
            torch.cuda.synchronize()
        d = out.cpu().numpy()[0, 0]
        errs_mid.append(abs(d[n // 2] - truth[n // 2]))
        errs_bnd.append(abs(d[0] - truth[0]))
    ratios_mid = [errs_mid[i] / errs_mid[i + 1] for i in range(3)]
    ratios_bnd = [errs_bnd[i] / errs_bnd[i + 1] for i in range(3)]
    assert min(ratios_mid) > 10, ratios_mid
    assert min(ratios_bnd) > 5, ratios_bnd


def test_bad_axis_extent_rejected(cuda):
    import ntk

    t = torch.zeros((4, 4, 16), dtype=torch.float64, device=cuda)
    with ntk.Plan(16, 0, COMPACT) as p:
        with pytest.raises(ValueError, match="extent"):
            p.compact_deriv(t, torch.empty_like(t), axis=1, h=0.1)
        with pytest.raises(ValueError):
            p.compact_deriv(t, t[:, :, 1:], axis=2, h=0.1)


# Two systems per warp (a CTA stages twice as many adjacent strided
# systems): same results on strided axes, also with padding (n = 300) and a
# partial last group; contiguous axes ignore the setting.  w = 16 stages 16
# systems per CTA with one system per warp and falls back to 8 warps with two.
@pytest.mark.parametrize("axis", [0, 1, 2])
@pytest.mark.parametrize("n,w", [(512, 8), (300, 4), (512, 4), (512, 16), (300, 16)])
def test_refine_two_systems_per_warp(cuda, oracle, axis, n, w):
    import ntk

    shape = [9, 7, 9]
    shape[axis] = n
    shape = tuple(shape)
    h = 1.0 / (n - 1)
    f = fourier_field(shape, seed=n + 3 * axis + w)
    t = torch.from_numpy(f).to(cuda)
    ref = oracle.banded_compact_deriv(f, h, axis)
    out1 = torch.empty_like(t)
    out2 = torch.empty_like(t)
    with ntk.Plan(n, 0, COMPACT, precision="fp32_refine") as p:
        p.set_tuning(refine_w=w, refine_spw=1)
        p.compact_deriv(t, out1, axis=axis, h=h)
        p.set_tuning(refine_spw=2)
        assert p.get_tuning()["refine_spw"] == 2
        p.compact_deriv(t, out2, axis=axis, h=h)
        torch.cuda.synchronize()
    assert oracle.rel_err(out2.cpu().numpy(), ref) < REFINE_TOL
    assert oracle.rel_err(out2.cpu().numpy(), out1.cpu().numpy()) < REFINE_TOL


# Compact derivatives along systems longer than 1024 rows (windows), each
# axis, out of place and in place.
@pytest.mark.parametrize("axis", [0, 1, 2])
@pytest.mark.parametrize("n", [2048, 1300])
def test_refine_long_derivative(cuda, oracle, axis, n):
    import ntk

    shape = [3, 5, 4]
    shape[axis] = n
    shape = tuple(shape)
    h = 1.0 / (n - 1)
    f = fourier_field(shape, seed=n + axis)
    ref = oracle.banded_compact_deriv(f, h, axis)
    t = torch.from_numpy(f).to(cuda)
    out = torch.empty_like(t)
    with ntk.Plan(n, 0, COMPACT, precision="fp32_refine") as p:
        p.compact_deriv(t, out, axis=axis, h=h)
        p.compact_deriv(t, t, axis=axis, h=h)  # in place
        torch.cuda.synchronize()
    assert oracle.rel_err(out.cpu().numpy(), ref) < REFINE_TOL
    assert oracle.rel_err(t.cpu().numpy(), ref) < REFINE_TOL


def test_cfg0_2d_field_x_direction(cuda, oracle):
    """The 2D workload exactly: a 256 x 256 field, derivative along x (256
    systems of n = 256), h = 1/255, f = 8 seeded Fourier modes (amplitudes
    N(0,1), integer wavenumbers 1-16), against the FP64 banded oracle
    (scipy solve_banded, experiments/run-compact.py:14-28) and the reference
    pipeline (RHS + CR restated)."""
    import ntk
    from ntk.workloads import fourier_field as ff

    n = 256
    h = 1.0 / (n - 1)
    f = ff((n, n), seed=0, device=cuda)
    fc = f.cpu().numpy()
    banded = oracle.banded_compact_deriv(fc[None], h, axis=2)[0]
    ref = reference_pipeline(oracle, fc[None], h, 2)[0]
    for prec, tol in (("fp64", FP64_TOL), ("fp32_refine", REFINE_TOL)):
        with ntk.Plan(n, 0, COMPACT, precision=prec) as p:
            out = torch.empty_like(f)
            p.compact_deriv(f, out, axis=1, h=h)
            torch.cuda.synchronize()
        x = out.cpu().numpy()
        assert oracle.rel_err(x, banded) < tol, (prec, oracle.rel_err(x, banded))
        assert oracle.rel_err(x, ref) < tol, (prec, oracle.rel_err(x, ref))
