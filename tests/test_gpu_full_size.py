"""The benchmark's workload at full size: dfdx, dfdy, dfdz of a 512^3 FP64
field (3 x 262144 systems of n = 512, experiments/run-compact.py:47-90).

The CPU oracle cannot solve the whole field in a test's time, so parity at
this size is checked through properties that do not depend on size:
* FP32 + refine against the FP64 GPU solve, every row (1e-12 relative);
* the FP64 GPU solve against the oracle's banded solve on sampled lines of
  every axis (1e-13);
* linearity: D(f + 2g) = D(f) + 2 D(g) (1e-12, both precisions);
* exactness for a trilinear field: d(xyz)/dx = yz to the stencils' rounding
  (the compact scheme is exact for it, experiments/run-parallel-compact.py:44,90)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

N = 512
H = 1.0 / (N - 1)


@pytest.fixture(scope="module")
def fields(cuda):
    import ntk  # noqa: F401  (loads the library before the first launch)
    from ntk.workloads import fourier_field

    f = fourier_field((N, N, N), seed=0, device=cuda)
    g = fourier_field((N, N, N), seed=1, device=cuda)
    return f, g


def _deriv(precision, f, axis):
    import ntk
    from ntk.workloads import COMPACT_COEFFS

    out = torch.empty_like(f)
    with ntk.Plan(N, 0, COMPACT_COEFFS, precision=precision) as p:
        p.compact_deriv(f, out, axis=axis, h=H)
        torch.cuda.synchronize()
    return out


def _max_rel(a, b):
    return ((a - b).abs().max() / b.abs().max()).item()


@pytest.mark.parametrize("axis", [0, 1, 2])
def test_full_size_refine_and_fp64_against_oracle(oracle, fields, axis):
    f, _ = fields
    d64 = _deriv("fp64", f, axis)
    dref = _deriv("fp32_refine", f, axis)
    assert _max_rel(dref, d64) < 1e-12
    # sampled lines along the axis: 64 (i, j) positions of the other two axes
    rng = np.random.default_rng(axis)
    other = [a for a in range(3) if a != axis]
    pos = rng.integers(0, N, size=(64, 2))
    idx = [slice(None)] * 3
    lines_f, lines_d = [], []
    for i, j in pos:
        idx[other[0]], idx[other[1]] = int(i), int(j)
        lines_f.append(f[tuple(idx)].cpu().numpy())
        lines_d.append(d64[tuple(idx)].cpu().numpy())
    lf = np.stack(lines_f)  # (64, N), the solved axis last
    ref = oracle.banded_compact_deriv(lf, H, 1)
    assert oracle.rel_err(np.stack(lines_d), ref) < 1e-13


@pytest.mark.parametrize("precision", ["fp64", "fp32_refine"])
def test_full_size_linearity(fields, precision):
    f, g = fields
    for axis in (0, 1, 2):
        lhs = _deriv(precision, f + 2.0 * g, axis)
        rhs = _deriv(precision, f, axis) + 2.0 * _deriv(precision, g, axis)
        assert _max_rel(lhs, rhs) < 1e-12, axis


@pytest.mark.parametrize("precision", ["fp64", "fp32_refine"])
def test_full_size_trilinear_exact(cuda, precision):
    x = torch.linspace(1.0, 2.0, N, dtype=torch.float64, device=cuda)
    f = x.view(N, 1, 1) * x.view(1, N, 1) * x.view(1, 1, N)  # z * y * x
    h = 1.0 / (N - 1)
    # the difference stencils cancel: a rounding of f (max|f| = 8) is
    # amplified by 1/h against the derivative (max|f'| = 4), a relative floor
    # of eps * 8 / (4 h) = 2.3e-13 at h = 1/511; 32x that (7.3e-12) covers
    # the three stencils and the solve (measured 1.02e-12 on GB300, both
    # precisions)
    eps = np.finfo(np.float64).eps
    tol = 32 * eps * 8.0 / (h * 4.0)
    import ntk
    from ntk.workloads import COMPACT_COEFFS

    out = torch.empty_like(f)
    with ntk.Plan(N, 0, COMPACT_COEFFS, precision=precision) as p:
        for axis in (0, 1, 2):
            p.compact_deriv(f, out, axis=axis, h=h)
            shape = [1, 1, 1]
            shape[axis] = N
            truth = f / x.view(shape)  # the product of the other two coordinates
            assert _max_rel(out, truth) < tol, axis
