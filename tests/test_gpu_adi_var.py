"""ADI with per-line coefficients (ntk_adi_var_*, the generalisation of the
reference's single ADI matrix, run-adi.py:50-53, to one near-Toeplitz
system per line) against the oracle's long-double restatement of the same
step (oracle.adi_step_var_exact); with unit coefficients it is the
reference's step (oracle.adi_step_exact).  Tolerances: FP64 1e-13, FP32 +
refinement 1e-12."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _run(cuda, u0, dx, dt, kx, ky, steps, precision):
    import ntk

    u = torch.from_numpy(np.ascontiguousarray(u0)).to(cuda)
    x, y = u.clone(), u.t().contiguous()
    with ntk.AdiVar(u0.shape[0], dx, dt, kx, ky, precision=precision) as adi:
        for _ in range(steps):
            adi.step(u, x, y)
        torch.cuda.synchronize()
        assert adi.status() == 0
    return u.cpu().numpy(), x.cpu().numpy(), y.cpu().numpy()


@pytest.mark.parametrize("N", [64, 256])
def test_unit_coefficients_reproduce_the_reference_step(cuda, oracle, N):
    from ntk.workloads import gaussians_2d

    dx = 1.0 / (N - 1)
    dt = dx * dx
    u0 = gaussians_2d(N, seed=N, device="cpu").numpy()
    one = np.ones(N)
    u, _, _ = _run(cuda, u0, dx, dt, one, one, 3, "fp64")
    ub, xb, yb = u0.copy(), u0.copy(), u0.T.copy()
    for _ in range(3):
        oracle.adi_step_exact(ub, xb, yb, dx, dt)
    assert oracle.rel_err(u, ub) < 1e-13


@pytest.mark.parametrize("N,steps", [(130, 4), (300, 3), (1000, 2)])
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-13), ("fp32_refine", 1e-12)])
def test_per_line_coefficients_match_the_oracle(cuda, oracle, N, steps, precision, tol):
    from ntk.workloads import gaussians_2d

    rng = np.random.default_rng(N)
    dx = 1.0 / (N - 1)
    dt = dx * dx
    kx = rng.uniform(0.5, 2.0, size=N)
    ky = rng.uniform(0.5, 2.0, size=N)
    u0 = gaussians_2d(N, seed=N + 7, device="cpu").numpy()
    u, x, y = _run(cuda, u0, dx, dt, kx, ky, steps, precision)
    ub, xb, yb = u0.copy(), u0.copy(), u0.T.copy()
    for _ in range(steps):
        oracle.adi_step_var_exact(ub, xb, yb, dx, dt, kx, ky)
    assert oracle.rel_err(u, ub) < tol, oracle.rel_err(u, ub)
    assert oracle.rel_err(x[1:-1], xb[1:-1]) < tol
    assert oracle.rel_err(y[1:-1], yb[1:-1]) < tol


def test_rejects_non_finite_coefficients(cuda):
    import ntk

    k = np.ones(16)
    k[3] = np.nan
    with pytest.raises(ValueError, match="finite"):
        ntk.AdiVar(16, 0.1, 0.01, k, np.ones(16))
