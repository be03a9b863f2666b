"""FP32 + refinement for long systems whose LU factors decay too slowly for
overlapping windows: exact 512-row partitions coupled by a reduced system
(ntk_spike.cu, the one-GPU form of the reference's partitioned solve,
parallelcompact/reduced.py:135-196, sum.py:8-31, misc.py:21-46), used by
plans with n > 1024 where the windows do not apply and by the ADI step at
large dt / dx^2.

Tolerances (normwise, max|x - ref| / max|ref|): FP32 + refinement 1e-12
against the long-double solve of the same systems (oracle.exact_solve); FP32
alone below 1e-3 (these matrices have condition numbers of ~600)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

# |l| -> 0.92 (beyond the windows' 0.9 limit); the second set has its own
# boundary rows (row 0: b = 2, c = 1; row n-1: a = 1, b = 2)
SLOW = (1.0, 0.0, 1.0, -2.007, 1.0, 0.0, 1.0)
SLOW_ENDS = (2.0, 1.0, 1.0, -2.007, 1.0, 1.0, 2.0)


def _plan_solve(cuda, n, nrhs, co, d, precision, sweeps):
    import ntk

    t = torch.from_numpy(np.ascontiguousarray(d)).to(cuda)
    with ntk.Plan(n, nrhs, co, precision=precision, refine_sweeps=sweeps) as p:
        p.solve(t)
        torch.cuda.synchronize()
        assert p.status() == 0
    return t.cpu().numpy()


@pytest.mark.parametrize("n", [1025, 1500, 2048, 3000, 4096])
@pytest.mark.parametrize("co", [SLOW, SLOW_ENDS])
def test_partitioned_refine_matches_exact(cuda, oracle, n, co):
    rng = np.random.default_rng(n)
    nrhs = 96
    d = rng.standard_normal((nrhs, n)) * 10.0 ** rng.uniform(-3, 3, size=(nrhs, 1))
    x = _plan_solve(cuda, n, nrhs, co, d, "fp32_refine", 2)
    ref = oracle.exact_solve(d, n, co)
    for s in range(nrhs):
        assert oracle.rel_err(x[s], ref[s]) < 1e-12, (s, oracle.rel_err(x[s], ref[s]))


def test_partitioned_one_sweep_and_fp32(cuda, oracle):
    n, nrhs = 2048, 32
    rng = np.random.default_rng(3)
    d = rng.standard_normal((nrhs, n))
    ref = oracle.exact_solve(d, n, SLOW)
    x1 = _plan_solve(cuda, n, nrhs, SLOW, d, "fp32_refine", 1)
    x0 = _plan_solve(cuda, n, nrhs, SLOW, d, "fp32", 1)
    e1, e0 = oracle.rel_err(x1, ref), oracle.rel_err(x0, ref)
    assert e0 < 1e-3 and e1 < 1e-7 and e1 < e0 * 1e-2, (e0, e1)


def test_partitioned_strided_out_of_place(cuda, oracle):
    """Systems as the columns of an (n, ncols) array, written to another
    buffer (ntk_solve_strided: element stride ncols)."""
    import ntk

    n, ncols = 2048, 40
    rng = np.random.default_rng(11)
    f = rng.standard_normal((n, ncols))
    src = torch.from_numpy(f).to(cuda)
    dst = torch.full_like(src, np.nan)
    with ntk.Plan(n, ncols, SLOW_ENDS, precision="fp32_refine", refine_sweeps=2) as p:
        p.solve_strided(src, dst, ncols, ncols, 1, 0, ncols)
        torch.cuda.synchronize()
    ref = oracle.exact_solve(f.T.copy(), n, SLOW_ENDS).T
    assert oracle.rel_err(dst.cpu().numpy(), ref) < 1e-12
    assert np.array_equal(src.cpu().numpy(), f)


def test_partitioned_rejects_three_sweeps(cuda):
    import ntk

    with pytest.raises(Exception, match="2 refinement sweeps"):
        ntk.Plan(2048, 4, SLOW, precision="fp32_refine", refine_sweeps=3)


def _adi(cuda, u0, dx, dt, steps, precision, graph):
    import ntk

    N = u0.shape[0]
    u = torch.from_numpy(u0.copy()).to(cuda)
    x = u.clone()
    y = u.t().contiguous()
    with ntk.Adi(N, dx, dt, precision=precision) as adi:
        seg = adi.segments
        if graph:
            adi.run(u, x, y, steps, graph=True)
        else:
            for _ in range(steps):
                adi.step(u, x, y)
        torch.cuda.synchronize()
        if precision != "fp64":
            assert adi.status() == 0
    return u.cpu().numpy(), x.cpu().numpy(), y.cpu().numpy(), seg


@pytest.mark.parametrize("N", [1000, 2048])
def test_adi_large_r_partitions_match_fp64(cuda, oracle, N):
    """r = 40: the windows' halo would leave too few central rows; the step
    runs the reference's kernel sequence with exact partitions instead."""
    from ntk.workloads import gaussians_2d

    dx = 1.0 / (N - 1)
    dt = 80 * dx * dx
    u0 = gaussians_2d(N, seed=N + 3, device="cpu").numpy()
    u64, x64, _, _ = _adi(cuda, u0, dx, dt, 3, "fp64", graph=False)
    for graph in (False, True):
        ur, xr, yr, seg = _adi(cuda, u0, dx, dt, 3, "fp32_refine", graph)
        assert seg == (512, 0, (N + 511) // 512), seg
        assert oracle.rel_err(ur, u64) < 1e-12, (graph, oracle.rel_err(ur, u64))
        assert oracle.rel_err(xr[1:-1], x64[1:-1]) < 1e-12
        # d_y is not written; u's boundary columns keep their values
        assert np.array_equal(yr, u0.T)
        assert np.array_equal(ur[:, 0], u0[:, 0]) and np.array_equal(ur[:, -1], u0[:, -1])
    uf, _, _, _ = _adi(cuda, u0, dx, dt, 3, "fp32", graph=False)
    assert oracle.rel_err(uf, u64) < 1e-4


@pytest.mark.parametrize("N", [1000, 2048])
def test_adi_large_r_matches_long_double_oracle(cuda, oracle, N):
    from ntk.workloads import gaussians_2d

    dx = 1.0 / (N - 1)
    dt = 80 * dx * dx
    u0 = gaussians_2d(N, seed=2, device="cpu").numpy()
    ur, xr, _, _ = _adi(cuda, u0, dx, dt, 2, "fp32_refine", graph=False)
    ub, xb, yb = u0.copy(), u0.copy(), u0.T.copy()
    for _ in range(2):
        oracle.adi_step_exact(ub, xb, yb, dx, dt)
    assert oracle.rel_err(ur, ub) < 1e-12
