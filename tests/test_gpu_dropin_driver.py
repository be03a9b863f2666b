"""The reference's compact-derivative driver (experiments/run-compact.py:47-90)
written with the drop-in modules, line for line: compute_rhs + solve for
d/dx; permute, compute_rhs, solve, permute back for d/dy and d/dz.  Its
output must match the oracle's restatement of the same pipeline and the
fused, permute-free ntk.Plan.compact_deriv."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

COMPACT = (1., 2., 1. / 4, 1., 1. / 4, 2., 1.)


def _oracle_pipeline(oracle, f, h, axis):
    perm = {2: None, 1: (0, 2, 1), 0: (1, 2, 0)}[axis]
    back = {2: None, 1: (0, 2, 1), 0: (2, 0, 1)}[axis]
    g = oracle.permute(f, perm) if perm else f
    x = oracle.cr_solve(oracle.compact_rhs(g, h), g.shape[-1], COMPACT)
    return oracle.permute(x, back) if back else x


@pytest.mark.parametrize("n", [32, 64])
def test_reference_driver_with_drop_ins(cuda, oracle, n):
    from compact.permute import permute
    from compact.rhs import compute_rhs
    from neato import NearToeplitzSolver

    import ntk

    rng = np.random.default_rng(n)
    f = rng.normal(size=(n, n, n))
    h = 1.0 / (n - 1)
    f_d = torch.from_numpy(f).to(cuda)
    rhs_d = torch.empty_like(f_d)
    tmp_d = torch.empty_like(f_d)
    solver = NearToeplitzSolver(n, n * n, COMPACT)  # experiments/run-compact.py:48

    # dfdx
    compute_rhs(f_d, rhs_d, h)
    solver.solve(rhs_d)
    dfdx = rhs_d.clone()
    # dfdy
    permute(f_d, tmp_d, (0, 2, 1))
    compute_rhs(tmp_d, rhs_d, h)
    solver.solve(rhs_d)
    dfdy = torch.empty_like(f_d)
    permute(rhs_d, dfdy, (0, 2, 1))
    # dfdz
    permute(f_d, tmp_d, (1, 2, 0))
    compute_rhs(tmp_d, rhs_d, h)
    solver.solve(rhs_d)
    dfdz = torch.empty_like(f_d)
    permute(rhs_d, dfdz, (2, 0, 1))
    torch.cuda.synchronize()

    fused = torch.empty_like(f_d)
    with ntk.Plan(n, 0, COMPACT) as p:
        for axis, got in ((2, dfdx), (1, dfdy), (0, dfdz)):
            ref = _oracle_pipeline(oracle, f, h, axis)
            assert oracle.rel_err(got.cpu().numpy(), ref) < 1e-13, axis
            p.compact_deriv(f_d, fused, axis=axis, h=h)
            torch.cuda.synchronize()
            assert oracle.rel_err(fused.cpu().numpy(), got.cpu().numpy()) < 1e-13, axis
