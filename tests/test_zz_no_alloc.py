"""ntk_adi_step_static: the ADI step for callers that cannot allocate device
memory (a fixed, pre-sized memory budget, hosts with no device allocator,
libraries limited to the buffers they are handed).  It keeps its work array
in a fixed static device array instead of a plan's cudaMalloc'd one.

Called through the C ABI and compared with the plan-based ntk_adi_step on
two calls in a row (the static array keeps the previous call's contents, so
the second call checks that nothing stale leaks in).  Tolerance: 1e-13
relative, the FP64 tolerance of the other tests.  This file is collected
last so a failure here cannot hide the results of the others."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

TOL = 1e-13


def _rel(a, b):
    a = a.double().cpu().numpy()
    b = b.double().cpu().numpy()
    den = np.abs(b).max()
    return float(np.abs(a - b).max() / den) if den > 0 else float(np.abs(a - b).max())


@pytest.mark.parametrize("N,r", [(256, 0.5), (512, 0.5), (96, 40.0)])
def test_static_step_matches_planned_step(cuda, N, r):
    import ntk
    from ntk import _lib
    from ntk.workloads import gaussians_2d

    lib = _lib.load()
    dx = 1.0 / (N - 1)
    dt = 2 * r * dx * dx
    u0 = gaussians_2d(N, seed=N, device=cuda)
    u_a, x_a, y_a = u0.clone(), u0.clone(), u0.t().contiguous()
    u_b, x_b, y_b = u0.clone(), u0.clone(), u0.t().contiguous()
    stream = torch.cuda.current_stream().cuda_stream
    with ntk.Adi(N, dx, dt) as adi:
        for _ in range(2):
            adi.step(u_a, x_a, y_a)
            rc = lib.ntk_adi_step_static(N, dx, dt, u_b.data_ptr(), x_b.data_ptr(), y_b.data_ptr(), stream)
            assert rc == 0, _lib.last_error()
            torch.cuda.synchronize()
            assert _rel(u_b, u_a) <= TOL
            assert _rel(x_b[1:-1], x_a[1:-1]) <= TOL


def test_static_steps_match_the_oracle_across_a_time_step_change(cuda, oracle):
    """Two static steps in a row with different time steps (r = 0.5, then
    r = 2), checked against the long-double ADI pipeline of the oracle after
    each call: the second call must use its own factor tables, not the ones
    the first call left in the static array."""
    from ntk import _lib
    from ntk.workloads import gaussians_2d

    lib = _lib.load()
    N = 256
    dx = 1.0 / (N - 1)
    u0 = gaussians_2d(N, seed=11, device=cuda)
    u, x, y = u0.clone(), u0.clone(), u0.t().contiguous()
    ub = u0.cpu().numpy().copy()
    xb, yb = ub.copy(), ub.T.copy()
    stream = torch.cuda.current_stream().cuda_stream
    for r in (0.5, 2.0):
        dt = 2 * r * dx * dx
        rc = lib.ntk_adi_step_static(N, dx, dt, u.data_ptr(), x.data_ptr(), y.data_ptr(), stream)
        assert rc == 0, _lib.last_error()
        torch.cuda.synchronize()
        oracle.adi_step_exact(ub, xb, yb, dx, dt)
        assert oracle.rel_err(u.cpu().numpy(), ub) <= TOL, r
        assert oracle.rel_err(x.cpu().numpy()[1:-1], xb[1:-1]) <= TOL, r


def test_static_step_rejects_sizes_beyond_its_array(cuda):
    from ntk import _lib

    lib = _lib.load()
    n = lib_max = 512
    big = torch.zeros((n + 1, n + 1), dtype=torch.float64, device=cuda)
    rc = lib.ntk_adi_step_static(lib_max + 1, 0.01, 0.01, big.data_ptr(), big.data_ptr(), big.data_ptr(), None)
    assert rc == _lib.NTK_ERR_INVALID
    assert "512" in _lib.last_error()
