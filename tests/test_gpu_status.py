"""Range status of the FP32 / FP32+refinement paths (ntk_plan_status,
ntk_adi_status, ntk_batch_status).

The double-word arithmetic cannot hold |x| >= 2^128; a solve that meets such
an input completes (no fault, no hang) and raises a status bit that the
caller reads back with the status call, which returns NTK_ERR_RANGE and
clears the bit.  The reference has no counterpart: it validates only the
system size (neato.py:145)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

COMPACT = (1., 2., 1. / 4, 1., 1. / 4, 2., 1.)


@pytest.mark.parametrize("n", [64, 512, 2048])
@pytest.mark.parametrize("precision", ["fp32", "fp32_refine"])
def test_plan_status_reports_out_of_range_input(cuda, n, precision):
    import ntk
    from ntk import _lib

    rng = np.random.default_rng(n)
    f = torch.from_numpy(rng.normal(size=(2, 8, n))).to(cuda)
    out = torch.empty_like(f)
    with ntk.Plan(n, 0, COMPACT, precision=precision) as p:
        p.compact_deriv(f, out, axis=2, h=1.0 / (n - 1))
        assert p.status() == 0                          # in range: clean
        g = f.clone()
        g[1, 3, n // 2] = 2.0 ** 130                    # built on the CPU side, copied in
        p.compact_deriv(g, out, axis=2, h=1.0 / (n - 1))
        with pytest.raises(ntk.NtkError) as ei:
            p.status()
        assert ei.value.status == _lib.NTK_ERR_RANGE
        assert p.status() == 0                          # the read cleared it
        d = g.reshape(-1, n)[8:12].contiguous()     # holds the out-of-range row (flat row 11)
        with ntk.Plan(n, 4, COMPACT, precision=precision) as q:
            q.solve(d)
            assert q.status(raise_on_error=False) & _lib.NTK_STATUS_RANGE


def test_fp64_plan_status_is_always_clean(cuda):
    import ntk

    f = torch.full((1, 4, 64), 2.0 ** 200, dtype=torch.float64, device=cuda)
    out = torch.empty_like(f)
    with ntk.Plan(64, 0, COMPACT, precision="fp64") as p:
        p.compact_deriv(f, out, axis=2, h=1.0 / 63)
        assert p.status() == 0


def test_adi_status_reports_out_of_range_input(cuda):
    import ntk
    from ntk import _lib
    from ntk.workloads import gaussians_2d

    N = 256
    dx = 1.0 / (N - 1)
    u = gaussians_2d(N, seed=2, device=cuda)
    x, y = u.clone(), u.t().contiguous()
    with ntk.Adi(N, dx, dx * dx, precision="fp32_refine") as adi:
        adi.step(u, x, y)
        assert adi.status() == 0
        u[N // 2, N // 3] = 2.0 ** 140
        x, y = u.clone(), u.t().contiguous()
        adi.step(u, x, y)
        assert adi.status(raise_on_error=False) == _lib.NTK_STATUS_RANGE
        assert adi.status() == 0


def test_batch_status_reports_out_of_range_input(cuda):
    import ntk
    from ntk import _lib

    lengths = np.array([40, 700, 3])
    interior = np.tile([0.2, 1.0, 0.25], (3, 1))
    head = np.tile([[0.0, 1.5, 0.3], [0.2, 1.2, 0.3]], (3, 1, 1))
    tail = np.tile([[0.2, 1.1, 0.3], [0.3, 1.4, 0.0]], (3, 1, 1))
    with ntk.UnevenBatch(lengths, interior, head, tail, precision="fp32_refine") as bt:
        d = torch.from_numpy(np.random.default_rng(0).normal(size=bt.elements)).to(cuda)
        bt.solve(d)
        assert bt.status() == 0
        d[100] = -2.0 ** 129
        bt.solve(d)
        with pytest.raises(ntk.NtkError) as ei:
            bt.status()
        assert ei.value.status == _lib.NTK_ERR_RANGE
