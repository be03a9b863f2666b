"""ADI time stepping (experiments/run-adi.py:59-71) on the GPU against the
oracle: the reference's own pipeline restated on the CPU (stencil + CR +
transpose, oracle/ntk_oracle.c) and the same pipeline with a long-double
Thomas solve as the accuracy reference.  FP64 tolerance 1e-13 relative, or
the reference's own distance from the exact pipeline where that is larger.
(LAPACK's pivoting banded solve is not used as the reference here: on the
ADI matrices -- identity boundary rows next to rows scaled by 1/dx^2 -- it
drifts 5e-11 from the exact result within five steps.)"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

TOL = 1e-13


def _run_gpu(cuda, u, d_x, d_y, dx, dt, steps, graph):
    import ntk

    tu, tx, ty = [torch.from_numpy(np.ascontiguousarray(a)).to(cuda) for a in (u, d_x, d_y)]
    with ntk.Adi(u.shape[0], dx, dt) as adi:
        if graph:
            adi.run(tu, tx, ty, steps, graph=True)
        else:
            for _ in range(steps):
                adi.step(tu, tx, ty)
        torch.cuda.synchronize()
        seg = adi.segments
    return tu.cpu().numpy(), tx.cpu().numpy(), seg


def test_golden_three_steps(cuda, oracle, golden):
    """Three steps from run-adi.py's initial state, N = 32, vs the reference's
    own kernels (golden vectors)."""
    u0 = golden["adi_step_u0"]
    dx, dt = float(golden["adi_step_dx"]), float(golden["adi_step_dt"])
    u, _, _ = _run_gpu(cuda, u0, u0.copy(), u0.T.copy(), dx, dt, 3, graph=False)
    ub, xb, yb = u0.copy(), u0.copy(), u0.T.copy()
    for _ in range(3):
        oracle.adi_step_exact(ub, xb, yb, dx, dt)
    ref = golden["adi_step_u3"]
    # dt = 0.1 with dx = 1/31 (r = 48): the step amplifies rounding; the
    # reference's own pipeline is `spread` away from the exact one, ours must
    # be no further than 1.5x that
    spread = oracle.rel_err(ref, ub)
    assert oracle.rel_err(u, ub) <= max(TOL, 1.5 * spread)
    assert oracle.rel_err(u, ref) <= oracle.rel_err(u, ub) + spread + TOL


# FP64 paths: N = 64 segmented sweeps; 256 and 512 one whole-system window
# (r = 40 included: slow decay, carried exactly by the lane scan); 130, 300
# and 1000 first / middle / last windows with 36-row halos; 1024 at r = 40
# the segmented fallback (a 276-row halo leaves no room for windows).
@pytest.mark.parametrize("N,r,steps", [(64, 0.5, 10), (256, 0.5, 20), (256, 40.0, 5), (512, 0.5, 5),
                                       (130, 0.5, 5), (300, 0.5, 5), (1000, 0.5, 3), (1024, 40.0, 2)])
def test_adi_matches_oracle(cuda, oracle, N, r, steps):
    from ntk.workloads import gaussians_2d

    dx = 1.0 / (N - 1)
    dt = 2 * r * dx * dx
    u0 = gaussians_2d(N, seed=N, device="cpu").numpy()
    for graph in (False, True):
        u, d_x, seg = _run_gpu(cuda, u0, u0.copy(), u0.T.copy(), dx, dt, steps, graph)
        ub, xb, yb = u0.copy(), u0.copy(), u0.T.copy()
        for _ in range(steps):
            oracle.adi_step_exact(ub, xb, yb, dx, dt)
        assert oracle.rel_err(u, ub) < TOL, (graph, seg)
        assert oracle.rel_err(d_x[1:-1], xb[1:-1]) < TOL


def test_adi_reference_pipeline(cuda, oracle):
    """Against the reference pipeline itself (CR restated), N = 128."""
    from ntk.workloads import gaussians_2d

    N = 128
    dx = 1.0 / (N - 1)
    dt = dx * dx
    u0 = gaussians_2d(N, seed=3, device="cpu").numpy()
    u, _, _ = _run_gpu(cuda, u0, u0.copy(), u0.T.copy(), dx, dt, 10, graph=True)
    ur, xr, yr = u0.copy(), u0.copy(), u0.T.copy()
    ub, xb, yb = u0.copy(), u0.copy(), u0.T.copy()
    for _ in range(10):
        oracle.adi_step(ur, xr, yr, dx, dt)
        oracle.adi_step_exact(ub, xb, yb, dx, dt)
    assert oracle.rel_err(u, ur) <= max(TOL, oracle.rel_err(ur, ub) + TOL)


def test_full_size_windows(cuda, oracle):
    """2048^2, r = 0.5 (the 2D ADI heat workload): FP64 windows are chosen
    (5 per system) and 4 steps agree with the reference pipeline (its CR is
    exact to rounding for r = 0.5)."""
    from ntk.workloads import gaussians_2d

    N = 2048
    dx = 1.0 / (N - 1)
    dt = dx * dx
    u0 = gaussians_2d(N, seed=0, device="cpu").numpy()
    u, _, seg = _run_gpu(cuda, u0, u0.copy(), u0.T.copy(), dx, dt, 4, graph=True)
    assert seg == (440, 36, 5), seg
    ub, xb, yb = u0.copy(), u0.copy(), u0.T.copy()
    for _ in range(4):
        oracle.adi_step(ub, xb, yb, dx, dt)
    assert oracle.rel_err(u, ub) < TOL


def test_graph_replay_is_repeatable(cuda):
    import ntk
    from ntk.workloads import gaussians_2d

    N = 256
    dx = 1.0 / (N - 1)
    u0 = gaussians_2d(N, seed=1, device=cuda)
    outs = []
    with ntk.Adi(N, dx, dx * dx) as adi:
        for _ in range(2):
            u, dx_, dy_ = u0.clone(), u0.clone(), u0.t().contiguous()
            adi.run(u, dx_, dy_, 7, graph=True)
            torch.cuda.synchronize()
            outs.append(u.cpu())
    assert torch.equal(outs[0], outs[1])


def _run(cuda, u0, dx, dt, steps, precision, graph):
    import ntk

    tu = torch.from_numpy(np.ascontiguousarray(u0)).to(cuda)
    tx, ty = tu.clone(), tu.t().contiguous()
    with ntk.Adi(u0.shape[0], dx, dt, precision=precision) as adi:
        if graph:
            adi.run(tu, tx, ty, steps, graph=True)
        else:
            for _ in range(steps):
                adi.step(tu, tx, ty)
        torch.cuda.synchronize()
        seg = adi.segments
    return tu.cpu().numpy(), tx.cpu().numpy(), seg


# FP32 solve + double-word refinement per half step, over overlapping
# windows (or one whole-system window when N equals the window length):
# within 1e-12 of the FP64 path (the refinement tolerance), also
# for a non-power-of-two N, middle windows (N = 1000, 2048) and a slowly
# decaying, badly conditioned matrix (r = 40, two sweeps).
@pytest.mark.parametrize("N,r,steps", [(128, 0.5, 5), (256, 0.5, 10), (300, 0.5, 5), (512, 0.5, 5),
                                       (1000, 0.5, 4), (512, 40.0, 3), (2048, 0.5, 3)])
def test_adi_refine_matches_fp64(cuda, oracle, N, r, steps):
    from ntk.workloads import gaussians_2d

    dx = 1.0 / (N - 1)
    dt = 2 * r * dx * dx
    u0 = gaussians_2d(N, seed=N + 1, device="cpu").numpy()
    u64, x64, _ = _run(cuda, u0, dx, dt, steps, "fp64", graph=True)
    for graph in (False, True):
        ur, xr, seg = _run(cuda, u0, dx, dt, steps, "fp32_refine", graph)
        L, H, P = seg
        assert L > 0 and P >= 1 and (P == 1 or H >= 8)
        assert oracle.rel_err(ur, u64) < 1e-12, (graph, seg, oracle.rel_err(ur, u64))
        assert oracle.rel_err(xr[1:-1], x64[1:-1]) < 1e-12
    if N <= 512:
        ub, xb, yb = u0.copy(), u0.copy(), u0.T.copy()
        for _ in range(steps):
            oracle.adi_step_exact(ub, xb, yb, dx, dt)
        assert oracle.rel_err(ur, ub) < 1e-12


def test_adi_fp32_only_error_is_reported_scale(cuda, oracle):
    """Without the refinement sweep the windows give FP32-level results."""
    from ntk.workloads import gaussians_2d

    N = 512
    dx = 1.0 / (N - 1)
    dt = dx * dx
    u0 = gaussians_2d(N, seed=5, device="cpu").numpy()
    u64, _, _ = _run(cuda, u0, dx, dt, 3, "fp64", graph=False)
    u32, _, _ = _run(cuda, u0, dx, dt, 3, "fp32", graph=False)
    e = oracle.rel_err(u32, u64)
    assert 1e-10 < e < 1e-4, e


def test_adi_refine_rejects_slow_decay_windows(cuda):
    """r = 40 at N = 300: the halo the 2^-56 truncation needs leaves no
    central rows in a 256-row window, and systems this short have no
    partitioned fallback (N > 512 has one, tests/test_gpu_spike.py); the
    plan says so instead of running."""
    import ntk

    N = 300
    dx = 1.0 / (N - 1)
    with pytest.raises(Exception) as ei:
        ntk.Adi(N, dx, 80 * dx * dx, precision="fp32_refine")
    assert "NTK_FP64" in str(ei.value)


def test_adi_refine_needs_n_128(cuda):
    import ntk
    from ntk import _lib

    with pytest.raises(Exception) as ei:
        ntk.Adi(64, 1.0 / 63, 1.0 / 63 ** 2, precision="fp32_refine")
    assert "128" in str(ei.value)
    assert _lib.PRECISIONS["fp32_refine"] != _lib.PRECISIONS["fp64"]


@pytest.fixture(scope="module")
def adi_2048_100_steps(oracle):
    """The benchmarked ADI workload: 2048^2, r = 0.5, the seeded Gaussian
    initial condition, 100 steps of the long-double ADI pipeline
    (experiments/run-adi.py:59-71 with an exact Thomas solve)."""
    from ntk.workloads import gaussians_2d

    N = 2048
    dx = 1.0 / (N - 1)
    dt = 2 * 0.5 * dx * dx
    u0 = gaussians_2d(N, seed=0, device="cpu").numpy()
    ub, xb, yb = u0.copy(), u0.copy(), u0.T.copy()
    for _ in range(100):
        oracle.adi_step_exact(ub, xb, yb, dx, dt)
    return u0, ub, xb, dx, dt


@pytest.mark.parametrize("precision,tol", [("fp64", TOL), ("fp32_refine", 1e-12)])
def test_adi_2048_hundred_steps_in_a_graph(cuda, oracle, adi_2048_100_steps, precision, tol):
    """The benchmark's own run (100 steps replayed as one CUDA graph) stays
    within the tolerance of the exact pipeline over all 100 steps."""
    u0, ub, xb, dx, dt = adi_2048_100_steps
    u, d_x, seg = _run(cuda, u0, dx, dt, 100, precision, graph=True)
    assert oracle.rel_err(u, ub) < tol, (precision, seg, oracle.rel_err(u, ub))
    assert oracle.rel_err(d_x[1:-1], xb[1:-1]) < tol
