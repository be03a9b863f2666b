"""Parity with the reference's own CUDA kernels, compiled for this GPU from
the reference's source strings (oracle/ref_gpu.cu, built by
__graft_entry__.build() when the rendered source is present) and launched
with the reference's grid/block shapes.  Skipped where that build is absent.

Criterion (the project's): FP64 within 1e-13 relative of the reference's
NearToeplitzSolver output; FP32+refine within 1e-12."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

COMPACT = (1., 2., 1. / 4, 1., 1. / 4, 2., 1.)


@pytest.fixture(scope="module")
def ref_gpu(cuda, oracle):
    R = oracle.ref_gpu()
    if R is None:
        pytest.skip("reference kernels were not built (oracle/_ref absent)")
    return R


class RefSolver:
    """NearToeplitzSolver (neato.py:129-197) on the reference's own kernel."""

    def __init__(self, R, oracle, n, nrhs, coeffs, device):
        self.R, self.n, self.nrhs, self.coeffs = R, n, nrhs, coeffs
        self.arrs = [torch.from_numpy(np.ascontiguousarray(a)).to(device) for a in oracle.precompute(n, coeffs)]

    def solve(self, x):
        co = self.coeffs
        rc = self.R.ntkref_gpu_cr(self.n, self.nrhs, *[a.data_ptr() for a in self.arrs], co[0], co[1], co[2],
                                  co[3], co[4], x.data_ptr(), torch.cuda.current_stream().cuda_stream)
        assert rc == 0


@pytest.mark.parametrize("L", [2, 5, 8, 9, 11])
def test_solve_vs_reference_kernel(ref_gpu, oracle, cuda, L):
    import ntk

    n = 1 << L
    nrhs = 1024
    d = torch.from_numpy(np.random.default_rng(L).normal(size=(nrhs, n))).to(cuda)
    ref = d.clone()
    RefSolver(ref_gpu, oracle, n, nrhs, COMPACT, cuda).solve(ref)
    precs = (("fp64", 1e-13), ("fp32_refine", 1e-12))
    for prec, tol in precs:
        x = d.clone()
        with ntk.Plan(n, nrhs, COMPACT, precision=prec) as p:
            p.solve(x)
        torch.cuda.synchronize()
        assert oracle.rel_err(x.cpu().numpy(), ref.cpu().numpy()) < tol, prec


@pytest.mark.parametrize("axis", [0, 1, 2])
def test_compact_derivative_vs_reference_kernels(ref_gpu, oracle, cuda, axis):
    """run-compact.py:57-90 on the reference kernels (permute + RHS + CR +
    permute) against the fused ntk derivative, 128^3."""
    import ntk

    n = 128
    h = 1.0 / (n - 1)
    rng = np.random.default_rng(axis)
    g = np.linspace(0, 1, n)
    z, y, x = np.meshgrid(g, g, g, indexing="ij")
    f = np.zeros((n, n, n))
    for _ in range(8):
        k = rng.integers(1, 17, size=3)
        f += rng.normal() * np.sin(2 * np.pi * (k[0] * x + k[1] * y + k[2] * z + rng.random()))
    ft = torch.from_numpy(f).to(cuda)
    s = torch.cuda.current_stream().cuda_stream
    st = [n * n, n, 1]

    def perm(a, b, p):
        ss = [st[i] for i in p]
        assert ref_gpu.ntkref_gpu_permute(a.data_ptr(), b.data_ptr(), n, n, n, ss[0], ss[1], ss[2], s) == 0

    tmp = torch.empty_like(ft)
    ref = torch.empty_like(ft)
    solver = RefSolver(ref_gpu, oracle, n, n * n, COMPACT, cuda)
    if axis == 2:
        assert ref_gpu.ntkref_gpu_compact_rhs(ft.data_ptr(), ref.data_ptr(), n, n, n, h, s) == 0
        solver.solve(ref)
    else:
        p_in, p_out = ((0, 2, 1), (0, 2, 1)) if axis == 1 else ((1, 2, 0), (2, 0, 1))
        g1 = torch.empty_like(ft)
        perm(ft, g1, p_in)
        assert ref_gpu.ntkref_gpu_compact_rhs(g1.data_ptr(), tmp.data_ptr(), n, n, n, h, s) == 0
        solver.solve(tmp)
        perm(tmp, ref, p_out)
    for prec, tol in (("fp64", 1e-13), ("fp32_refine", 1e-12)):
        out = torch.empty_like(ft)
        with ntk.Plan(n, 0, COMPACT, precision=prec) as p:
            p.compact_deriv(ft, out, axis=axis, h=h)
        torch.cuda.synchronize()
        assert oracle.rel_err(out.cpu().numpy(), ref.cpu().numpy()) < tol, prec


@pytest.fixture(scope="module")
def field_512(cuda):
    import ntk  # noqa: F401  (loads the library before the first launch)
    from ntk.workloads import fourier_field

    return fourier_field((512, 512, 512), seed=0, device=cuda)


@pytest.mark.parametrize("axis", [0, 1, 2])
def test_compact_derivative_vs_reference_kernels_512cube(ref_gpu, oracle, cuda, field_512, axis):
    """The benchmark's workload at full size (run-compact.py:47-90 on a 512^3
    field, 262144 systems of n = 512 per axis) on the reference's kernels,
    every row compared with the ntk derivative in both precisions."""
    import ntk

    n = 512
    h = 1.0 / (n - 1)
    ft = field_512
    s = torch.cuda.current_stream().cuda_stream
    st = [n * n, n, 1]
    ref = torch.empty_like(ft)
    tmp = torch.empty_like(ft)
    solver = RefSolver(ref_gpu, oracle, n, n * n, COMPACT, cuda)
    if axis == 2:
        assert ref_gpu.ntkref_gpu_compact_rhs(ft.data_ptr(), ref.data_ptr(), n, n, n, h, s) == 0
        solver.solve(ref)
    else:
        p_in, p_out = ((0, 2, 1), (0, 2, 1)) if axis == 1 else ((1, 2, 0), (2, 0, 1))
        ss = [st[i] for i in p_in]
        assert ref_gpu.ntkref_gpu_permute(ft.data_ptr(), ref.data_ptr(), n, n, n, ss[0], ss[1], ss[2], s) == 0
        assert ref_gpu.ntkref_gpu_compact_rhs(ref.data_ptr(), tmp.data_ptr(), n, n, n, h, s) == 0
        solver.solve(tmp)
        ss = [st[i] for i in p_out]
        assert ref_gpu.ntkref_gpu_permute(tmp.data_ptr(), ref.data_ptr(), n, n, n, ss[0], ss[1], ss[2], s) == 0
    del tmp
    scale = ref.abs().max()
    for prec, tol in (("fp64", 1e-13), ("fp32_refine", 1e-12)):
        out = torch.empty_like(ft)
        with ntk.Plan(n, 0, COMPACT, precision=prec) as p:
            p.compact_deriv(ft, out, axis=axis, h=h)
        torch.cuda.synchronize()
        err = ((out - ref).abs().max() / scale).item()
        assert err < tol, (prec, err)
        del out
