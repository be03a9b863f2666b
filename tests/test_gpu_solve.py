"""In-place batched solves (NearToeplitzSolver.solve, neato.py:168-197) on the
GPU through the C ABI, against the oracle.

Tolerances: FP64 within 1e-13 relative (normwise, max|x-ref|/max|ref|) of
the reference's own CR output; FP32+refine within 1e-12 of the FP64 banded
solve; FP32 alone within 2e-6."""
import numpy as np
import pytest
import torch

from golden.make_golden import COEFF_SETS

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-13
REFINE_TOL = 1e-12


def _solve(cuda, n, nrhs, coeffs, d, precision="fp64", sweeps=1):
    import ntk

    t = torch.from_numpy(np.ascontiguousarray(d)).to(cuda)
    with ntk.Plan(n, nrhs, coeffs, precision=precision, refine_sweeps=sweeps) as p:
        p.solve(t)
        torch.cuda.synchronize()
    return t.cpu().numpy()


def _banded(oracle, n, coeffs, d):
    """FP64 ground truth: the near-Toeplitz systems solved in long double
    (LAPACK's pivoting banded solve loses up to ~6e-13 on the ADI tuples)."""
    return oracle.exact_solve(d, n, coeffs)


@pytest.mark.parametrize("cname", ["compact", "dominant"])
@pytest.mark.parametrize("L", range(2, 12))
def test_fp64_matches_reference_cr(cuda, oracle, cname, L):
    n = 1 << L
    co = COEFF_SETS[cname]
    nrhs = max(1, 4096 // n)
    d = np.random.default_rng(L).normal(size=(nrhs, n))
    x = _solve(cuda, n, nrhs, co, d)
    ref = oracle.cr_solve(d, n, co)
    assert oracle.rel_err(x, ref) < FP64_TOL


@pytest.mark.parametrize("cname", ["adi256", "adi2048_r05"])
@pytest.mark.parametrize("L", [3, 5, 8, 11])
def test_fp64_adi_coefficients(cuda, oracle, cname, L):
    """ADI coefficient tuples: our solve is within 1e-13 of the exact solve,
    and within the reference CR's own deviation of the reference output."""
    n = 1 << L
    co = COEFF_SETS[cname]
    d = np.random.default_rng(L).normal(size=(8, n))
    x = _solve(cuda, n, 8, co, d)
    xb = _banded(oracle, n, co, d)
    ref = oracle.cr_solve(d, n, co)
    assert oracle.rel_err(x, xb) < FP64_TOL
    assert oracle.rel_err(x, ref) <= oracle.rel_err(ref, xb) + FP64_TOL


def test_golden_cr_outputs(cuda, oracle, golden):
    for cname, co in COEFF_SETS.items():
        for L in range(2, 11):
            n = 1 << L
            key = "cr_%s_n%d_in" % (cname, n)
            if key not in golden:
                continue
            d = golden[key]
            x = _solve(cuda, n, d.shape[0], co, d)
            ref = golden["cr_%s_n%d_out" % (cname, n)]
            xb = _banded(oracle, n, co, d)
            assert oracle.rel_err(x, ref) <= oracle.rel_err(ref, xb) + FP64_TOL, (cname, n)


@pytest.mark.parametrize("n", [3, 5, 7, 33, 100, 333, 1000, 3000, 8192])
def test_fp64_any_length(cuda, oracle, n):
    """Beyond the reference (powers of two <= 2048 only): any n >= 3."""
    co = COEFF_SETS["dominant"]
    d = np.random.default_rng(n).normal(size=(37, n))
    x = _solve(cuda, n, 37, co, d)
    assert oracle.rel_err(x, _banded(oracle, n, co, d)) < FP64_TOL


@pytest.mark.parametrize("n", [4, 16, 64, 100, 256, 512, 700, 1024])
@pytest.mark.parametrize("sweeps", [1, 2])
def test_refine_matches_banded(cuda, oracle, n, sweeps):
    co = COEFF_SETS["compact"]
    d = np.random.default_rng(n + sweeps).normal(size=(50, n))
    x = _solve(cuda, n, 50, co, d, precision="fp32_refine", sweeps=sweeps)
    assert oracle.rel_err(x, _banded(oracle, n, co, d)) < REFINE_TOL


@pytest.mark.parametrize("cname", ["dominant", "adi256"])
@pytest.mark.parametrize("n", [64, 512, 1000])
def test_refine_general_coefficients(cuda, oracle, cname, n):
    co = COEFF_SETS[cname]
    d = np.random.default_rng(n).normal(size=(20, n))
    x = _solve(cuda, n, 20, co, d, precision="fp32_refine", sweeps=2)
    assert oracle.rel_err(x, _banded(oracle, n, co, d)) < REFINE_TOL


def test_fp32_only_error_is_fp32_level(cuda, oracle):
    n = 512
    co = COEFF_SETS["compact"]
    d = np.random.default_rng(1).normal(size=(64, n))
    x = _solve(cuda, n, 64, co, d, precision="fp32")
    err = oracle.rel_err(x, _banded(oracle, n, co, d))
    assert 1e-9 < err < 2e-6


def test_pointer_offset_view(cuda, oracle):
    """solve(d_x_gpu[1, 0]) as in experiments/run-adi.py:65: N-2 rows from row 1."""
    import neato

    N = 64
    co = COEFF_SETS["adi256"]
    d = np.random.default_rng(3).normal(size=(N, N))
    t = torch.from_numpy(d).to(cuda)
    s = neato.NearToeplitzSolver(N, N - 2, co)
    s.solve(t[1, 0])
    torch.cuda.synchronize()
    out = t.cpu().numpy()
    assert np.array_equal(out[0], d[0]) and np.array_equal(out[-1], d[-1])
    ref = _banded(oracle, N, co, d[1:N - 1].copy())
    assert oracle.rel_err(out[1:N - 1], ref) < FP64_TOL


def test_empty_batch_is_a_no_op(cuda):
    import ntk

    t = torch.zeros(8, dtype=torch.float64, device=cuda)
    with ntk.Plan(8, 0, COEFF_SETS["compact"]) as p:
        p.solve(t)
    torch.cuda.synchronize()
    assert float(t.abs().sum()) == 0.0


def test_drop_in_strictness(cuda):
    import neato

    with pytest.raises(AssertionError):
        neato.NearToeplitzSolver(100, 1, COEFF_SETS["compact"])
    neato.NearToeplitzSolver(100, 1, COEFF_SETS["compact"], strict=False)


def test_buffer_too_small_rejected(cuda):
    import ntk

    t = torch.zeros(100, dtype=torch.float64, device=cuda)
    with ntk.Plan(64, 2, COEFF_SETS["compact"]) as p:
        with pytest.raises(ValueError):
            p.solve(t)


def test_singular_matrix_rejected(cuda):
    import ntk

    with pytest.raises(ValueError, match="pivot"):
        ntk.Plan(8, 1, (0., 1., 1., 0., 1., 1., 0.))


def test_strided_solve_matches_contiguous(cuda, oracle):
    """ntk_solve_strided on a y-sweep layout equals a contiguous solve of the
    permuted data (the permute of compact/permute.py made unnecessary)."""
    import ntk

    nz, ny, nx = 3, 128, 40
    co = COEFF_SETS["compact"]
    d = np.random.default_rng(5).normal(size=(nz, ny, nx))
    t = torch.from_numpy(d).to(cuda)
    out = torch.empty_like(t)
    for prec, tol in (("fp64", FP64_TOL), ("fp32_refine", REFINE_TOL)):
        with ntk.Plan(ny, 0, co, precision=prec) as p:
            p.solve_strided(t, out, nz * nx, nx, 1, nx * ny, nx)
            torch.cuda.synchronize()
        ref = oracle.cr_solve(np.ascontiguousarray(np.transpose(d, (0, 2, 1))), ny, co)
        got = np.transpose(out.cpu().numpy(), (0, 2, 1))
        assert oracle.rel_err(got, ref) < tol


@pytest.mark.parametrize("variant", [0, 1, 2])
@pytest.mark.parametrize("n", [4, 33, 512, 700])
def test_fp64_x_variants(cuda, oracle, variant, n):
    """Every launch variant of the contiguous FP64 sweep gives the same solve
    (and the fused compact derivative)."""
    import ntk

    co = COEFF_SETS["compact"]
    nrhs = 70
    d = np.random.default_rng(n + variant).normal(size=(nrhs, n))
    t = torch.from_numpy(d).to(cuda)
    with ntk.Plan(n, nrhs, co) as p:
        p.set_tuning(f64_x_variant=variant)
        assert p.get_tuning()["f64_x_variant"] == variant
        p.solve(t)
        torch.cuda.synchronize()
    assert oracle.rel_err(t.cpu().numpy(), _banded(oracle, n, co, d)) < FP64_TOL
    f = np.random.default_rng(n).normal(size=(3, nrhs // 3, n))
    ft = torch.from_numpy(f).to(cuda)
    out = torch.empty_like(ft)
    with ntk.Plan(n, 0, co) as p:
        p.set_tuning(f64_x_variant=variant)
        p.compact_deriv(ft, out, axis=2, h=0.1)
        torch.cuda.synchronize()
    assert oracle.rel_err(out.cpu().numpy(), oracle.banded_compact_deriv(f, 0.1, 2)) < FP64_TOL


@pytest.mark.parametrize("w", [4, 8, 16])
def test_refine_w_tuning(cuda, oracle, w):
    import ntk

    co = COEFF_SETS["compact"]
    d = np.random.default_rng(w).normal(size=(37, 512))
    t = torch.from_numpy(d).to(cuda)
    with ntk.Plan(512, 37, co, precision="fp32_refine") as p:
        p.set_tuning(refine_w=w)
        p.solve(t)
        torch.cuda.synchronize()
    assert oracle.rel_err(t.cpu().numpy(), _banded(oracle, 512, co, d)) < REFINE_TOL


# Systems longer than one warp's register tile (n > 1024): overlapping
# 512-row windows with halos below 2^-56, in place through the plan's work
# array; the reference's largest size (n = 2048) included.
@pytest.mark.parametrize("cname", ["compact", "dominant", "adi2048_r05"])
@pytest.mark.parametrize("n", [1025, 1500, 2048, 4096])
def test_refine_long_systems(cuda, oracle, cname, n):
    co = COEFF_SETS[cname]
    d = np.random.default_rng(n + len(cname)).normal(size=(9, n))
    x = _solve(cuda, n, 9, co, d, precision="fp32_refine")
    assert oracle.rel_err(x, _banded(oracle, n, co, d)) < REFINE_TOL
    x32 = _solve(cuda, n, 9, co, d, precision="fp32")
    assert oracle.rel_err(x32, _banded(oracle, n, co, d)) < 2e-5


@pytest.mark.parametrize("n", [600, 700, 1024])
@pytest.mark.parametrize("tps", [32, 64])
def test_refine_threads_per_system(cuda, oracle, n, tps):
    """512 < n <= 1024: one warp per system (32 threads, 32 rows per lane) or
    two overlapping 512-row windows (64 threads, 16 rows per lane), for the
    plain solve and the compact derivative: both within 1e-12."""
    import ntk

    co = COEFF_SETS["compact"]
    nrhs = 48
    rng = np.random.default_rng(n + tps)
    d = rng.standard_normal((nrhs, n))
    t = torch.from_numpy(d.copy()).to(cuda)
    with ntk.Plan(n, nrhs, co, precision="fp32_refine") as p:
        p.set_tuning(refine_tps=tps)
        p.solve(t)
        f = torch.from_numpy(rng.standard_normal((1, nrhs, n))).to(cuda)
        out = torch.empty_like(f)
        p.compact_deriv(f, out, axis=2, h=1.0 / (n - 1))
        torch.cuda.synchronize()
    ref = _banded(oracle, n, co, d)
    assert oracle.rel_err(t.cpu().numpy(), ref) < REFINE_TOL
    dref = oracle.banded_compact_deriv(f.cpu().numpy(), 1.0 / (n - 1), axis=2)
    assert oracle.rel_err(out.cpu().numpy(), dref) < REFINE_TOL
