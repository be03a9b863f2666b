"""The FP32 + refinement paths at the edges of their arithmetic: strong
cancellation in the compact stencil differences, inputs scaled by powers
of two across the double-word range, and a non-power-of-two interior at
n = 512 with |d| near 2^100 (the chunked kernel).  The CPU counterparts run
the same arithmetic through the host emulation (tests/test_r2_emul.py)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

N = 512
H = 1.0 / (N - 1)
COMPACT = (1., 2., .25, 1., .25, 2., 1.)
SHAPES = {0: (512, 4, 32), 1: (4, 512, 32), 2: (4, 32, 512)}


def _field(shape, seed, cuda):
    from ntk.workloads import fourier_field

    return fourier_field(shape, seed=seed, device=cuda)


def _deriv(f, axis, precision, **tuning):
    import ntk

    out = torch.empty_like(f)
    with ntk.Plan(N, 0, COMPACT, precision=precision) as p:
        if tuning:
            p.set_tuning(**tuning)
        p.compact_deriv(f, out, axis=axis, h=H)
    torch.cuda.synchronize()
    return out


@pytest.mark.parametrize("axis", [0, 1, 2])
def test_strong_cancellation_in_the_stencil(cuda, axis):
    """f = 2^20 + g: the differences f[i+1] - f[i-1] cancel 20 bits; formed in
    FP64 from the full values they are exact, so away from the one-sided end
    stencils (whose FP64 rounding any evaluation shares) FP32 + refinement
    stays within 1e-12 of the FP64 solve relative to the derivative's size."""
    f = _field(SHAPES[axis], 3, cuda) + 2.0 ** 20
    r = _deriv(f, axis, "fp32_refine")
    ref = _deriv(f, axis, "fp64")
    sl = [slice(None)] * 3
    sl[axis] = slice(40, N - 40)
    sl = tuple(sl)
    err = float((r[sl] - ref[sl]).abs().max() / ref[sl].abs().max())
    assert err < 1e-12, err


@pytest.mark.parametrize("axis", [0, 1, 2])
@pytest.mark.parametrize("scale", [2.0 ** 100, 2.0 ** -60])
def test_power_of_two_scaling_is_exact(cuda, axis, scale):
    """Inside the double-word range every operation of the paired-chunk
    kernels scales exactly by a power of two: scaled input, scaled result,
    bit for bit."""
    f = _field(SHAPES[axis], 4, cuda)
    r = _deriv(f, axis, "fp32_refine")
    rs = _deriv(f * scale, axis, "fp32_refine")
    assert torch.equal(rs, r * scale)


@pytest.mark.parametrize("scale", [2.0 ** 100, 2.0 ** -60])
def test_general_interior_near_the_range_ends(cuda, oracle, scale):
    """A non-power-of-two interior (0.3, 1, 0.3) at n = 512 (the chunked
    kernel: the paired-chunk one serves powers of two) with |d| near 2^100
    and 2^-60: within 1e-12 of a long-double Thomas solve."""
    import ntk

    coeffs = (1.0, 0.4, 0.3, 1.0, 0.3, 0.4, 1.0)
    rng = np.random.default_rng(12)
    d = rng.normal(size=(24, N)) * scale
    t = torch.from_numpy(d).to(cuda)
    with ntk.Plan(N, 24, coeffs, precision="fp32_refine") as p:
        p.solve(t)
        torch.cuda.synchronize()
        assert p.status() == 0
    x = t.cpu().numpy()
    a, b, c = oracle.near_toeplitz_bands(N, coeffs)
    ref = np.array([oracle.thomas_ld(a, b, c, row) for row in d])
    assert oracle.rel_err(x, ref) < 1e-12
