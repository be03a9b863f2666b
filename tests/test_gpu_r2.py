"""The paired-chunk TMA kernels for systems of 512 rows (csrc/ntk_r2.cu, the
plans' FP32 and FP32+refine path for n = 512) on the GPU:

* bit for bit equal to their host emulation (tests/r2_emul.cpp, the same
  arithmetic run chunk by chunk on the CPU) for x, y and z derivatives,
  plain solves, partial CTA groups, in-place calls and every systems-per-CTA
  setting;
* within 1e-12 of the FP64 banded oracle (refinement) and near 1e-6 without
  refinement, and within 1e-12 of the chunked kernel they replace;
* a misaligned view falls back to the chunked kernel and stays correct."""
import numpy as np
import pytest
import torch

from conftest import r2emu_solve

pytestmark = pytest.mark.gpu

N = 512
H = 1.0 / (N - 1)
COMPACT = (1., 2., .25, 1., .25, 2., 1.)


def _field(shape, seed, cuda):
    from ntk.workloads import fourier_field

    return fourier_field(shape, seed=seed, device=cuda)


def _lines(a, axis):
    return np.ascontiguousarray(np.moveaxis(a, axis, -1).reshape(-1, N))


def _bits_equal(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.int64), np.ascontiguousarray(b).view(np.int64))


# x: whole and partial CTA groups; y: 48 and 24 columns (a partial 16-column
# group per plane); z: 320 and 72 columns per plane
SHAPES = [((8, 64, 512), 2), ((3, 7, 512), 2), ((4, 512, 48), 1), ((2, 512, 24), 1), ((512, 8, 40), 0),
          ((512, 3, 24), 0)]


@pytest.mark.parametrize("shape,axis", SHAPES)
@pytest.mark.parametrize("precision", ["fp32_refine", "fp32"])
def test_derivative_bitwise_equal_to_emulation(cuda, r2emu, oracle, shape, axis, precision):
    import ntk

    f = _field(shape, seed=sum(shape) + axis, cuda=cuda)
    out = torch.empty_like(f)
    with ntk.Plan(N, 0, COMPACT, precision=precision) as p:
        p.compact_deriv(f, out, axis=axis, h=H)
        assert p.status() == 0
    torch.cuda.synchronize()
    fl = _lines(f.cpu().numpy(), axis)
    x = _lines(out.cpu().numpy(), axis)
    rc, xe = r2emu_solve(r2emu, fl, sweeps=1 if precision == "fp32_refine" else 0)
    assert rc == 0
    assert _bits_equal(x, xe), np.abs(x - xe).max()
    ref = oracle.banded_compact_deriv(fl[:, None, :], H, axis=2)[:, 0, :]
    err = oracle.rel_err(x, ref)
    assert err < (1e-12 if precision == "fp32_refine" else 2e-5), err


@pytest.mark.parametrize("w", [4, 8, 16])
def test_systems_per_cta_do_not_change_the_result(cuda, r2emu, w):
    import ntk

    f = _field((5, 13, 512), seed=w, cuda=cuda)
    out = torch.empty_like(f)
    with ntk.Plan(N, 0, COMPACT, precision="fp32_refine") as p:
        p.set_tuning(refine_w=w)
        p.compact_deriv(f, out, axis=2, h=H)
    torch.cuda.synchronize()
    rc, xe = r2emu_solve(r2emu, _lines(f.cpu().numpy(), 2))
    assert rc == 0 and _bits_equal(_lines(out.cpu().numpy(), 2), xe)


@pytest.mark.parametrize("axis", [0, 1, 2])
def test_in_place_equals_out_of_place(cuda, axis):
    import ntk

    f = _field((512, 32, 32) if axis == 0 else (16, 512, 32) if axis == 1 else (16, 32, 512), seed=7, cuda=cuda)
    out = torch.empty_like(f)
    g = f.clone()
    with ntk.Plan(N, 0, COMPACT, precision="fp32_refine") as p:
        p.compact_deriv(f, out, axis=axis, h=H)
        p.compact_deriv(g, g, axis=axis, h=H)
    torch.cuda.synchronize()
    assert torch.equal(out, g)


def test_plain_solve_bitwise_and_accurate(cuda, r2emu, oracle):
    import ntk

    rng = np.random.default_rng(11)
    d = rng.normal(size=(37, N))
    t = torch.from_numpy(d).to(cuda)
    with ntk.Plan(N, 37, COMPACT, precision="fp32_refine") as p:
        p.solve(t)
    torch.cuda.synchronize()
    x = t.cpu().numpy()
    rc, xe = r2emu_solve(r2emu, d, compact=False)
    assert rc == 0 and _bits_equal(x, xe)
    a, b, c = oracle.near_toeplitz_bands(N, COMPACT)
    ref = np.array([oracle.thomas_ld(a, b, c, row) for row in d])
    assert oracle.rel_err(x, ref) < 1e-12


@pytest.mark.parametrize("axis", [0, 1, 2])
def test_agrees_with_the_chunked_kernel(cuda, axis):
    import ntk

    shape = {0: (512, 16, 48), 1: (8, 512, 48), 2: (8, 48, 512)}[axis]
    f = _field(shape, seed=3, cuda=cuda)
    o2, o1 = torch.empty_like(f), torch.empty_like(f)
    with ntk.Plan(N, 0, COMPACT, precision="fp32_refine") as p:
        p.compact_deriv(f, o2, axis=axis, h=H)
        p.set_tuning(refine_kernel=1)
        p.compact_deriv(f, o1, axis=axis, h=H)
    torch.cuda.synchronize()
    den = float(o1.abs().max())
    assert float((o2 - o1).abs().max()) / den < 1e-12


def test_misaligned_view_falls_back_and_stays_correct(cuda, oracle):
    """A system batch starting 8 bytes into a buffer cannot be a TMA tensor
    (16-byte base): the plan runs the chunked kernel instead."""
    import ntk

    rng = np.random.default_rng(12)
    d = rng.normal(size=(9, N))
    buf = torch.zeros(9 * N + 1, dtype=torch.float64, device=cuda)
    buf[1:] = torch.from_numpy(d.reshape(-1)).to(cuda)
    view = buf[1:]
    with ntk.Plan(N, 9, COMPACT, precision="fp32_refine") as p:
        p.solve(view)
    torch.cuda.synchronize()
    a, b, c = oracle.near_toeplitz_bands(N, COMPACT)
    ref = np.array([oracle.thomas_ld(a, b, c, row) for row in d])
    assert oracle.rel_err(view.cpu().numpy().reshape(9, N), ref) < 1e-12


@pytest.mark.parametrize("shape,axis", [((160, 512, 64), 1), ((512, 96, 112), 0)])
def test_persistent_ctas_cycle_their_tile_buffers(cuda, r2emu, shape, axis):
    """Enough 16-system groups (640 and 672) that every persistent CTA (one
    per SM) reloads each of its three tile buffers at least once; the result
    equals the emulation bit for bit and the one-group-per-CTA kernel's."""
    import ntk

    f = _field(shape, seed=5, cuda=cuda)
    o0, o2 = torch.empty_like(f), torch.empty_like(f)
    with ntk.Plan(N, 0, COMPACT, precision="fp32_refine") as p:
        p.set_tuning(refine_kernel=3)
        p.compact_deriv(f, o0, axis=axis, h=H)
        p.set_tuning(refine_kernel=2)
        p.compact_deriv(f, o2, axis=axis, h=H)
        assert p.status() == 0
    torch.cuda.synchronize()
    assert torch.equal(o0, o2)
    rc, xe = r2emu_solve(r2emu, _lines(f.cpu().numpy(), axis))
    assert rc == 0 and _bits_equal(_lines(o0.cpu().numpy(), axis), xe)


@pytest.mark.parametrize("precision", ["fp32_refine", "fp32"])
def test_one_launch_gradient_equals_three_derivatives(cuda, precision):
    """ntk_compact_grad on a 512^3 field (one launch of the combined kernel)
    gives the same bits as the three ntk_compact_deriv calls."""
    import ntk

    f = _field((N, N, N), seed=9, cuda=cuda)
    g = [torch.empty_like(f) for _ in range(3)]
    d = [torch.empty_like(f) for _ in range(3)]
    with ntk.Plan(N, 0, COMPACT, precision=precision) as p:
        p.compact_grad(f, g[0], g[1], g[2], h=H)
        for k, axis in enumerate((2, 1, 0)):
            p.compact_deriv(f, d[k], axis=axis, h=H)
        assert p.status() == 0
    torch.cuda.synchronize()
    for k in range(3):
        assert torch.equal(g[k], d[k]), k
    del g, d, f
    torch.cuda.empty_cache()


def test_gradient_falls_back_to_three_calls(cuda, oracle):
    """Other sizes and FP64 run the three derivatives one after another."""
    import ntk

    n = 64
    f = _field((n, n, n), seed=4, cuda=cuda)
    for prec, tol in (("fp64", 1e-13), ("fp32_refine", 1e-12)):
        outs = [torch.empty_like(f) for _ in range(3)]
        with ntk.Plan(n, 0, COMPACT, precision=prec) as p:
            p.compact_grad(f, *outs, h=1.0 / (n - 1))
        torch.cuda.synchronize()
        fc = f.cpu().numpy()
        for o, axis in zip(outs, (2, 1, 0)):
            ref = oracle.banded_compact_deriv(fc, 1.0 / (n - 1), axis=axis)
            assert oracle.rel_err(o.cpu().numpy(), ref) < tol, (prec, axis)
