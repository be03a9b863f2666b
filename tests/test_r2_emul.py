"""The arithmetic of the paired-chunk FP32 + refinement solve (the n = 512
kernels of csrc/ntk_r2.cu), run on the CPU through its host emulation
(tests/r2_emul.cpp, built from the same header the kernels use) against the
oracle: the compact derivative and the plain solve within 1e-12 of the FP64
banded / long-double solves (the refinement tolerance), FP32 alone near
1e-6, two special rows at each end, and the range and edge checks.  The GPU
tests compare the kernels with this emulation bit for bit."""
import numpy as np
import pytest

from conftest import r2emu_solve

N = 512
H = 1.0 / (N - 1)
COMPACT = (1., 2., .25, 1., .25, 2., 1.)


def _fourier_lines(count, seed):
    from ntk.workloads import fourier_block

    return fourier_block((count, N), (0, 0), (count, N), seed=seed)


def test_compact_derivative_within_refine_tolerance(r2emu, oracle):
    f = _fourier_lines(64, 0)
    ref = oracle.banded_compact_deriv(f[:, None, :], H, axis=2)[:, 0, :]
    rc, x = r2emu_solve(r2emu, f)
    assert rc == 0
    assert oracle.rel_err(x, ref) < 1e-12
    rng = np.random.default_rng(1)
    g = rng.normal(size=(64, N))
    rc, x = r2emu_solve(r2emu, g)
    assert rc == 0
    assert oracle.rel_err(x, oracle.banded_compact_deriv(g[:, None, :], H, axis=2)[:, 0, :]) < 1e-12


def test_fp32_only_is_fp32_accurate(r2emu, oracle):
    f = _fourier_lines(16, 2)
    ref = oracle.banded_compact_deriv(f[:, None, :], H, axis=2)[:, 0, :]
    rc, x = r2emu_solve(r2emu, f, sweeps=0)
    assert rc == 0
    assert 1e-9 < oracle.rel_err(x, ref) < 2e-5


def test_plain_solve_matches_long_double_thomas(r2emu, oracle):
    rng = np.random.default_rng(3)
    d = rng.normal(size=(32, N))
    rc, x = r2emu_solve(r2emu, d, compact=False)
    assert rc == 0
    a, b, c = oracle.near_toeplitz_bands(N, COMPACT)
    ref = np.array([oracle.thomas_ld(a, b, c, row) for row in d])
    assert oracle.rel_err(x, ref) < 1e-12


def test_two_special_rows_at_each_end(r2emu, oracle):
    head = [0., 1.5, .5, .25, 1.25, .5]
    tail = [.5, 1.25, .25, .5, 1.5, 0.]
    rng = np.random.default_rng(4)
    d = rng.normal(size=(16, N))
    rc, x = r2emu_solve(r2emu, d, compact=False, head=head, tail=tail)
    assert rc == 0
    a = np.full(N, .25)
    b = np.ones(N)
    c = np.full(N, .25)
    b[0], c[0] = 1.5, .5
    a[1], b[1], c[1] = .25, 1.25, .5
    a[-2], b[-2], c[-2] = .5, 1.25, .25
    a[-1], b[-1] = .5, 1.5
    a[0] = c[-1] = 0.
    ref = np.array([oracle.thomas_ld(a, b, c, row) for row in d])
    assert oracle.rel_err(x, ref) < 1e-12


def test_zero_field_gives_exact_zeros_and_range_is_flagged(r2emu):
    rc, x = r2emu_solve(r2emu, np.zeros((2, N)))
    assert rc == 0 and not np.any(x)
    g = np.random.default_rng(5).normal(size=(2, N))
    g[1, 200] = 2.0 ** 130
    rc, _ = r2emu_solve(r2emu, g)
    assert rc == 2


@pytest.mark.parametrize("coeffs", [(1., 2., .3, 1., .3, 2., 1.), (1., 0., .5, 1., .5, 0., 1.)])
def test_matrices_outside_its_scope_are_declined(r2emu, coeffs):
    """Non-power-of-two interior coefficients, or multipliers that decay too
    slowly for 16-row carries (a = c = 1/2: l -> 1), are not served."""
    rc, _ = r2emu_solve(r2emu, np.zeros((1, N)), coeffs=coeffs)
    assert rc == 1


def test_split_and_assembly(r2emu):
    import ctypes

    rng = np.random.default_rng(6)
    m = 200_000
    # magnitudes in [2^-78, 2^126): the double-word range (lo is dropped below 2^-80)
    x = (1 + rng.random(m)) * np.sign(rng.normal(size=m)) * np.exp2(rng.integers(-78, 125, size=m))
    hi = np.zeros(m, np.float32)
    lo = np.zeros(m, np.float32)
    F = ctypes.POINTER(ctypes.c_float)
    D = ctypes.POINTER(ctypes.c_double)
    r2emu.r2emu_split(x.ctypes.data_as(D), m, hi.ctypes.data_as(F), lo.ctypes.data_as(F))
    assert np.all(np.abs(hi) <= np.abs(x))                       # hi is x truncated
    assert np.max(np.abs(hi.astype(np.float64) + lo - x) / np.abs(x)) < 2.0 ** -46
    # normalised pairs as TwoSum makes them, powers of two included
    h = ((1 + rng.random(m)) * np.sign(rng.normal(size=m)) * np.exp2(rng.integers(-78, 120, size=m))).astype(np.float32)
    h[:2000] = (np.exp2(rng.integers(-78, 120, size=2000)) * np.sign(rng.normal(size=2000))).astype(np.float32)
    d = (h.astype(np.float64) * rng.normal(size=m) * 2.0 ** -20).astype(np.float32)
    s = (h + d).astype(np.float32)
    bb = (s - h).astype(np.float32)
    e = ((h - (s - bb)) + (d - bb)).astype(np.float32)
    out = np.zeros(m)
    r2emu.r2emu_dw(s.ctypes.data_as(F), e.ctypes.data_as(F), m, out.ctypes.data_as(D))
    exact = h.astype(np.float64) + d.astype(np.float64)
    assert np.max(np.abs(out - exact) / np.abs(exact)) <= 2.0 ** -47 * (1 + 2.0 ** -20)


def _window_rows(kind, abc, head6, tail6):
    """Bands of one 512-row window of an uneven-batch system (ntk_batch_refine.cu):
    kind 'first' (the system's head rows, the tail cut), 'middle' (both cut:
    row 0 = (0, b, c), the last row (a, b, 0)), 'last' (head cut, the
    system's tail rows) or 'whole'."""
    ai, bi, ci = abc
    a = np.full(N, ai)
    b = np.full(N, bi)
    c = np.full(N, ci)
    if kind in ("first", "whole"):
        a[0], b[0], c[0] = 0., head6[1], head6[2]
        a[1], b[1], c[1] = head6[3:6]
        nh, head = 2, [0., head6[1], head6[2]] + list(head6[3:6])
    else:
        nh, head = 1, [0., bi, ci, 0., 1., 0.]
    if kind in ("last", "whole"):
        a[-2], b[-2], c[-2] = tail6[0:3]
        a[-1], b[-1] = tail6[3], tail6[4]
        nt, tail = 2, list(tail6[0:5]) + [0.]
    else:
        nt, tail = 0, [0., 1., 0., 0., 1., 0.]
    a[0] = c[-1] = 0.
    return (a, b, c), nh, nt, head, tail


@pytest.mark.parametrize("kind", ["first", "middle", "last", "whole"])
def test_general_coefficient_windows_match_long_double_thomas(r2emu, oracle, kind):
    """The uneven batch's paired-chunk windows: interior coefficients of any
    value (a, c up to 0.3, b = 1, the benchmark batch's range, and the
    slowest decay it has), random diagonally dominant end rows, one sweep
    within the refinement tolerance of a long-double solve."""
    import ctypes

    P = ctypes.POINTER(ctypes.c_double)
    rng = np.random.default_rng(11)
    for ai, ci in ((0.1, 0.1), (0.3, 0.3), (0.137, 0.291)):
        h = []
        for _ in range(2):
            aa, cc = rng.uniform(-0.4, 0.4, size=2)
            h += [aa, abs(aa) + abs(cc) + rng.uniform(0.5, 1.5), cc]
        t = []
        for _ in range(2):
            aa, cc = rng.uniform(-0.4, 0.4, size=2)
            t += [aa, abs(aa) + abs(cc) + rng.uniform(0.5, 1.5), cc]
        (a, b, c), nh, nt, head, tail = _window_rows(kind, (ai, 1.0, ci), h, t)
        d = rng.normal(size=(8, N))
        out = np.zeros_like(d)
        hd = np.ascontiguousarray(head, dtype=np.float64)
        tl = np.ascontiguousarray(tail, dtype=np.float64)
        why = ctypes.create_string_buffer(256)
        rc = r2emu.r2emu_solve_general(nh, nt, hd.ctypes.data_as(P), tl.ctypes.data_as(P), ai, 1.0, ci,
                                       2.0 ** -22, 2.0 ** -22, 1, d.shape[0], d.ctypes.data_as(P),
                                       out.ctypes.data_as(P), why, 256)
        assert rc == 0, why.value
        ref = np.array([oracle.thomas_ld(a, b, c, row) for row in d])
        assert oracle.rel_err(out, ref) < 1e-13, (kind, ai, ci)


def test_strong_cancellation_in_the_compact_rhs(r2emu, oracle):
    """f = 2^20 + g with |g| ~ 1: the stencil differences f[i+1] - f[i-1]
    cancel 20 bits of f.  They are formed in FP64 from the full values
    (exact here), so away from the ends the derivative keeps the refinement
    tolerance relative to its own size; rounding f to the double-word split
    before differencing would leave ~2^-48 * 2^20 of error, far outside it.
    The one-sided end stencils (-5 f0 + 4 f1 + f2) cancel 2^20 in any FP64
    evaluation (the banded oracle's included); their rounding fades like
    0.27^k into the interior, so rows 40..471 are compared."""
    for offset in (2.0 ** 20, 2.0 ** 30):
        f = _fourier_lines(32, 7) + offset
        g = f - offset  # the perturbation f holds (exact)
        ref = oracle.banded_compact_deriv(g[:, None, :], H, axis=2)[:, 0, :]
        rc, x = r2emu_solve(r2emu, f)
        assert rc == 0
        assert oracle.rel_err(x[:, 40:N - 40], ref[:, 40:N - 40]) < 1e-12


@pytest.mark.parametrize("scale", [2.0 ** 100, 2.0 ** -60])
def test_power_of_two_scaling_is_exact(r2emu, scale):
    """Inside the double-word range (largest |input| in [2^-80, 2^128)) every
    operation of the solve scales exactly by a power of two: the results of
    a scaled input are the scaled results, bit for bit."""
    f = _fourier_lines(16, 8)
    rc, x = r2emu_solve(r2emu, f)
    assert rc == 0
    rc, xs = r2emu_solve(r2emu, f * scale)
    assert rc == 0
    assert np.array_equal(xs, x * scale)


def test_general_windows_decline_slow_decay(r2emu):
    """With a = c = 0.45, b = 1 the multipliers (l = 0.63) decay too slowly
    for 16-row carries even at the batch's relaxed limit (2^-22): the window
    is declined, and the batch solves that system with the chunked kernel."""
    import ctypes

    P = ctypes.POINTER(ctypes.c_double)
    head = np.ascontiguousarray([0., 1.5, .3, .2, 1.4, .3])
    tail = np.ascontiguousarray([.2, 1.4, .3, .3, 1.5, 0.])
    d = np.zeros((1, N))
    out = np.zeros_like(d)
    why = ctypes.create_string_buffer(256)
    rc = r2emu.r2emu_solve_general(2, 2, head.ctypes.data_as(P), tail.ctypes.data_as(P), 0.45, 1.0, 0.45,
                                   2.0 ** -22, 2.0 ** -22, 1, 1, d.ctypes.data_as(P), out.ctypes.data_as(P),
                                   why, 256)
    assert rc == 1 and b"decay" in why.value
