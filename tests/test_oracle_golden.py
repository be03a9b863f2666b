"""The oracle (C restatement of the reference, oracle/ntk_oracle.c) against
golden vectors produced by the reference's own code (tests/golden/).  All
comparisons are bit-exact: the restatement keeps the reference's operation
order and both sides are strict IEEE double without contraction."""
import numpy as np
import pytest

from golden.make_golden import COEFF_SETS


@pytest.mark.parametrize("cname", sorted(COEFF_SETS))
def test_precompute_coefficients_bitwise(oracle, golden, cname):
    co = COEFF_SETS[cname]
    for L in range(2, 12):
        n = 1 << L
        mine = np.stack(oracle.precompute(n, co))
        assert np.array_equal(mine, golden["coef_%s_n%d" % (cname, n)]), n


@pytest.mark.parametrize("cname", sorted(COEFF_SETS))
def test_cr_solve_bitwise(oracle, golden, cname):
    co = COEFF_SETS[cname]
    seen = 0
    for L in range(2, 11):
        n = 1 << L
        key = "cr_%s_n%d_in" % (cname, n)
        if key not in golden:
            continue
        x = oracle.cr_solve(golden[key], n, co)
        assert np.array_equal(x, golden["cr_%s_n%d_out" % (cname, n)]), n
        seen += 1
    assert seen >= 7


# How far the reference's cyclic reduction lands from LAPACK's banded solve.
# With the ADI coefficients (identity boundary rows next to interior rows
# scaled by 1/dx^2, experiments/run-adi.py:50-53) and random right-hand sides
# the reference CR loses up to ~2.3e-12 (measured on these fixtures); with the
# compact and diagonally dominant sets it is at FP64 rounding.
CR_VS_BANDED = {"compact": 1e-15, "dominant": 1e-15, "adi256": 5e-12, "adi2048_r05": 2e-11}


@pytest.mark.parametrize("cname", sorted(COEFF_SETS))
def test_cr_matches_banded_solve(oracle, golden, cname):
    co = COEFF_SETS[cname]
    for L in range(2, 9):
        n = 1 << L
        d = golden["cr_%s_n%d_in" % (cname, n)]
        a, b, c = oracle.near_toeplitz_bands(n, co)
        xb = oracle.tridiagonal_solve(a, b, c, d.T).T
        assert oracle.rel_err(golden["cr_%s_n%d_out" % (cname, n)], xb) < CR_VS_BANDED[cname], n


def test_compact_rhs_bitwise(oracle, golden):
    out = oracle.compact_rhs(golden["rhs_in"], float(golden["rhs_dx"]))
    assert np.array_equal(out, golden["rhs_out"])


@pytest.mark.parametrize("perm", [(0, 2, 1), (1, 2, 0), (2, 0, 1)])
def test_permute_bitwise(oracle, golden, perm):
    out = oracle.permute(golden["perm_in"], perm)
    assert np.array_equal(out, golden["perm_%d%d%d" % perm])
    assert np.array_equal(out, np.transpose(golden["perm_in"], perm))


def test_adi_rhs_and_transpose_bitwise(oracle, golden):
    d = golden["adi_rhs_d"].copy()
    oracle.adi_rhs(golden["adi_rhs_u"], d, 1.0 / 31, 0.01)
    assert np.array_equal(d, golden["adi_rhs_out"])
    assert np.array_equal(oracle.transpose(golden["transpose_in"]), golden["transpose_out"])


def test_adi_steps_bitwise(oracle, golden):
    u = golden["adi_step_u0"].copy()
    d_x = u.copy()
    d_y = u.T.copy()
    dx, dt = float(golden["adi_step_dx"]), float(golden["adi_step_dt"])
    for _ in range(3):
        oracle.adi_step(u, d_x, d_y, dx, dt)
    assert np.array_equal(u, golden["adi_step_u3"])


def test_compact_derivative_end_to_end_bitwise(oracle, golden):
    f = golden["deriv_f"]
    h = float(golden["deriv_h"])
    n = f.shape[0]
    from golden.make_golden import COMPACT

    dfdx = oracle.cr_solve(oracle.compact_rhs(f, h), n, COMPACT)
    assert np.array_equal(dfdx, golden["deriv_dfdx"])
    fy = oracle.permute(f, (0, 2, 1))
    tmp = oracle.cr_solve(oracle.compact_rhs(fy, h), n, COMPACT)
    assert np.array_equal(oracle.permute(tmp, (0, 2, 1)), golden["deriv_dfdy"])
    # and the SciPy banded path agrees to rounding
    assert oracle.rel_err(oracle.banded_compact_deriv(f, h, axis=2), dfdx) < 1e-13
    assert oracle.rel_err(oracle.banded_compact_deriv(f, h, axis=1), golden["deriv_dfdy"]) < 1e-13


def test_compact_scheme_exact_for_linear_field(oracle):
    """Linear f: the compact scheme's derivative is exact (the known answer
    of experiments/run-parallel-compact.py:44,90, f = xyz)."""
    n = 32
    x = np.linspace(0, 1, n)
    z, y, xx = np.meshgrid(x, x, x, indexing="ij")
    f = xx * y * z
    h = 1.0 / (n - 1)
    d = oracle.banded_compact_deriv(f, h, axis=2)
    np.testing.assert_allclose(d, y * z, rtol=0, atol=1e-12)
