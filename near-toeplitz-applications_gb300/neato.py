"""Drop-in for the reference's neato.py (NearToeplitzSolver, neato.py:129-197).

Same constructor and solve() as the reference; the work is done by libntk
(hand-written sm_103a CUDA) instead of a PyCUDA-compiled cyclic-reduction
kernel.  Extra keyword arguments select the precision mode.
"""
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import ntk  # noqa: E402

__all__ = ["NearToeplitzSolver"]


class NearToeplitzSolver:

    def __init__(self, n, nrhs, coeffs, precision="fp64", refine_sweeps=1, strict=True):
        """
        n: the size of the tridiagonal system.
        nrhs: the number of right-hand sides (systems, contiguous).
        coeffs: (b1, c1, ai, bi, ci, an, bn) -- row 0 = [b1 c1], interior
            rows [ai bi ci], row n-1 = [an bn] (neato.py:136-138).
        precision: "fp64" (default), "fp32" or "fp32_refine".
        strict: keep the reference's power-of-two check (neato.py:145); the
            library itself accepts any n >= 3.
        """
        self.n = n
        self.nrhs = nrhs
        self.coeffs = coeffs
        if strict:
            # the reference asserts a power of two (neato.py:145) and needs
            # n >= 4 (its coefficient recurrence is empty for n = 2)
            assert int(n).bit_length() - 1 >= 2 and (int(n) & (int(n) - 1)) == 0
        self._plan = ntk.Plan(n, nrhs, coeffs, precision=precision, refine_sweeps=refine_sweeps)

    def solve(self, x_d, stream=None):
        """Solve the nrhs systems stored contiguously from x_d, in place."""
        self._plan.solve(x_d, stream=stream)
