"""Drop-in for compact/rhs.py: compute_rhs(f, rhs, dx) (compact/rhs.py:47-53).

RHS of the compact 4th-order first derivative along the last axis of a 3D
(or 2D) float64 field, on the GPU through libntk.  Unlike the reference it
accepts any extents (the reference needs multiples of 8).  For the full
derivative use ntk.Plan.compact_deriv, which fuses this into the solve.
"""
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import ntk  # noqa: E402


def compute_rhs(f, rhs, dx, stream=None):
    ntk.compact_rhs(f, rhs, dx, stream=stream)
