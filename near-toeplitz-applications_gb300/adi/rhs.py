"""Drop-in for adi/rhs.py: compute_rhs(u, d, dx, dt, N) (adi/rhs.py:35-55).

Explicit half of the ADI step: interior points of d get
bottom*u[i-N] + center*u[i] + top*u[i+N] with bottom = top = -1/dx^2 and
center = 2(-1/dt + 1/dx^2) (adi/rhs.py:46-49); boundary points untouched."""
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import ntk  # noqa: E402


def compute_rhs(u, d, dx, dt, N, stream=None):
    ntk.adi_rhs(u, d, dx, dt, N, stream=stream)
