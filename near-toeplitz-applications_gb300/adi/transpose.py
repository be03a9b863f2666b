"""Drop-in for adi/transpose.py: transpose(a, b, N) writes b = a^T
(adi/transpose.py:40-50), N x N float64, any N."""
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import ntk  # noqa: E402


def transpose(a, b, N, stream=None):
    ntk.transpose2d(a, b, N, stream=stream)
