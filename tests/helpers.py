"""Numeric helpers shared by the tests."""
import numpy as np


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    d = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (d if d > 0 else 1.0)


def lap7(u, hx, hy, hz):
    """7-point Dirichlet Laplacian (zero outside the box) of a (z, y, x) array."""
    p = np.pad(u, 1)
    return ((p[1:-1, 1:-1, 2:] + p[1:-1, 1:-1, :-2] - 2 * u) / hx**2
            + (p[1:-1, 2:, 1:-1] + p[1:-1, :-2, 1:-1] - 2 * u) / hy**2
            + (p[2:, 1:-1, 1:-1] + p[:-2, 1:-1, 1:-1] - 2 * u) / hz**2)
