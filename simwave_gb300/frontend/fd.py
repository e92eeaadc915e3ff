"""Finite-difference weights and the CFL time step.

The reference takes its weights from the third-party ``findiff`` package
(``findiff>=0.8.9``, simwave/kernel/frontend/fd.py:31-52, requirements.txt:5),
which is not vendored. ``findiff.coefficients(deriv, acc)['center']`` is the
centred scheme on the integer offsets ``-acc/2 .. acc/2`` (for deriv 1 and 2
the number of nodes is ``acc + 1``). Its weights are the unique solution of the
Taylor moment system; here they are generated with Fornberg's recursion
(B. Fornberg, "Generation of finite difference formulas on arbitrarily spaced
grids", Math. Comp. 51, 1988) in exact rational arithmetic and rounded once to
float64, which reproduces the values pinned by the reference's
tests/test_space_model.py:133-155.
"""
from fractions import Fraction
from functools import lru_cache

import numpy as np


@lru_cache(maxsize=None)
def _fornberg(derivative_order, offsets):
    """Exact weights of the ``derivative_order``-th derivative at 0 on ``offsets``."""
    nodes = [Fraction(o) for o in offsets]
    n_nodes = len(nodes)
    m_max = derivative_order
    # w[m][j]: weight of node j for derivative m using the nodes seen so far
    w = [[Fraction(0)] * n_nodes for _ in range(m_max + 1)]
    w[0][0] = Fraction(1)
    c1 = Fraction(1)
    for n in range(1, n_nodes):
        c2 = Fraction(1)
        prev = [row[:] for row in w]
        for j in range(n):
            c3 = nodes[n] - nodes[j]
            c2 *= c3
            for m in range(min(n, m_max), -1, -1):
                lower = prev[m - 1][j] if m > 0 else Fraction(0)
                w[m][j] = (nodes[n] * prev[m][j] - m * lower) / c3
        for m in range(min(n, m_max), -1, -1):
            lower = prev[m - 1][n - 1] if m > 0 else Fraction(0)
            w[m][n] = c1 / c2 * (m * lower - nodes[n - 1] * prev[m][n - 1])
        c1 = c2
    return tuple(w[m_max])


def coefficients(derivative_order, space_order):
    """Centred FD weights (length ``space_order + 1``) as float64.

    Mirrors simwave/kernel/frontend/fd.py:31-52.
    """
    if derivative_order < 1:
        raise ValueError("derivative order must be >= 1")
    num_central = 2 * ((derivative_order + 1) // 2) - 1 + space_order
    half = num_central // 2
    offsets = tuple(range(-half, half + 1))
    return np.array([float(c) for c in _fornberg(derivative_order, offsets)],
                    dtype=np.float64)


def half_coefficients(derivative_order, space_order):
    """Weights from the centre outwards: ``[c0, c1, .., cr]``.

    Mirrors simwave/kernel/frontend/fd.py:5-28.
    """
    full = coefficients(derivative_order, space_order)
    return full[len(full) // 2:]


def calculate_dt(dimension, space_order, grid_spacing, velocity_model):
    """CFL time step ``sqrt(4 / (dim * sum|c2|)) * min(h) / max(v)``.

    Mirrors simwave/kernel/frontend/fd.py:55-95 (Lines 1986 SEG criterion for
    a 2nd-order-in-time leapfrog). The dtype flow is the reference's: the
    factor is float64, the spacing and velocity extrema keep the model dtype.
    """
    weights = coefficients(derivative_order=2, space_order=space_order)
    factor = np.sqrt(4 / (dimension * np.sum(np.abs(weights))))
    return factor * np.min(grid_spacing) / np.max(velocity_model)
