"""1D quadrature rules and the Lagrange basis tables of the tensor H1 basis.

This is the host-side setup that libCEED's frontend does before it hands the tables to a backend:
Gauss and Gauss-Lobatto points by Newton iteration on Legendre polynomials
(interface/ceed-basis.c:2529-2634) and Fornberg's recurrence for the interpolation and derivative
matrices on Gauss-Lobatto nodes (interface/ceed-basis.c:1617-1680).  Tables are row-major Q x P.
"""
import math

import numpy as np

GAUSS, GAUSS_LOBATTO = 0, 1
_EPS = 1e-16  # CEED_EPSILON of include/ceed/ceed-f64.h


def _legendre(x, n):
    p0, p1, p2 = 1.0, x, 0.0
    for j in range(2, n + 1):
        p2 = ((2 * j - 1) * x * p1 - (j - 1) * p0) / j
        p0, p1 = p1, p2
    return p0, p2


def gauss_quadrature(Q):
    """Gauss-Legendre points and weights on [-1, 1]."""
    x_out, w_out = np.zeros(Q), np.zeros(Q)
    for i in range(Q // 2 + 1):
        x = math.cos(math.pi * (2 * i + 1) / (2 * Q))
        p0, p2 = _legendre(x, Q)
        dp2 = (x * p2 - p0) * Q / (x * x - 1.0)
        x = x - p2 / dp2
        k = 0
        while k < 100 and abs(p2) > 10 * _EPS:
            p0, p2 = _legendre(x, Q)
            dp2 = (x * p2 - p0) * Q / (x * x - 1.0)
            x = x - p2 / dp2
            k += 1
        w = 2.0 / ((1.0 - x * x) * dp2 * dp2)
        w_out[i] = w_out[Q - 1 - i] = w
        x_out[i], x_out[Q - 1 - i] = -x, x
    return x_out, w_out


def lobatto_quadrature(Q):
    """Gauss-Lobatto-Legendre points and weights on [-1, 1] (Q >= 2)."""
    if Q < 2:
        raise ValueError(f"Cannot create Lobatto quadrature with Q={Q} < 2 points")
    x_out, w_out = np.zeros(Q), np.zeros(Q)
    w = 2.0 / (Q * (Q - 1))
    w_out[0] = w_out[Q - 1] = w
    x_out[0], x_out[Q - 1] = -1.0, 1.0
    for i in range(1, (Q - 1) // 2 + 1):
        x = math.cos(math.pi * i / (Q - 1))
        p0, p2 = _legendre(x, Q - 1)
        dp2 = (x * p2 - p0) * Q / (x * x - 1.0)
        d2p2 = (2 * x * dp2 - Q * (Q - 1) * p2) / (1.0 - x * x)
        x = x - dp2 / d2p2
        k = 0
        while k < 100 and abs(dp2) > 10 * _EPS:
            p0, p2 = _legendre(x, Q - 1)
            dp2 = (x * p2 - p0) * Q / (x * x - 1.0)
            d2p2 = (2 * x * dp2 - Q * (Q - 1) * p2) / (1.0 - x * x)
            x = x - dp2 / d2p2
            k += 1
        w = 2.0 / ((Q * (Q - 1)) * p2 * p2)
        w_out[i] = w_out[Q - 1 - i] = w
        x_out[i], x_out[Q - 1 - i] = -x, x
    return x_out, w_out


def lagrange_1d(P, Q, qmode=GAUSS):
    """(interp, grad, q_ref, q_weight): Lagrange basis on P Gauss-Lobatto nodes at Q points."""
    nodes, _ = lobatto_quadrature(P)
    qref, qw = gauss_quadrature(Q) if qmode == GAUSS else lobatto_quadrature(Q)
    interp = np.zeros((Q, P))
    grad = np.zeros((Q, P))
    for i in range(Q):
        c1, c3 = 1.0, nodes[0] - qref[i]
        interp[i, 0] = 1.0
        for j in range(1, P):
            c2, c4 = 1.0, c3
            c3 = nodes[j] - qref[i]
            for k in range(j):
                dx = nodes[j] - nodes[k]
                c2 *= dx
                if k == j - 1:
                    grad[i, j] = c1 * (interp[i, k] - c4 * grad[i, k]) / c2
                    interp[i, j] = -c1 * c4 * interp[i, k] / c2
                grad[i, k] = (c3 * grad[i, k] - interp[i, k]) / dx
                interp[i, k] = c3 * interp[i, k] / dx
            c1 = c2
    return interp, grad, qref, qw
