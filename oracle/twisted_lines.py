"""Oracle (test infrastructure only): the two-sided ("twisted") banded solve
that the FDM line-solve kernel runs with two threads per line, restated in
numpy to check the algorithm on the CPU.

A complex-symmetric band matrix of half-bandwidth P is cut at row m. The top
half is eliminated from row 0 down, the bottom half from row n-1 up (the same
elimination on the reversed line, the band row read backwards). Each half's
elimination runs over the band's columns past its end, so its last P rows of
U hold the coupling to the other half. With those rows scaled by their
reciprocal pivots, U1 T1 + W1 T2 = c1 and U2 T2 + W2 T1 = c2 (U unit upper
triangular, T the P unknowns next to the cut on each side, the bottom's in
reversed order); the 2P x 2P system is solved by the Schur complement on T2,
and each half back-substitutes from the other's values at the cut.
"""
from __future__ import annotations

import numpy as np


def _half(band, b, P, m, bottom):
    """Elimination of one half; returns the U rows (reciprocal pivot first),
    L^-1 b, and the row map."""
    n = band.shape[0]
    L = n - m if bottom else m
    phys = (lambda k: n - 1 - k) if bottom else (lambda k: k)
    Uw = [np.ones(P + 1, complex) for _ in range(P)]
    yw = [0j] * P
    U, y = [], []
    for k in range(L):
        pk = phys(k)
        a = np.array([band[pk, 2 * P - o] if bottom else band[pk, o] for o in range(2 * P + 1)], complex)
        r = complex(b[pk])
        for d in range(P, 0, -1):
            if k - d < 0:
                continue
            Ur = Uw[d - 1]
            f = a[P - d] * Ur[0]
            a[P - d + 1:P - d + P + 1] -= f * Ur[1:]
            r -= f * yw[d - 1]
        a[P] = 1.0 / a[P]
        Uw = [a[P:].copy()] + Uw[:-1]
        yw = [r] + yw[:-1]
        U.append(a[P:].copy())
        y.append(r)
    return U, y, Uw, yw, phys, L


def _tail(Uw, yw, P):
    """U (strict upper part), W and c of the last P rows, scaled by the pivots."""
    U = np.zeros((P, P), complex)
    W = np.zeros((P, P), complex)
    c = np.zeros(P, complex)
    for r in range(P):
        d = P - 1 - r
        rp = Uw[d][0]
        for k in range(P):
            if k > r:
                U[r, k] = rp * Uw[d][k - r]
            if k >= P - 1 - r:
                W[r, k] = rp * Uw[d][2 * P - 1 - r - k]
        c[r] = rp * yw[d]
    return U, W, c


def twisted_solve(band, b, P, m):
    """Solve A x = b; band[k, o] = A(k, k - P + o) (zero outside the matrix)."""
    n = band.shape[0]
    h1 = _half(band, b, P, m, False)
    h2 = _half(band, b, P, m, True)
    U1, W1, c1 = _tail(h1[2], h1[3], P)
    U2, W2, c2 = _tail(h2[2], h2[3], P)
    I = np.eye(P)
    z1 = np.linalg.solve(I + U1, c1)
    M1 = np.linalg.solve(I + U1, W1)
    T2 = np.linalg.solve(I + U2 - W2 @ M1, c2 - W2 @ z1)
    T1 = z1 - M1 @ T2
    x = np.zeros(n, complex)
    for (U, y, _, _, phys, L), Tp in ((h1, T2), (h2, T1)):
        xw = [Tp[P - 1 - c] for c in range(P)]   # this half's row L + c is the partner's tail row P-1-c
        for k in range(L - 1, -1, -1):
            v = y[k] - sum(U[k][q] * xw[q - 1] for q in range(1, P + 1))
            v *= U[k][0]
            xw = [v] + xw[:-1]
            x[phys(k)] = v
    return x
