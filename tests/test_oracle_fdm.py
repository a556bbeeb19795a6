"""The algebra of the fast-diagonalisation inverse with complex symmetric
axis pencils, restated in numpy on the oracle's assembled matrices: for a
separable 2D stage operator with absorbing layers on both axes,
A = (B_y + lam_i C_y) in the eigenbasis of the x pencil (S_x, M_x) with
V^T M_x V = I, V^T S_x V = diag(lam) (bilinear form), so one transform, one
banded solve per line and the inverse transform give A^-1 b exactly; the
same for the end term's indefinite stage E M - H. This is the factorisation
fdm.cu applies (complex lam in the line shifts, V and V^T as complex
matrices)."""
import numpy as np
import pytest
import scipy.linalg as sl

from oracle import bspline as ob
from oracle import operators as oo


def _axis(p, L, nel, kmin):
    S = ob.Space([ob.Axis(ob.uniform_knots(nel, -L, L, p), p, p + 2)])
    A = oo.Assembled(S, oo.Physics(dim=1, cap_kmin=kmin, bounds=[(-L, L)], coupled=(0,)))
    return A.M.toarray(), A.H_total().toarray()


@pytest.mark.parametrize("alpha,g", [(1.0, 0.25j), (0.8, -1.0)])
def test_complex_pencil_fdm_is_exact(alpha, g):
    Mx, Hx = _axis(3, 18.0, 18, 1.0)        # x: 21 B-splines, absorbing layers at both ends
    My, Hy = _axis(3, 16.0, 15, 1.0)        # y (outer): 18 B-splines
    lam, V = sl.eig(Hx, Mx)
    for i in range(V.shape[1]):              # bilinear scaling v^T M v = 1
        V[:, i] /= np.sqrt(V[:, i] @ Mx @ V[:, i])
    assert np.abs(V.T @ Mx @ V - np.eye(len(lam))).max() < 1e-9
    # A = alpha M_y (x) M_x + g (H_y (x) M_x + M_y (x) H_x), y outer (index = y n_x + x)
    A = alpha * np.kron(My, Mx) + g * (np.kron(Hy, Mx) + np.kron(My, Hx))
    b = np.random.default_rng(3).standard_normal(A.shape[0]) + 0j
    nx = len(lam)
    T = b.reshape(-1, nx) @ V                     # forward transform along x: V^T per row
    X = np.empty_like(T)
    for i in range(nx):                           # one line per eigenvalue: B_y + lam_i C_y
        X[:, i] = np.linalg.solve(alpha * My + g * Hy + g * lam[i] * My, T[:, i])
    x = (X @ V.T).reshape(-1)                     # inverse transform: V per row
    xd = np.linalg.solve(A, b)
    assert np.linalg.norm(x - xd) / np.linalg.norm(xd) < 1e-9
