"""The two-sided banded solve of the FDM line solves (oracle restatement)
against a dense solve, for degrees 2..5, several lengths and cut positions."""
import numpy as np
import pytest

from oracle.twisted_lines import twisted_solve


@pytest.mark.parametrize("P", [2, 3, 4, 5])
@pytest.mark.parametrize("n,m", [(32, 16), (41, 24), (64, 32), (77, 40)])
def test_twisted_solve(P, n, m):
    rng = np.random.default_rng(100 * P + n)
    A = np.zeros((n, n), complex)
    for o in range(0, P + 1):
        d = rng.standard_normal(n - o) + 1j * rng.standard_normal(n - o)
        A += np.diag(d, o) + (np.diag(d, -o) if o else 0)
    A += np.eye(n) * (4.0 * P + 4.0)           # no pivoting needed
    band = np.zeros((n, 2 * P + 1), complex)
    for k in range(n):
        for o in range(2 * P + 1):
            j = k - P + o
            if 0 <= j < n:
                band[k, o] = A[k, j]
    b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    x = twisted_solve(band, b, P, m)
    xr = np.linalg.solve(A, b)
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < 1e-12
