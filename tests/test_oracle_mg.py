"""Preconditioner independence on the oracle (the reference's `mg == asm`
pin, tests/test_multigrid.py:54-64 of TDSE-Z): GMRES with a geometric
B-spline multigrid V-cycle built from the oracle's knot hierarchy, Boehm
prolongations and Galerkin coarse operators reaches the same stage solution
as GMRES with an incomplete LU, and as a direct solve, to 1e-9. (The
Gauss-Seidel V-cycle here only checks the hierarchy; the GPU multigrid's
smoother and iteration counts are tested in tests/test_gpu_solve.py.)"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as sla

from oracle import multigrid as omg
from tests.cases import CASES, oracle_of


def _vcycle_operator(A, Ps):
    """V(1,1) cycle with symmetric Gauss-Seidel sweeps; exact coarsest solve."""
    levels = [A.tocsr()]
    for P in Ps:
        levels.append((P.T @ levels[-1] @ P).tocsr())
    lu = sla.splu(levels[-1].tocsc())
    tri = [(sp.tril(L, format="csr"), sp.triu(L, format="csr")) for L in levels[:-1]]

    def cycle(l, b):
        if l == len(levels) - 1:
            return lu.solve(b)
        L, U = tri[l]
        A_l = levels[l]
        x = sla.spsolve_triangular(L, b, lower=True)
        x = x + sla.spsolve_triangular(U, b - A_l @ x, lower=False)
        r = b - A_l @ x
        x = x + Ps[l] @ cycle(l + 1, Ps[l].T @ r)
        x = x + sla.spsolve_triangular(U, b - A_l @ x, lower=False)
        x = x + sla.spsolve_triangular(L, b - A_l @ x, lower=True)
        return x
    return sla.LinearOperator(A.shape, lambda b: cycle(0, np.asarray(b).ravel()), dtype=np.complex128)


def test_mg_equals_ilu_and_direct():
    c = CASES["2d_cap_softcore_sep"]()
    S, ph, A = oracle_of(c)
    tau = 0.2
    cc = [0.02 * (k + 1) for k in range(len(c["coupled"]))]
    Am = (A.M + 1j * tau * (A.H_total() + sum(ck * T for ck, T in zip(cc, A.terms())))).tocsr()
    K = omg.hierarchy(c["knots"], c["p"], levels=3)
    assert len(K) >= 2
    Ps = []
    for f, g in zip(K[:-1], K[1:]):
        Ps.append(omg.kron_prolongation([sp.csr_matrix(omg.prolongation(np.asarray(g[d]), np.asarray(f[d]), c["p"]))
                                         for d in range(S.dim)]))
    rng = np.random.default_rng(5)
    b = rng.standard_normal(S.ndof) + 1j * rng.standard_normal(S.ndof)
    xd = sla.spsolve(Am.tocsc(), b)
    its = {}

    def solve(M, key):
        cnt = [0]
        x, info = sla.gmres(Am, b, rtol=1e-12, atol=0.0, restart=30, maxiter=300, M=M,
                            callback=lambda _: cnt.__setitem__(0, cnt[0] + 1), callback_type="pr_norm")
        assert info == 0
        its[key] = cnt[0]
        return x
    x_mg = solve(_vcycle_operator(Am, Ps), "mg")
    ilu = sla.spilu(Am.tocsc(), drop_tol=1e-4, fill_factor=2.0)
    x_ilu = solve(sla.LinearOperator(Am.shape, ilu.solve, dtype=np.complex128), "ilu")
    rel = lambda u, v: np.linalg.norm(u - v) / np.linalg.norm(v)
    assert rel(x_mg, x_ilu) < 1e-9 and rel(x_mg, xd) < 1e-9, (rel(x_mg, x_ilu), rel(x_mg, xd), its)
