"""Bound states on the GPU (tdz_eigen_solve) against the oracle's FP64
eigensolve of the assembled matrices (oracle.propagate.ground_state):
energies within 1e-10 relative, eigenvectors up to phase within 1e-7, and
the reference's acceptance bar, backward error <= 1e-8 (src/core.cpp:814)."""
import numpy as np
import pytest

from tests.cases import CASES, oracle_of, product_of


def _check(name, nev, target, **inner):
    import torch
    from oracle.propagate import ground_state
    from tdsez_gb300.eigen import bound_states
    c = CASES[name]()
    S, ph, A = oracle_of(c)
    PS, op = product_of(c)
    E_ref, V_ref = ground_state(A, target=target, k=nev)
    E, V, berr, solves = bound_states(op, nev=nev, target=target, tol=1e-11, **inner)
    print(name, "E", E, "oracle", list(E_ref), "backward errors", berr, "inner solves", solves)
    for i in range(nev):
        assert abs(E[i] - E_ref[i]) <= 1e-10 * max(1.0, abs(E_ref[i])), (i, E[i], E_ref[i])
        assert berr[i] <= 1e-8, berr
        v = V[i].cpu().numpy()
        ov = np.vdot(V_ref[:, i], A.M @ v)
        assert abs(abs(ov) - 1.0) < 1e-9, ov
        assert np.linalg.norm(v - ov * V_ref[:, i]) / np.linalg.norm(v) < 1e-7
    return solves


@pytest.mark.gpu
def test_ground_state_heterostructure_fdm(cuda):
    """z-layered 3D heterostructure, FDM inverse inside the shift-invert
    solves (exact for this operator family)."""
    _check("3d_heterostructure", 3, -0.3)


@pytest.mark.gpu
def test_ground_state_heterostructure_mg(cuda):
    """The same with the multigrid V-cycle; target below the spectrum, so
    H - s M is positive definite."""
    _check("3d_heterostructure", 2, -0.3, pc="mg", precision="fp32", rtol=1e-11, outer="df")


@pytest.mark.gpu
def test_ground_state_1d_oscillator(cuda):
    """The 1D harmonic oscillator with Dirichlet walls of the plain CPU
    configuration (p = 5): E_n = n + 1/2 to the discretisation error, and
    the oracle's values to 1e-10."""
    _check("1d_dirichlet_ho", 3, 0.0, pc="mass", precision="fp64", rtol=1e-12, maxit=2000)


@pytest.mark.gpu
def test_ground_state_softcore_3d(cuda):
    """Non-separable soft-core potential (per-element quadrature term),
    multigrid preconditioner, ground state nearest -0.7 Ha."""
    _check("3d_softcore", 1, -0.7, pc="mg", precision="fp32", rtol=1e-11, outer="df")
