"""The plain CPU configuration end to end on the GPU, against the oracle:
1D harmonic oscillator V = x^2/2 on [-20, 20], 400 uniform elements of
degree 5, Dirichlet walls, 6 Gauss points per element; the ground state by
the GPU shift-invert eigensolver (banded-LU inner solves); then Crank-
Nicolson with dt = 0.05 over T = 2 * 2 pi / 0.057 (4410 steps, the last one
shortened) under E(t) = 0.01 sin^2(pi t / T) cos(0.057 t) along x, the
observables recorded every step into the observables file by the GPU
monitor. The oracle: dense generalised eigensolve and CN by direct sparse
solves of the assembled FP64 matrices. Each GPU step is solved to a
relative residual of 1e-12 and |eigenvalues of M^-1 (M + i dt/2 H)| >= 1,
so the state error stays below 4410 x 1e-12; the file's dipole series
(peak 1e-2), ground-state population and autocorrelation agree with the
oracle's to 1e-8. Both propagations start from the GPU's ground state,
checked against the oracle's eigenvector first."""
import math

import numpy as np
import pytest

from oracle import bspline as ob
from tests import h5lite
from tests.cases import oracle_of, product_of


def _case():
    return dict(knots=[ob.uniform_knots(400, -20.0, 20.0, 5)], p=5, nq=6, charge=-1.0, mass=1.0,
                V=[lambda x: 0.5 * x * x], coupled=(0,), dirichlet=True)


@pytest.mark.gpu
def test_plain_configuration_end_to_end(cuda, tmp_path):
    from oracle.propagate import OraclePropagator, ground_state
    from tdsez_gb300.eigen import bound_states
    from tdsez_gb300.outputs import ObservablesMonitor
    from tdsez_gb300.propagator import Propagator
    c = _case()
    S, ph, A = oracle_of(c)
    PS, op = product_of(c)
    assert S.ndof == 405
    T, dt = 2 * 2 * math.pi / 0.057, 0.05

    def field(t):
        return [0.01 * math.sin(math.pi * t / T) ** 2 * math.cos(0.057 * t)]

    E_ref, V_ref = ground_state(A, 0.0, 1)
    E, V, berr, _ = bound_states(op, nev=1, target=0.0, tol=1e-11, pc="band", precision="fp64", rtol=1e-12)
    assert abs(E[0] - E_ref[0]) <= 1e-10 and berr[0] <= 1e-8
    assert abs(E[0] - 0.5) < 1e-8           # E_0 = 1/2 to the discretisation error

    # both propagations start from the GPU's ground state, which the eigensolve
    # delivers to its own accuracy (backward error 1e-11): compare it once here
    phi0 = V[0].cpu().numpy()
    ov = np.vdot(V_ref[:, 0], A.M @ phi0)
    assert abs(abs(ov) - 1.0) < 1e-9 and np.linalg.norm(phi0 - ov * V_ref[:, 0]) < 1e-7 * np.linalg.norm(phi0)
    ref = []

    def observe(t, x):
        ref.append((t, np.vdot(x, A.D[0] @ x).real, np.vdot(x, A.M @ x).real, np.vdot(phi0, A.M @ x)))
    OraclePropagator(A, field, "cn").evolve(phi0.copy(), dt, T, observe=observe)

    path = tmp_path / "td" / "ho_observables.h5"
    psi = V[0].clone()
    mon = ObservablesMonitor(path, op, field=field, charge=-1.0, bound=[V[0].clone()])
    G = Propagator(op, "cn", field=field, pc="band", precision="fp64", rtol=1e-12)
    G.evolve(psi, dt, T, monitor=mon)
    mon.close()
    f = h5lite.File(str(path))
    dip, ene, pop, auto = (f[s].read() for s in ("dipoles", "energies", "populations", "autocorrelation"))
    assert dip.shape == (4411, 4) and pop.shape == (4411, 2)
    t_ref = np.array([r[0] for r in ref])
    assert np.array_equal(dip[:, 0], t_ref) and dip[-1, 0] == T
    assert np.array_equal(dip[:, 1], [field(t)[0] for t in t_ref])
    d_ref = -np.array([r[1] for r in ref])                      # D_x = q <x>, q = -1
    assert np.abs(d_ref).max() > 5e-3
    err = np.abs(dip[:, 2] - d_ref).max()
    print("plain configuration: max dipole error", err, "of", np.abs(d_ref).max())
    assert err <= 1e-8
    assert np.abs(ene[:, 6] - np.array([r[2] for r in ref])).max() <= 1e-8
    c_ref = np.array([r[3] for r in ref])
    pe, ae = np.abs(pop[:, 1] - np.abs(c_ref) ** 2).max(), np.abs(auto[:, 1] + 1j * auto[:, 2] - c_ref).max()
    print("population error", pe, "autocorrelation error", ae)
    assert pe <= 1e-8 and ae <= 1e-8
