"""The oracle against the reference's own analytic pins (tests/test_analytic.py,
tests/test_tsurff.py, tests/test_tensorops.py, tests/test_multigrid.py of the
TDSE-Z tree): closed forms and exact transfer-matrix energies."""
import json
import math
import os

import numpy as np
import pytest
import scipy.linalg as la

from oracle import bspline as ob
from oracle import multigrid as omg
from oracle import operators as oo
from oracle import propagate as op
from oracle import tsurff as ots

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
PINS = json.load(open(os.path.join(GOLDEN, "analytic_pins.json")))


def _eig(A, k):
    E = la.eigh(A.H.toarray(), A.M.toarray(), eigvals_only=True)
    return np.sort(E)[:k]


def test_infinite_well():
    """E_n = n^2 pi^2 / (2 L^2), Dirichlet walls, p = 7 (test_analytic.py:113-133)."""
    ax = ob.Axis(ob.uniform_knots(30, 0.0, 10.0, 7), 7, 10)
    A = oo.Assembled(ob.Space([ax]), oo.Physics(dim=1, potential=lambda x, y, z: 0.0, dirichlet=True))
    E = _eig(A, 4)
    exact = np.array(PINS["infinite_well"]["E"])
    assert np.max(np.abs(E - exact) / exact) < 1e-11


def test_double_quantum_well():
    """GaAs/AlGaAs double well with interface knots: exact BDD energies to
    1e-8 meV (test_analytic.py:193-219)."""
    pin = PINS["double_quantum_well"]
    NM = 18.8973
    a, b, L = 2 * NM, 10 * NM, 15 * NM
    mw, mb, V0 = 0.067, 0.0879, 0.00893
    mf = lambda x, y, z: 1.0 / (mb if abs(x) < a else (mw if abs(x) < b else mb))
    vf = lambda x, y, z: V0 if abs(x) < a else (0.0 if abs(x) < b else V0)
    ax = ob.Axis(ob.interface_knots(-L, L, 199, 7, [-b, -a, a, b]), 7, 9)
    A = oo.Assembled(ob.Space([ax]), oo.Physics(dim=1, potential=vf, inv_mass=mf, mass_const=None))
    E = _eig(A, 2) * pin["hartree_mev"]
    assert np.max(np.abs(E - np.array(pin["E_meV"]))) < 1e-8


@pytest.mark.parametrize("bc", ["Dirichlet", "Neumann"])
def test_mass_step(bc):
    """Mass step m = 1 | 4 with C0 interface knots (test_analytic.py:159-190)."""
    ax = ob.Axis(ob.interface_knots(-1.0, 1.0, 11, 7, [0.0]), 7, 10)
    ph = oo.Physics(dim=1, potential=lambda x, y, z: 0.0, inv_mass=lambda x, y, z: 1.0 if x < 0 else 0.25,
                    mass_const=None, dirichlet=(bc == "Dirichlet"))
    E = _eig(oo.Assembled(ob.Space([ax]), ph), 3)
    pin = PINS["mass_step"][bc]
    assert np.max(np.abs(E[:2] - np.array(pin["E"][:2]))) < 1e-10
    assert abs(E[2] - pin["E"][2]) < 1e-8


@pytest.mark.parametrize("kind,dt,order,tol", [("cn", 0.02, 2.0, 2e-3), ("magnus4", 0.2, 4.0, 2e-4)])
def test_driven_oscillator(kind, dt, order, tol):
    """Coherent state of the driven oscillator: accuracy, observed order and
    norm (test_analytic.py:226-273; p = 7, 200 elements on [-20, 20])."""
    ax = ob.Axis(ob.uniform_knots(120, -20.0, 20.0, 7), 7, 10)
    A = oo.Assembled(ob.Space([ax]), oo.Physics(dim=1, potential=lambda x, y, z: 0.5 * x * x))
    _, V = op.ground_state(A)
    xex = lambda t: -0.5 / (1 - 0.36) * (np.cos(0.6 * t) - np.cos(t))
    errs, norms = [], []
    for h in (dt, dt / 2):
        P = op.OraclePropagator(A, lambda t: [0.5 * np.cos(0.6 * t)], kind)
        _, out = P.evolve(V[:, 0], h, 10.0, lambda t, psi: (t, op.expect(A.D[0], psi).real,
                                                             op.expect(A.M, psi).real))
        out = np.array(out)
        errs.append(np.max(np.abs(out[:, 1] - xex(out[:, 0]))))
        norms.append(np.max(np.abs(out[:, 2] - 1)))
    assert errs[0] < tol
    assert abs(math.log2(errs[0] / errs[1]) - order) < 0.3
    assert max(norms) < 1e-9


def test_kron_equals_assembled():
    """Factorised (Kronecker) apply == assembled quadrature operator
    (test_tensorops.py:93-102, TDSEZTensorOps::Validate at 1e-10)."""
    from tests.cases import CASES, oracle_of
    for name in ("3d_heterostructure", "3d_const_mass_cap", "2d_cap_softcore_sep"):
        c = CASES[name]()
        S, ph, A = oracle_of(c)
        g, cc = 0.3 + 0.7j, [0.05 * (k + 1) for k in range(len(c["coupled"]))]
        terms = oo.kron_terms(S, ph, g=g, c=cc)
        x = np.random.default_rng(3).standard_normal(S.ndof) * (1 + 0.5j)
        ref = A.M @ x + g * (A.H_total() @ x + sum(ck * (T @ x) for ck, T in zip(cc, A.terms())))
        y = oo.kron_apply(S, terms, x)
        assert np.abs(y - ref).max() <= 1e-12 * np.abs(ref).max(), name


@pytest.mark.parametrize("knots,p", [
    (ob.uniform_knots(16, -1.0, 1.0, 3), 3),
    (ob.interface_knots(-12.0, 12.0, 15, 3, [-3.0, 2.0]), 3),
    (ob.symexp_knots(-60.0, 60.0, 31, 0.9, 4), 4),
])
def test_prolongation_exact(knots, p):
    """Partition of unity and linear precision of the Boehm prolongation
    (multigrid.cpp:280-293, 1e-10)."""
    C, dropped = omg.coarsen_knots(knots)
    assert dropped
    P = omg.prolongation(C, knots, p)
    assert np.abs(P.sum(1) - 1).max() < 1e-10
    assert np.abs(P @ omg.greville(C, p) - omg.greville(knots, p)).max() < 1e-10
    # C0 interface knots survive coarsening
    for u in set(knots):
        if list(knots).count(u) == p and u not in (knots[0], knots[-1]):
            assert list(C).count(u) == p


def test_tsurff_free_packet():
    """Free Gaussian packet, deck FREE1D of test_tsurff.py:20-52 (p = 7, 400
    elements on [-40, 40], Pade(2,2) dt = 0.025, T = 20, R = 10, CAP kmin 0.5):
    |b(k)|^2 against prod (2w^2/pi)^1/2 exp(-2w^2(k-k0)^2) at 1e-4 with the
    interior term (test_tsurff.py:82-90)."""
    p, L = 7, 40.0
    ax = ob.Axis(ob.uniform_knots(400, -L, L, p), p, 10)
    S = ob.Space([ax])
    A = oo.Assembled(S, oo.Physics(dim=1, potential=None, cap_kmin=0.5, bounds=[(-L, L)]))
    w, k0 = 1.0, 2.0
    g = lambda x: (2 * np.pi * w * w) ** -0.25 * np.exp(-x * x / (4 * w * w) + 1j * k0 * x)
    b = S.axes[0].basis_matrix(0).T @ (S.axes[0].wq.reshape(-1) * g(S.axes[0].xq.reshape(-1)))
    import scipy.sparse.linalg as sla
    psi = sla.spsolve(A.M.tocsc(), b)
    dt, T = 0.025, 20.0
    P = op.OraclePropagator(A, lambda t: [0.0], "pade22")
    ks = np.linspace(-1.0, 5.0, 61)
    ts = ots.OracleTSurff(S, 10.0, [ks], 1.0, 0.0, 1.0, lambda t: [0.0, 0.0, 0.0], dt)
    amp = np.zeros(len(ks), dtype=complex)
    amp = ts.add_flux(0.0, psi, [ks], amp)
    n = int(round(T / dt))
    for i in range(n):
        psi = P.step(psi, i * dt, dt)
        amp = ts.add_flux((i + 1) * dt, psi, [ks], amp)
    ex = (2 * w * w / np.pi) ** 0.5 * np.exp(-2 * w * w * (ks - k0) ** 2)
    tot = amp + ts.interior(psi, [ks])
    assert np.abs(np.abs(tot) ** 2 - ex).max() / ex.max() < 1e-4


@pytest.mark.parametrize("charge", [-1.0, 1.0])
def test_tsurff_field_mass_offset(charge):
    """Canonical momentum is conserved (test_tsurff.py:93-103): the FREE1D
    packet under the pulse 0.2 sin^2(pi t/15) sin(1.3 t) (t < 15), with mass
    0.5, a constant potential 0.3 (exterior potential s V = -q 0.3) and
    either carrier sign, stopped at T = 15: flux plus interior term give the
    field-free analytic spectrum to 2e-4 of its peak, and A(T) != 0."""
    import scipy.sparse.linalg as sla
    p, L = 7, 40.0
    ax = ob.Axis(ob.uniform_knots(400, -L, L, p), p, 10)
    S = ob.Space([ax])
    A = oo.Assembled(S, oo.Physics(dim=1, charge=charge, potential=lambda x, y, z: 0.3, mass_const=0.5,
                                   cap_kmin=0.5, bounds=[(-L, L)]))

    def field(t):
        return [0.2 * math.sin(math.pi * t / 15) ** 2 * math.sin(1.3 * t) if t < 15 else 0.0]
    w, k0 = 1.0, 2.0
    g = (2 * np.pi * w * w) ** -0.25 * np.exp(-ax.xq.reshape(-1) ** 2 / (4 * w * w) + 1j * k0 * ax.xq.reshape(-1))
    psi = sla.spsolve(A.M.tocsc().astype(complex), ax.basis_matrix(0).T @ (ax.wq.reshape(-1) * g))
    dt, T = 0.025, 15.0
    ks = np.linspace(-1.0, 5.0, 61)
    s = -charge
    ts = ots.OracleTSurff(S, 10.0, [ks], 0.5, s * 0.3, s, lambda t: [field(t)[0], 0.0, 0.0], dt)
    amp = ts.add_flux(0.0, psi, [ks], np.zeros(len(ks), dtype=complex))

    def observe(t, x):
        nonlocal amp
        if t > 0:
            amp = ts.add_flux(t, x, [ks], amp)
    psi, _ = op.OraclePropagator(A, field, "pade22").evolve(psi, dt, T, observe=observe)
    tot = amp + ts.interior(psi, [ks])
    ex = (2 * w * w / np.pi) ** 0.5 * np.exp(-2 * w * w * (ks - k0) ** 2)
    err = np.abs(np.abs(tot) ** 2 - ex).max() / ex.max()
    print("charge", charge, "spectrum error", err, "A(T)", ts.A[0])
    assert err < 2e-4, err
    assert abs(ts.A[0]) > 1e-3


def test_quesne_position_dependent_mass():
    """Quesne oscillator (test_analytic.py:136-157): m(x) = (1 + x/2)^-1,
    V = x^2 / (4 (x + 2)) on [-1.999999999, 50] with Dirichlet walls, p = 7,
    1000 elements, 10 Gauss points: E_n = (n + 1/2) / 2 to 1e-9."""
    ax = ob.Axis(ob.uniform_knots(1000, -1.999999999, 50.0, 7), 7, 10)
    A = oo.Assembled(ob.Space([ax]), oo.Physics(dim=1, potential=lambda x, y, z: x * x / (4.0 * (x + 2.0)),
                                                inv_mass=lambda x, y, z: 1.0 + x / 2.0, mass_const=None,
                                                mass_axis=0, dirichlet=True))
    E = _eig(A, 5)
    assert np.abs(E - 0.5 * (np.arange(5) + 0.5)).max() < 1e-9, E


def test_hole_inverts_potential_and_coupling():
    """Charge +1 (test_analytic.py:276-296): H = K - (V + x E) with
    V = -x^2/2 is the oscillator for the hole (E = 1/2, 3/2, 5/2), and the
    drive 0.5 cos(0.6 t) pushes it the other way: the dipole q<x> = +<x>
    follows +0.5/(1 - 0.36) (cos 0.6t - cos t) to 1e-4 (Magnus-4, dt 0.05,
    T = 20)."""
    ax = ob.Axis(ob.uniform_knots(120, -20.0, 20.0, 7), 7, 10)
    A = oo.Assembled(ob.Space([ax]), oo.Physics(dim=1, charge=1.0, potential=lambda x, y, z: -0.5 * x * x))
    assert np.abs(_eig(A, 3) - [0.5, 1.5, 2.5]).max() < 1e-8
    _, V = op.ground_state(A, 0.5)
    P = op.OraclePropagator(A, lambda t: [0.5 * np.cos(0.6 * t)], "magnus4")
    _, out = P.evolve(V[:, 0], 0.05, 20.0, lambda t, psi: (t, op.expect(A.D[0], psi).real))
    out = np.array(out)
    x = 0.5 / (1 - 0.36) * (np.cos(0.6 * out[:, 0]) - np.cos(out[:, 0]))
    assert np.abs(1.0 * out[:, 1] - x).max() < 1e-4


def test_tsurff_free_packet_2d():
    """2D deck of test_tsurff.py:122-153: packet with momentum (2, 1) and
    widths 1 on [-20, 20]^2, 60 elements of degree 4 per axis, CN dt 0.02 to
    T = 2, CAP k_min 1, R = 6, 31 x 31 momenta on [-1, 5] x [-2, 4]: flux
    plus interior term against the analytic spectrum, 5e-3 of its peak."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla
    p, L = 4, 20.0
    axes = [ob.Axis(ob.uniform_knots(60, -L, L, p), p, 6) for _ in range(2)]
    S = ob.Space(axes)
    A = oo.Assembled(S, oo.Physics(dim=2, potential=None, cap_kmin=1.0, bounds=[(-L, L)] * 2, coupled=(0, 1)))
    w, k0 = 1.0, (2.0, 1.0)
    part = []
    for d, ax in enumerate(axes):
        x = ax.xq.reshape(-1)
        g = (2 * np.pi * w * w) ** -0.25 * np.exp(-x * x / (4 * w * w) + 1j * k0[d] * x)
        B = ax.basis_matrix(0)
        Md = (B.T @ sp.diags(ax.wq.reshape(-1)) @ B).tocsc()
        part.append(sla.spsolve(Md.astype(complex), ax.basis_matrix(0).T @ (ax.wq.reshape(-1) * g)))
    psi = np.kron(part[1], part[0])          # x fastest
    ks = [np.linspace(-1.0, 5.0, 31), np.linspace(-2.0, 4.0, 31)]
    dt, T = 0.02, 2.0
    ts = ots.OracleTSurff(S, 6.0, ks, 1.0, 0.0, 1.0, lambda t: [0.0, 0.0, 0.0], dt)
    amp = ts.add_flux(0.0, psi, ks, np.zeros(31 * 31, dtype=complex))

    def observe(t, x):
        nonlocal amp
        if t > 0:
            amp = ts.add_flux(t, x, ks, amp)
    psi, _ = op.OraclePropagator(A, lambda t: [0.0, 0.0], "cn").evolve(psi, dt, T, observe=observe)
    tot = amp + ts.interior(psi, ks)
    kx, ky = np.meshgrid(ks[0], ks[1], indexing="ij")
    ex = ((2 * w * w / np.pi) * np.exp(-2 * w * w * ((kx - k0[0]) ** 2 + (ky - k0[1]) ** 2))).reshape(-1)
    err = np.abs(np.abs(tot) ** 2 - ex).max() / ex.max()
    print("2D spectrum error", err)
    assert err < 5e-3, err
