"""GPU stage solves and time steps against the oracle (direct sparse solves
of the assembled FP64 matrices), through the C ABI."""
import math

import numpy as np
import pytest
import scipy.sparse.linalg as sla

from tests.cases import CASES, oracle_of, product_of


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _berr(Am, x, b):
    """Normwise backward error ||b - A x|| / (||b|| + || |A| |x| ||): the
    measure that does not charge the solver for the rounding-level difference
    between the oracle's assembled matrix and the library's operator, which
    ||A|| ||x|| / ||b|| magnifies for stiff (high-degree) cases."""
    return np.linalg.norm(b - Am @ x) / (np.linalg.norm(b) + np.linalg.norm(abs(Am) @ np.abs(x)))


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["3d_heterostructure", "3d_const_mass_cap", "2d_cap_softcore_sep", "3d_p2_hole",
                                  "3d_softcore"])
@pytest.mark.parametrize("pc,prec,outer", [("mg", "fp32", "fp64"), ("mg", "fp64", "fp64"), ("mass", "fp32", "fp64"),
                                           ("mass", "fp64", "fp64"), ("mg", "fp32", "df")])
def test_stage_solve_parity(cuda, name, pc, prec, outer):
    """FGMRES + (mixed-precision) preconditioner reaches the FP64 solution of
    (M + i tau H_E) x = b: true residual of the oracle matrix <= 1e-11, also
    when the Krylov method's applies run in double-float arithmetic."""
    import torch
    from tdsez_gb300.propagator import Solver
    c = CASES[name]()
    S, ph, A = oracle_of(c)
    PS, op = product_of(c)
    tau = 0.2
    cc = [0.02 * (k + 1) for k in range(len(c["coupled"]))]
    op.set_stage(1.0, 1j * tau, cc)
    Am = (A.M + 1j * tau * (A.H_total() + sum(ck * T for ck, T in zip(cc, A.terms())))).tocsc()
    rng = np.random.default_rng(3)
    b = rng.standard_normal(S.ndof) + 1j * rng.standard_normal(S.ndof)
    xref = sla.spsolve(Am, b)
    s = Solver(op, pc=pc, precision=prec, rtol=1e-12, maxit=400, outer=outer)
    bd = torch.tensor(b, device=cuda)
    xd = torch.zeros_like(bd)
    its, reason, rn = s.solve(bd, xd)
    x = xd.cpu().numpy()
    assert reason > 0, (its, reason, rn)
    # the solver's own criterion, or (ill-conditioned soft-core system, ||x|| / ||b|| ~ 1e2,
    # after many restarted iterations of the weak mass preconditioner) rounding-level backward error
    rres = np.linalg.norm(b - Am @ x) / np.linalg.norm(b)
    assert rres < 1e-11 or _berr(Am, x, b) < 1e-13, (rres, _berr(Am, x, b))
    assert _rel(x, xref) < 1e-9
    if pc == "mg":
        # 3d_const_mass_cap has under 2000 DoFs: one level, whose coarse solve
        # is the Chebyshev polynomial (the reference factorises it with LU)
        assert its <= (100 if name == "3d_const_mass_cap" else 60), its


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["3d_heterostructure", "3d_p2_hole", "3d_p5_sym", "2d_cap_softcore_sep",
                                  "3d_softcore"])
def test_fdm_solve(cuda, name):
    """Fast-diagonalisation preconditioner: exact (FP32) for operators whose
    inner axes carry only mass and stiffness (heterostructure), approximate
    otherwise; FGMRES reaches the FP64 solution either way."""
    import torch
    from tdsez_gb300.propagator import Solver
    c = CASES[name]()
    S, ph, A = oracle_of(c)
    PS, op = product_of(c)
    tau = 0.2
    cc = [0.02 * (k + 1) for k in range(len(c["coupled"]))]
    op.set_stage(1.0, 1j * tau, cc)
    Am = (A.M + 1j * tau * (A.H_total() + sum(ck * T for ck, T in zip(cc, A.terms())))).tocsc()
    rng = np.random.default_rng(8)
    b = rng.standard_normal(S.ndof) + 1j * rng.standard_normal(S.ndof)
    s = Solver(op, pc="fdm", precision="fp32", rtol=1e-12, maxit=400)
    bd = torch.tensor(b, device=cuda)
    xd = torch.zeros_like(bd)
    its, reason, rn = s.solve(bd, xd)
    x = xd.cpu().numpy()
    assert reason > 0, (its, reason, rn)
    assert _berr(Am, x, b) < 1e-12, _berr(Am, x, b)
    if name == "3d_heterostructure":
        assert its <= 4, its            # exact inverse up to FP32: one digit group per iteration


@pytest.mark.gpu
@pytest.mark.parametrize("name,cc,cap", [("3d_heterostructure", [0.02], None), ("3d_const_mass_cap", [0.0, 0.02], 4),
                                         ("2d_cap_free", [0.0], None)])
def test_mg_exact_coarse_solve(cuda, name, cc, cap):
    """The coarsest multigrid level solved by the FDM inverse (mg_coarse =
    "fdm", in the role of the reference's coarse LU): the same FP64
    solution, in no more FGMRES iterations than with the Chebyshev coarse
    polynomial. The 3D CAP case's knots admit no coarser level, so its
    V-cycle becomes the exact inverse (81 iterations with the polynomial)."""
    import torch
    from tdsez_gb300.propagator import Solver
    c = CASES[name]()
    S, ph, A = oracle_of(c)
    PS, op = product_of(c)
    tau = 0.2
    op.set_stage(1.0, 1j * tau, cc)
    Am = (A.M + 1j * tau * (A.H_total() + sum(ck * T for ck, T in zip(cc, A.terms())))).tocsc()
    rng = np.random.default_rng(11)
    b = rng.standard_normal(S.ndof) + 1j * rng.standard_normal(S.ndof)
    xref = sla.spsolve(Am, b)
    bd = torch.tensor(b, device=cuda)
    its = {}
    for coarse in ("chebyshev", "fdm"):
        s = Solver(op, pc="mg", precision="fp32", rtol=1e-12, maxit=400, mg_coarse=coarse)
        xd = torch.zeros_like(bd)
        its[coarse], reason, rn = s.solve(bd, xd)
        assert reason > 0, (coarse, its, reason)
        assert _rel(xd.cpu().numpy(), xref) < 1e-9
    print(name, its)
    assert its["fdm"] <= its["chebyshev"], its
    if cap is not None:
        assert its["fdm"] <= cap, its


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp32", "fp64"])
@pytest.mark.parametrize("name,cc", [("2d_cap_free", [0.0]), ("2d_cap_softcore_sep", [0.0]),
                                     ("3d_const_mass_cap", [0.0, 0.03])])
def test_fdm_complex_pencils(cuda, name, cc, prec):
    """Absorbing layers (and separable potentials) on the inner axes enter the
    fast-diagonalisation inverse through complex symmetric axis pencils
    S_d = K_d + V_d - i W_d with V^T M V = I: with no field along an inner
    axis the inverse is exact to FP32, so FGMRES needs one digit group per
    iteration, and reaches the direct solution."""
    import torch
    from tdsez_gb300.propagator import Solver
    c = CASES[name]()
    S, ph, A = oracle_of(c)
    PS, op = product_of(c)
    tau = 0.2
    op.set_stage(1.0, 1j * tau, cc)
    Am = (A.M + 1j * tau * (A.H_total() + sum(ck * T for ck, T in zip(cc, A.terms())))).tocsc()
    rng = np.random.default_rng(9)
    b = rng.standard_normal(S.ndof) + 1j * rng.standard_normal(S.ndof)
    s = Solver(op, pc="fdm", precision=prec, rtol=1e-12, maxit=100)
    bd = torch.tensor(b, device=cuda)
    xd = torch.zeros_like(bd)
    its, reason, rn = s.solve(bd, xd)
    x = xd.cpu().numpy()
    assert reason > 0, (its, reason, rn)
    assert _berr(Am, x, b) < 1e-12, _berr(Am, x, b)
    assert its <= (4 if prec == "fp32" else 2), its
    # the end term's indefinite stage E M - H as well
    E = 0.6
    op.set_stage(E, -1.0, [0.0] * len(cc))
    Ah = (E * A.M - A.H_total()).tocsc()
    xref = sla.spsolve(Ah, b)
    xd.zero_()
    its, reason, rn = s.solve(bd, xd)
    assert reason > 0 and its <= (6 if prec == "fp32" else 2), (its, reason)
    assert _rel(xd.cpu().numpy(), xref) < 1e-9


@pytest.mark.gpu
@pytest.mark.parametrize("p,nel_z", [(2, 62), (2, 80), (3, 29), (3, 45), (3, 61), (4, 40), (5, 33), (5, 57)])
def test_fdm_line_solve_lengths(cuda, p, nel_z):
    """FDM inverse on z-layered operators with long z axes (the two-thread line
    solve, twist and ragged last blocks on either side): P^-1 b equals the
    direct FP64 solve to FP32 accuracy, and FGMRES converges in a few
    iterations to 1e-12."""
    import torch
    from tdsez_gb300.propagator import Solver
    from tests.cases import heterostructure_lines
    c = heterostructure_lines(p, nel_z)
    S, ph, A = oracle_of(c)
    PS, op = product_of(c)
    tau = 0.25
    op.set_stage(1.0, 1j * tau, [0.01])
    Am = (A.M + 1j * tau * (A.H_total() + 0.01 * A.terms()[0])).tocsc()
    rng = np.random.default_rng(p * 100 + nel_z)
    b = rng.standard_normal(S.ndof) + 1j * rng.standard_normal(S.ndof)
    xref = sla.spsolve(Am, b)
    s = Solver(op, pc="fdm", precision="fp32", rtol=1e-12, maxit=50)
    bd = torch.tensor(b, device=cuda)
    zd = torch.empty_like(bd)
    s.precondition(bd, zd)
    err = _rel(zd.cpu().numpy(), xref)
    assert err < 1e-4, err
    xd = torch.zeros_like(bd)
    its, reason, rn = s.solve(bd, xd)
    assert reason > 0 and its <= 4, (its, reason, rn)
    assert _berr(Am, xd.cpu().numpy(), b) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["3d_heterostructure", "2d_cap_softcore_sep", "3d_const_mass_cap", "2d_softcore",
                                  "3d_two_centres_p3"])
@pytest.mark.parametrize("kind", ["cn", "pade22", "magnus4"])
def test_propagation_parity(cuda, name, kind):
    """Several steps with a time-dependent field: GPU state == oracle state."""
    import torch
    from oracle.propagate import OraclePropagator
    from tdsez_gb300.propagator import Propagator
    c = CASES[name]()
    S, ph, A = oracle_of(c)
    PS, op = product_of(c)
    ncpl = len(c["coupled"])
    field = lambda t: [0.05 * math.sin(0.3 * t + k) for k in range(ncpl)]
    rng = np.random.default_rng(9)
    psi0 = rng.standard_normal(S.ndof) + 1j * rng.standard_normal(S.ndof)
    psi0 /= math.sqrt(np.vdot(psi0, A.M @ psi0).real)
    P = OraclePropagator(A, field, kind)
    G = Propagator(op, kind, field=field, pc="mg", precision="fp32", rtol=1e-12)
    dt = 0.1
    psi = psi0.copy()
    pd = torch.tensor(psi0, device=cuda)
    for step in range(6):
        psi = P.step(psi, step * dt, dt)
        G.step(pd, step * dt, dt)
    assert _rel(pd.cpu().numpy(), psi) < 1e-9
    st = G.stats()
    assert st["solves"] == 6 * {"cn": 1, "pade22": 2, "magnus4": 4}[kind]
    assert st["last_rres"] <= 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("kind,dt,order,tol", [("cn", 0.02, 2.0, 2e-3), ("magnus4", 0.2, 4.0, 2e-4)])
def test_driven_oscillator_gpu(cuda, kind, dt, order, tol):
    """Driven harmonic oscillator (test_analytic.py:226-273) on the GPU:
    accuracy against the coherent-state <x>(t), observed order, norm 1e-9."""
    import torch
    from oracle import bspline as ob
    from oracle import operators as oo
    from oracle.propagate import ground_state
    from tdsez_gb300 import _lib
    from tdsez_gb300.operators import Operator, Physics
    from tdsez_gb300.propagator import Propagator
    from tdsez_gb300.space import Space
    kn = ob.uniform_knots(120, -20.0, 20.0, 7)
    A = oo.Assembled(ob.Space([ob.Axis(kn, 7, 10)]), oo.Physics(dim=1, potential=lambda x, y, z: 0.5 * x * x))
    _, V = ground_state(A)
    S = Space([kn], 7, 10)
    op = Operator(S, Physics(potential=[lambda x: 0.5 * x * x], coupled=(0,)))
    xex = lambda t: -0.5 / (1 - 0.36) * (np.cos(0.6 * t) - np.cos(t))
    errs, norms = [], []
    for h in (dt, dt / 2):
        G = Propagator(op, kind, field=lambda t: [0.5 * math.cos(0.6 * t)], pc="mg", precision="fp32")
        psi = torch.tensor(V[:, 0], device=cuda)
        dx = torch.empty_like(psi)
        mx = torch.empty_like(psi)
        out = []

        def mon(step, t, p):
            op.apply(_lib.TDZ_DIPOLE_X, p, dx)
            op.apply(_lib.TDZ_MASS, p, mx)
            out.append((t, torch.vdot(p, dx).real.item(), torch.vdot(p, mx).real.item()))
        G.evolve(psi, h, 10.0, mon)
        o = np.array(out)
        errs.append(np.max(np.abs(o[:, 1] - xex(o[:, 0]))))
        norms.append(np.max(np.abs(o[:, 2] - 1)))
    assert errs[0] < tol
    assert abs(math.log2(errs[0] / errs[1]) - order) < 0.3
    assert max(norms) < 1e-9


@pytest.mark.gpu
def test_failed_solve_is_a_status(cuda):
    """A stage solve that cannot converge returns TDZ_ERR_NOT_CONVERGED (the
    PetscCheck(reason > 0) of propagator.cpp:671-672); a NaN state returns a
    breakdown status. The failure is made on the host: an iteration cap of 1
    and a NaN input, no device fault."""
    import torch
    from tdsez_gb300 import _lib
    from tdsez_gb300.propagator import Propagator
    c = CASES["3d_heterostructure"]()
    PS, op = product_of(c)
    G = Propagator(op, "cn", field=lambda t: [0.0], pc="none", maxit=1, rtol=1e-14)
    psi = torch.randn(PS.ndof, dtype=torch.complex128, device=cuda)
    with pytest.raises(_lib.TDZError) as e:
        G.step(psi, 0.0, 0.5)
    assert e.value.status == 3
    G2 = Propagator(op, "cn", field=lambda t: [0.0], pc="mass")
    psi[5] = float("nan")
    with pytest.raises(_lib.TDZError) as e:
        G2.step(psi, 0.0, 0.5)
    assert e.value.status == 6
    # the library stays usable afterwards
    psi = torch.randn(PS.ndof, dtype=torch.complex128, device=cuda)
    G2.step(psi, 0.0, 0.5)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["3d_heterostructure", "3d_softcore", "2d_cap_softcore_sep"])
@pytest.mark.parametrize("pc", ["fdm", "mg"])
def test_relaxed_arnoldi_solve(cuda, name, pc):
    """Relaxed (inexact) Krylov: Arnoldi applies in FP32, every restart
    residual in double-float. The answer is still the FP64 solution: true
    residual of the oracle matrix <= 1e-11, and the reported residual is a
    true one."""
    import torch
    from tdsez_gb300.propagator import Solver
    c = CASES[name]()
    S, ph, A = oracle_of(c)
    PS, op = product_of(c)
    tau = 0.2
    cc = [0.02 * (k + 1) for k in range(len(c["coupled"]))]
    op.set_stage(1.0, 1j * tau, cc)
    Am = (A.M + 1j * tau * (A.H_total() + sum(ck * T for ck, T in zip(cc, A.terms())))).tocsc()
    rng = np.random.default_rng(31)
    b = rng.standard_normal(S.ndof) + 1j * rng.standard_normal(S.ndof)
    s = Solver(op, pc=pc, precision="fp32", rtol=1e-12, maxit=400, outer="df", relaxed=True)
    bd = torch.tensor(b, device=cuda)
    xd = torch.zeros_like(bd)
    its, reason, rn = s.solve(bd, xd)
    x = xd.cpu().numpy()
    assert reason > 0, (its, reason, rn)
    rres = np.linalg.norm(b - Am @ x) / np.linalg.norm(b)
    assert rres < 1e-11 or _berr(Am, x, b) < 1e-13, (rres, _berr(Am, x, b))
    assert rn <= 1e-12 * np.linalg.norm(b) * 1.0001


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["cn", "pade22"])
@pytest.mark.parametrize("relaxed", [False, True])
def test_pc_guess_propagation(cuda, kind, relaxed):
    """Initial guess x0 = P^-1 b (guess order -1) with the FDM preconditioner,
    with and without relaxed Arnoldi applies: the same states as the oracle,
    one Krylov iteration per stage solve on the z-layered case."""
    import torch
    from oracle.propagate import OraclePropagator
    from tdsez_gb300.propagator import Propagator
    c = CASES["3d_heterostructure"]()
    S, ph, A = oracle_of(c)
    PS, op = product_of(c)
    field = lambda t: [0.05 * math.sin(0.3 * t)]
    rng = np.random.default_rng(19)
    psi0 = rng.standard_normal(S.ndof) + 1j * rng.standard_normal(S.ndof)
    psi0 /= math.sqrt(np.vdot(psi0, A.M @ psi0).real)
    P = OraclePropagator(A, field, kind)
    G = Propagator(op, kind, field=field, pc="fdm", precision="fp32", rtol=1e-10, outer="df", guess_order=-1,
                   relaxed=relaxed)
    dt = 0.1
    psi = psi0.copy()
    pd = torch.tensor(psi0, device=cuda)
    for step in range(4):
        psi = P.step(psi, step * dt, dt)
        G.step(pd, step * dt, dt)
    assert _rel(pd.cpu().numpy(), psi) < 1e-8
    st = G.stats()
    assert st["its"] <= st["solves"] * (2 if relaxed else 1), st
