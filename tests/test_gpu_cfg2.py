"""The 2D soft-core Pade(2,2) configuration (V = -1/sqrt(x^2 + y^2 + 1),
CAP of width 20 a.u. on every wall, field along x) at a reduced 64^2
elements of degree 4: 50 GPU steps from the pulse's peak against the
oracle's Pade(2,2) with direct sparse solves of the assembled FP64
matrices, FP32 multigrid or the FP32 FDM inverse of the separable part
(absorbing layers through complex axis pencils; the soft-core term and the
field along x left to FGMRES) inside FP64 FGMRES at rtol 1e-12: the states
agree to 1e-9 and the norm decays only through the CAP (same as the
oracle)."""
import numpy as np
import pytest

from tests.cases import oracle_of, product_of


@pytest.mark.gpu
@pytest.mark.parametrize("pc", ["mg", "fdm"])
def test_softcore2d_pade_50_steps(cuda, pc):
    import torch
    from oracle.propagate import OraclePropagator
    from tdsez_gb300.propagator import Propagator
    from tdsez_gb300.workloads import softcore2d
    w = softcore2d(nel=64)
    c = dict(knots=w.knots, p=w.p, nq=w.nq, charge=w.phys.charge, mass=1.0, coupled=(0,),
             cap_kmin=w.phys.cap_kmin, bounds=list(w.phys.bounds), soft=list(w.phys.softcore))
    S, ph, A = oracle_of(c)
    PS, op = product_of(c)
    psi = op.separable_state([lambda x: np.exp(-x * x / 8.0)] * 2)
    p0 = psi.cpu().numpy()
    t0, dt, steps = 0.5 * w.meta["T"], 0.5, 50    # a larger step than the configuration's: more work per solve
    P = OraclePropagator(A, w.field, "pade22")
    G = Propagator(op, "pade22", field=w.field, pc=pc, precision="fp32", outer="df", rtol=1e-12)
    ref = p0.copy()
    for k in range(steps):
        ref = P.step(ref, t0 + k * dt, dt)
        G.step(psi, t0 + k * dt, dt)
    torch.cuda.synchronize()
    got = psi.cpu().numpy()
    err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    st = G.stats()
    print(pc, "relative state error", err, "its per solve", st["its"] / st["solves"])
    assert err < 1e-9, err
    n0, n1 = np.vdot(p0, A.M @ p0).real, np.vdot(got, A.M @ got).real
    assert n1 < n0 and abs(n1 - np.vdot(ref, A.M @ ref).real) < 1e-9
