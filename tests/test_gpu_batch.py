"""Batched propagations (intensity / carrier-envelope-phase scan): runs with
different fields, and different grids, stepped together by
tdz_prop_step_batch on their own streams give the states of the same runs
stepped one by one."""
import math

import numpy as np
import pytest

from tests.cases import CASES, product_of


def _runs(cuda, specs):
    import torch
    from tdsez_gb300.propagator import Propagator
    out = []
    for name, E0, phi in specs:
        c = CASES[name]()
        S, op = product_of(c)
        ncpl = len(c["coupled"])
        field = (lambda E0, phi: (lambda t: [E0 * math.sin(0.5 * t + phi + k) for k in range(ncpl)]))(E0, phi)
        G = Propagator(op, "cn", field=field, pc="fdm" if S.dim == 3 else "mg", precision="fp32", rtol=1e-11,
                       outer="df")
        rng = np.random.default_rng(len(out) + 1)
        psi = torch.tensor(rng.standard_normal(S.ndof) + 1j * rng.standard_normal(S.ndof), device=cuda)
        out.append((G, psi))
    return out


@pytest.mark.gpu
def test_batch_equals_serial(cuda):
    import torch
    from tdsez_gb300.propagator import BatchPropagator
    specs = [("2d_softcore", 10 ** (-2 + k / 4), 2 * math.pi * k / 6) for k in range(6)]
    specs += [("3d_heterostructure", 0.01, 0.3), ("2d_cap_softcore_sep", 0.05, 1.0)]
    serial = _runs(cuda, specs)
    batch = _runs(cuda, specs)
    B = BatchPropagator([G for G, _ in batch], threads=4)
    psis = [p for _, p in batch]
    dt = 0.05
    for step in range(3):
        for G, p in serial:
            G.step(p, step * dt, dt)
        B.step(psis, step * dt, dt)
    torch.cuda.synchronize()
    # the soft-core quadrature term adds element contributions with atomics, whose
    # order differs between two executions: agreement to rounding, not bit for bit
    for (Gs, ps), pb in zip(serial, psis):
        a, b = ps.cpu().numpy(), pb.cpu().numpy()
        assert np.linalg.norm(a - b) <= 1e-10 * np.linalg.norm(a)
    for G, _ in batch:
        assert G.stats()["solves"] == 3


@pytest.mark.gpu
def test_batch_fdm_ragged_outer_axes(cuda):
    """FDM-preconditioned 2D runs whose outer axes have different lengths
    (degree 5, 240 to 300 elements: line solves with different, large
    shared-memory footprints), stepped together from the thread pool: the
    same states as stepping them one by one."""
    import torch
    from oracle import bspline as ob
    from tdsez_gb300.operators import Operator, Physics
    from tdsez_gb300.propagator import BatchPropagator, Propagator
    from tdsez_gb300.space import Space

    def make():
        out = []
        for k, nel in enumerate((240, 260, 280, 300)):
            p = 5
            S = Space([ob.uniform_knots(16, -12.0, 12.0, p), ob.uniform_knots(nel, -60.0, 60.0, p)], p, 6)
            op = Operator(S, Physics(charge=-1.0, mass=1.0, coupled=(0,), softcore=[(1.0, 0.0, 0.0, 0.0, 1.0)]))
            E0 = 0.02 * (k + 1)
            G = Propagator(op, "cn", field=(lambda E0: (lambda t: [E0 * math.sin(0.3 * t)]))(E0), pc="fdm",
                           precision="fp32", rtol=1e-11, outer="df")
            psi = op.separable_state([lambda x: np.exp(-x * x / 4.0), lambda y: np.exp(-y * y / 8.0)])
            out.append((G, psi))
        return out
    serial, batch = make(), make()
    B = BatchPropagator([G for G, _ in batch], threads=4)
    psis = [p for _, p in batch]
    for step in range(3):
        for G, p in serial:
            G.step(p, step * 0.05, 0.05)
        B.step(psis, step * 0.05, 0.05)
    torch.cuda.synchronize()
    for (Gs, ps), pb in zip(serial, psis):
        a, b = ps.cpu().numpy(), pb.cpu().numpy()
        assert np.linalg.norm(a - b) <= 1e-10 * np.linalg.norm(a)
