"""GPU t-SURFF sampler against the oracle's FluxList/AddFlux restatement:
identical amplitudes (FP64, 1e-11 relative) for a field-driven sequence of
states in 1D, 2D and 3D, and the free-packet spectrum on the reference deck."""
import math

import numpy as np
import pytest

from oracle import bspline as ob
from oracle import tsurff as ots


def _field(t):
    return [0.05 * math.sin(0.3 * t), 0.02 * math.cos(0.2 * t), -0.03 * math.sin(0.1 * t + 1.0)]


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [1, 2, 3])
def test_tsurff_parity(cuda, dim):
    import torch
    from tdsez_gb300.space import Space
    from tdsez_gb300.tsurff import TSurff
    p, nq = 4, 5
    kn = [ob.uniform_knots(10, -20.0, 20.0, p), ob.symexp_knots(-18.0, 18.0, 9, 0.9, p),
          ob.uniform_knots(8, -16.0, 16.0, p)][:dim]
    S = ob.Space([ob.Axis(k, p, nq) for k in kn])
    R = 9.0
    kg = [(-1.5, 1.5, 7), (-1.0, 2.0, 5), (-0.5, 0.5, 3)][:dim]
    dt, mass, V0, charge = 0.1, 0.8, 0.05, -1.0
    ora = ots.OracleTSurff(S, R, [np.linspace(*k) for k in kg], mass, V0, -charge, _field, dt)
    PS = Space(kn, p, nq)
    gpu = TSurff(PS, R, kg, _field, dt, mass=mass, v0=V0, charge=charge)
    rng = np.random.default_rng(4)
    amp = np.zeros(int(np.prod([k[2] for k in kg])), dtype=complex)
    for i in range(6):
        t = 0.3 * i
        psi = rng.standard_normal(S.ndof) + 1j * rng.standard_normal(S.ndof)
        amp = ora.add_flux(t, psi, [np.linspace(*k) for k in kg], amp)
        gpu.sample(t, torch.tensor(psi, device=cuda))
    a = gpu.amplitudes()
    assert np.abs(a - amp).max() <= 1e-11 * np.abs(amp).max()
    v = gpu.volkov()
    assert np.allclose(v[:3], ora.A) and np.allclose(v[3:6], ora.B) and abs(v[6] - ora.C) < 1e-12
    # interior projection of the last state onto the Volkov states at the last sample
    ki = gpu.interior(torch.tensor(psi, device=cuda))
    kr = ora.interior(psi, [np.linspace(*k) for k in kg])
    assert np.abs(ki - kr).max() <= 1e-11 * np.abs(kr).max(), np.abs(ki - kr).max() / np.abs(kr).max()


@pytest.mark.gpu
def test_tsurff_free_packet_gpu(cuda):
    """FREE1D deck of test_tsurff.py (p = 7, 400 elements, Pade(2,2), dt 0.025,
    T = 20, R = 10): GPU propagation, GPU flux and the GPU interior
    projection of psi(T), against the analytic spectrum at 1e-4."""
    import torch
    from tdsez_gb300.operators import Operator, Physics
    from tdsez_gb300.propagator import Propagator
    from tdsez_gb300.space import Space
    from tdsez_gb300.tsurff import TSurff
    p, L = 7, 40.0
    kn = ob.uniform_knots(400, -L, L, p)
    PS = Space([kn], p, 10)
    op = Operator(PS, Physics(cap_kmin=0.5, bounds=[(-L, L)], coupled=(0,)))
    w, k0 = 1.0, 2.0
    psi = op.separable_state([lambda x: (2 * np.pi * w * w) ** -0.25 * np.exp(-x * x / (4 * w * w) + 1j * k0 * x)])
    G = Propagator(op, "pade22", field=lambda t: [0.0], pc="mass", precision="fp64")
    ts = TSurff(PS, 10.0, [(-1.0, 5.0, 61)], lambda t: [0.0, 0.0, 0.0], 0.025)
    G.evolve(psi, 0.025, 20.0, monitor=lambda step, t, ps: ts.sample(t, ps))
    amp = ts.amplitudes()
    tot = amp + ts.interior(psi)
    ks = np.linspace(-1, 5, 61)
    ex = (2 * w * w / np.pi) ** 0.5 * np.exp(-2 * w * w * (ks - k0) ** 2)
    assert np.abs(np.abs(tot) ** 2 - ex).max() / ex.max() < 1e-4
