"""Output files from GPU runs, read back with tests/h5lite.py: the
observables monitor's rows (dipoles, the energy split, <1/m>, populations,
autocorrelation) against the oracle's assembled matrices (1e-12), on a 2D
case with a CAP and a 1D case with a layered mass,
and the t-SURFF spectra file against the sampler's own amplitudes and the
reference's schema (src/tsurff.cpp:1018-1057)."""
import math

import numpy as np
import pytest

from oracle import bspline as ob
from tests import h5lite
from tests.cases import CASES, oracle_of, product_of


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["2d_cap_softcore_sep", "1d_layered_mass"])
def test_observables_monitor_rows(cuda, tmp_path, name):
    import scipy.sparse as sp
    import torch
    from oracle import operators as oo
    from tdsez_gb300.outputs import ObservablesMonitor
    from tdsez_gb300.propagator import Propagator
    c = CASES[name]()
    S, ph, A = oracle_of(c)
    PS, op = product_of(c)
    dim = S.dim
    rng = np.random.default_rng(3)
    psi0 = rng.standard_normal(S.ndof) + 1j * rng.standard_normal(S.ndof)
    psi0 /= math.sqrt(np.vdot(psi0, A.M @ psi0).real)
    phi = [rng.standard_normal(S.ndof) + 1j * rng.standard_normal(S.ndof) for _ in range(2)]
    coords = [cc.reshape(-1) for cc in S.quad_coords()]
    w = S.quad_weights().reshape(-1)
    Minv = (A.B.T @ sp.diags(w * oo._eval_grid(ph.minv, coords, dim)) @ A.B).tocsr()

    def field(t):
        return [0.02 * math.sin(0.5 * t), 0.0][:dim]
    q = c["charge"]
    mon = ObservablesMonitor(tmp_path / "td" / "run_observables.h5", op, field=field, charge=q,
                             bound=[torch.tensor(v, device=cuda) for v in phi], flush_rows=3)
    psi = torch.tensor(psi0, device=cuda)
    states = []
    G = Propagator(op, "cn", field=lambda t: [field(t)[0]], pc="mass", precision="fp64", rtol=1e-12)

    def monitor(step, t, ps):
        mon(step, t, ps)
        states.append((t, ps.cpu().numpy()))
    G.evolve(psi, 0.1, 0.5, monitor=monitor)
    mon.close()
    f = h5lite.File(str(tmp_path / "td" / "run_observables.h5"))
    dip, ene, pop, auto, cur = (f[s].read() for s in ("dipoles", "energies", "populations", "autocorrelation",
                                                     "currents"))
    assert dip.shape == (6, 1 + 3 * dim) and ene.shape == (6, 7) and pop.shape == (6, 3) and cur.shape == (6, 11)
    H = A.H_total()
    for r, (t, x) in enumerate(states):
        n = np.vdot(x, A.M @ x).real
        e = np.vdot(x, H @ x)
        kin = np.vdot(x, A.K @ x).real
        pot = np.vdot(x, A.V @ x).real
        inv = np.vdot(x, Minv @ x).real
        d = [np.vdot(x, A.D[a] @ x).real for a in range(dim)]
        E = field(t)
        e_int = -q * sum(E[a] * d[a] for a in range(dim))
        assert all(row[0] == t for row in (dip[r], ene[r], pop[r], auto[r], cur[r]))
        assert np.array_equal(dip[r, 1:1 + dim], E) and not np.any(dip[r, 1 + 2 * dim:])
        assert np.allclose(dip[r, 1 + dim:1 + 2 * dim], [q * v for v in d], rtol=1e-12, atol=1e-12 * n)
        scale = abs(e) + abs(kin) + n
        assert abs(ene[r, 1] - kin) <= 1e-12 * scale
        assert abs(ene[r, 2] - pot) <= 1e-12 * scale
        assert abs(ene[r, 3] - e_int) <= 1e-12 * (abs(e_int) + n)
        assert abs(ene[r, 4] - (e.real + e_int)) <= 1e-12 * scale
        assert abs(ene[r, 5] - inv) <= 1e-12 * inv
        assert abs(ene[r, 6] - n) <= 1e-12 * n
        for i, v in enumerate(phi):
            ref = abs(np.vdot(v, A.M @ x)) ** 2
            assert abs(pop[r, 1 + i] - ref) <= 1e-11 * ref
        ac = np.vdot(psi0, A.M @ x)
        assert abs(auto[r, 1] + 1j * auto[r, 2] - ac) <= 1e-12
        assert not np.any(cur[r, 1:])
    assert abs(auto[0, 1] - 1.0) < 1e-12 and abs(auto[0, 2]) < 1e-12


@pytest.mark.gpu
def test_surff_file(cuda, tmp_path):
    import torch
    from tdsez_gb300.outputs import write_surff
    from tdsez_gb300.space import Space
    from tdsez_gb300.tsurff import TSurff
    p, nq = 4, 5
    kn = [ob.uniform_knots(10, -20.0, 20.0, p), ob.symexp_knots(-18.0, 18.0, 9, 0.9, p)]
    PS = Space(kn, p, nq)
    kg = [(-1.5, 1.5, 7), (-1.0, 2.0, 5)]

    def field(t):
        return [0.05 * math.sin(0.3 * t), 0.02 * math.cos(0.2 * t), 0.0]
    ts = TSurff(PS, 9.0, kg, field, 0.1, mass=0.8, v0=0.05, charge=-1.0)
    rng = np.random.default_rng(8)
    n = int(np.prod(PS.n))
    for i in range(5):
        psi = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        ts.sample(0.3 * i, torch.tensor(psi, device=cuda))
    amp = ts.amplitudes()
    inner = ts.interior(torch.tensor(psi, device=cuda))
    path = tmp_path / "td" / "run_surff.h5"
    write_surff(path, ts, amp + inner, flux=amp, interior=True, stride=3)
    f = h5lite.File(str(path))
    assert sorted(f.keys()) == sorted(["momenta", "amplitude", "pes", "amplitude_flux", "k_x", "k_y", "pes_grid"])
    tot = amp + inner
    assert np.array_equal(f["amplitude"].read(), np.stack([tot.real, tot.imag], 1))
    assert np.array_equal(f["amplitude_flux"].read(), np.stack([amp.real, amp.imag], 1))
    assert np.array_equal(f["pes"].read(), np.abs(tot) ** 2)
    assert np.array_equal(f["pes_grid"].read(), (np.abs(tot) ** 2).reshape(7, 5))
    kx, ky = f["k_x"].read(), f["k_y"].read()
    assert np.allclose(kx, np.linspace(-1.5, 1.5, 7), rtol=0, atol=1e-15)
    assert np.allclose(ky, np.linspace(-1.0, 2.0, 5), rtol=0, atol=1e-15)
    mom = f["momenta"].read()
    assert mom.shape == (35, 2) and np.array_equal(mom[:, 0], np.repeat(kx, 5)) and np.array_equal(mom[:, 1],
                                                                                                  np.tile(ky, 7))
    a = {k: v.ravel() for k, v in f.attrs.items()}
    assert a["final_time"][0] == 0.3 * 4 and a["radius"][0] == 9.0 and a["n_samples"][0] == 5
    assert a["exterior_mass"][0] == 0.8 and a["exterior_potential"][0] == 0.05 and a["stride"][0] == 3
    assert a["interior"][0] == 1 and a["end_term"][0] == 0 and a["charge"][0] == -1.0
    assert np.array_equal(a["A_final"], ts.volkov()[:2])
    # surface Gauss points: nq per knot span clipped to [-R, R], on both faces |x_a| = R of every axis
    nodes = [sum(1 for e in range(len(k) - 1) if min(k[e + 1], 9.0) > max(k[e], -9.0)) * nq for k in kn]
    assert a["n_surface_points"][0] == 2 * nodes[1] + 2 * nodes[0]
