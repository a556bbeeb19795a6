"""Pin of the oracle's t-SURFF end term (``src/tsurff.cpp:650-976``) on the
reference's own acceptance case (END1D of the reference's test_tsurff.py):
a slow packet (k0 = 0.8) under a short pulse, stopped at T = 16 while a
third of it is still inside the box. Plain t-SURFF misses that third; with
the end term the spectrum is the analytic one,

    |b(k)|^2 = (2 w^2 / pi)^(1/2) exp(-2 w^2 (k - k0)^2),

to 2e-4 of its peak for |k| > 0.3 (below the absorber's k_min it reflects),
and the yield is 1 to 1e-3 — the reference's thresholds. Also the node
rule and the Lagrange weights on their own."""
import math

import numpy as np
import scipy.sparse.linalg as sla

from oracle import bspline as ob
from oracle import operators as oo
from oracle import propagate as opg
from oracle import tsurff as ots


def end1d_run(nel=400):
    """END1D: p = 7, [-40, 40], CAP k_min 0.5, Pade(2,2) dt 0.025, R = 10,
    181 momenta in [-1.5, 3], LaserX = 0.2 sin^2(pi t / 15) sin(1.3 t) for t < 15."""
    p, L = 7, 40.0
    S = ob.Space([ob.Axis(ob.uniform_knots(nel, -L, L, p), p, 10)])
    phys = oo.Physics(dim=1, cap_kmin=0.5, bounds=[(-L, L)], coupled=(0,))
    asm = oo.Assembled(S, phys)

    def field(t):
        return [0.2 * math.sin(math.pi * t / 15) ** 2 * math.sin(1.3 * t) if t < 15 else 0.0]
    w, k0 = 1.0, 0.8
    ax = S.axes[0]
    g = (2 * np.pi * w * w) ** -0.25 * np.exp(-ax.xq.reshape(-1) ** 2 / (4 * w * w) + 1j * k0 * ax.xq.reshape(-1))
    psi = sla.spsolve(asm.M.tocsc().astype(complex), ax.basis_matrix(0).T @ (ax.wq.reshape(-1) * g))
    psi /= math.sqrt((psi.conj() @ (asm.M @ psi)).real)
    ks = np.linspace(-1.5, 3.0, 181)
    ts = ots.OracleTSurff(S, 10.0, [ks], 1.0, 0.0, 1.0, lambda t: [field(t)[0], 0.0, 0.0], 0.025)
    amp = np.zeros(len(ks), complex)

    def observe(t, ps):
        nonlocal amp
        amp = ts.add_flux(t, ps, [ks], amp)
    psi, _ = opg.OraclePropagator(asm, field, kind="pade22").evolve(psi, 0.025, 16.0, observe=observe)
    return S, asm, ts, psi, ks, amp, (w, k0)


def test_end_nodes_rule():
    # fine spacing below the split, coarse above, both ends included
    n = ots.end_nodes(0.1, 3.0, 1.0, 0.01, 0.05)
    assert n[0] == 0.1 and n[-1] == 3.0
    d = np.diff(n)
    assert np.all(d > 0)
    assert np.allclose(d[n[:-1] < 1.0 - 1e-12], 0.9 / 90) and np.allclose(d[n[:-1] >= 1.0 - 1e-12], 2.0 / 40)
    # each segment ends exactly at its end: no near-duplicate node when the split is p_max
    for pmax in (1.8411387545741371, 1.0 + 1e-13, 0.7 + 3 * 0.1):
        n = ots.end_nodes(0.3910663495531109, pmax, pmax, 0.25, 0.25)
        assert n[-1] == pmax and np.all(np.diff(n) > 1e-6)
    # too few nodes: midpoints until there are four
    assert len(ots.end_nodes(1.0, 1.1, 1.0, 1.0, 1.0)) == 5
    assert len(ots.end_nodes(2.0, 2.0, 2.0, 0.1, 0.1)) == 1


def test_lagrange_weights_reproduce_cubics():
    node = ots.end_nodes(0.2, 2.0, 0.8, 0.03, 0.07)
    f = lambda p: 1.0 - 2 * p + 0.5 * p ** 2 - 0.3 * p ** 3
    for p in np.linspace(0.2, 2.0, 37):
        j0, w = ots.lagrange_weights(node, p)
        assert len(w) == 4 and 0 <= j0 <= len(node) - 4
        assert abs(w @ f(node[j0:j0 + 4]) - f(p)) < 1e-12


def test_end_term_restores_the_analytic_spectrum():
    S, asm, ts, psi, ks, amp, (w, k0) = end1d_run()
    end, nodes = ots.end_term(ts, psi, asm.M, asm.H_total(), [ks], cap_width=oo.cap_width(0.5))
    ex = (2 * w * w / np.pi) ** 0.5 * np.exp(-2 * w * w * (ks - k0) ** 2)
    pes = np.abs(amp + end) ** 2
    fast = np.abs(ks) > 0.3
    err = np.abs(pes - ex)[fast].max() / ex.max()
    assert err < 2e-4, err
    assert abs(np.trapezoid(pes, ks) - 1.0) < 1e-3
    assert abs(np.trapezoid(np.abs(amp) ** 2, ks) - 1.0) > 0.2     # the flux part alone is far off
    assert len(nodes) > 50
