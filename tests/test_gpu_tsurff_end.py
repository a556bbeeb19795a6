"""GPU t-SURFF end term (``src/tsurff.cpp:650-976``) and the banded LU
preconditioner it uses in 1D, through the C ABI:

* the banded LU inverts 1D stage operators (absorbing layer, walls, layered
  mass) exactly: FGMRES converges in one iteration to the direct solution;
* end-term amplitudes equal the oracle's (one direct sparse solve per energy
  node) on the same states, in 1D, 2D and 3D;
* the reference's END1D acceptance case run entirely on the GPU: the end
  term restores the analytic spectrum of a packet stopped inside the box;
* the guards: the field must be over at T, the operator must carry the
  absorbing layer."""
import math

import numpy as np
import pytest
import scipy.sparse.linalg as sla

from oracle import operators as oo
from oracle import tsurff as ots
from tests.cases import CASES, oracle_of, product_of


def _pulse(t):
    """Field on axis 0 for t < 1.2, off after (its samples are the run)."""
    return 0.05 * math.sin(math.pi * t / 1.2) ** 2 * math.sin(2.0 * t) if t < 1.2 else 0.0


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["1d_cap_free", "1d_dirichlet_ho", "1d_layered_mass"])
def test_band_lu_is_exact(cuda, name):
    import torch
    from tdsez_gb300.propagator import Solver
    c = CASES[name]()
    S, ph, A = oracle_of(c)
    PS, op = product_of(c)
    tau, cc = 0.3, [0.04]
    op.set_stage(1.0, 1j * tau, cc)
    Am = (A.M + 1j * tau * (A.H_total() + sum(ck * T for ck, T in zip(cc, A.terms())))).tocsc()
    rng = np.random.default_rng(5)
    b = rng.standard_normal(S.ndof) + 1j * rng.standard_normal(S.ndof)
    xref = sla.spsolve(Am, b)
    s = Solver(op, pc="band", precision="fp64", rtol=1e-12, maxit=20)
    bd = torch.tensor(b, device=cuda)
    xd = torch.zeros_like(bd)
    its, reason, _ = s.solve(bd, xd)
    assert reason > 0 and its <= 2, (its, reason)
    x = xd.cpu().numpy()
    assert np.linalg.norm(x - xref) / np.linalg.norm(xref) < 1e-10
    # an indefinite Helmholtz-type stage E M - H (the end term's) as well
    E = 0.7
    op.set_stage(E, -1.0, [0.0])
    Ah = (E * A.M - A.H_total()).tocsc()
    xref = sla.spsolve(Ah, b)
    s2 = Solver(op, pc="band", precision="fp64", rtol=1e-12, maxit=20)
    xd.zero_()
    its, reason, _ = s2.solve(bd, xd)
    assert reason > 0 and its <= 3, (its, reason)
    assert np.linalg.norm(xd.cpu().numpy() - xref) / np.linalg.norm(xref) < 1e-9


def _packet(S, c, k0, width=1.0):
    """M-projection of a Gaussian packet (product over axes) on the oracle space."""
    _, _, A = oracle_of(c)
    vecs = []
    for d, ax in enumerate(S.axes):
        x = ax.xq.reshape(-1)
        g = np.exp(-x * x / (4 * width * width) + 1j * k0[d] * x)
        vecs.append(ax.basis_matrix(0).T @ (ax.wq.reshape(-1) * g))
    b = vecs[-1]
    for v in reversed(vecs[:-1]):
        b = np.outer(b, v).reshape(-1)
    psi = sla.spsolve(A.M.tocsc().astype(complex), b)
    return psi / math.sqrt((psi.conj() @ (A.M @ psi)).real), A


@pytest.mark.gpu
@pytest.mark.parametrize("name,R,kg,dp", [
    ("1d_cap_free", 5.0, [(-1.0, 2.5, 15)], 0.0),
    ("2d_cap_free", 6.0, [(-0.5, 2.0, 6), (-1.0, 1.5, 5)], 0.12),
    ("3d_cap_free", 4.0, [(-0.5, 1.0, 3), (-0.5, 1.0, 3), (-0.2, 1.2, 4)], 0.25),
])
def test_end_term_parity(cuda, name, R, kg, dp):
    """Same states sampled by both, then the end term: GPU (FGMRES per node,
    relative residual 1e-11) against the oracle (direct sparse solve per node)."""
    import torch
    from tdsez_gb300.tsurff import TSurff
    c = CASES[name]()
    S, ph, _ = oracle_of(c)
    PS, op = product_of(c)
    dim = S.dim
    psi, A = _packet(S, c, [1.2, 0.6, 0.9][:dim])
    field3 = lambda t: [_pulse(t), 0.0, 0.0]
    dt = 0.1
    ks = [np.linspace(*k) for k in kg]
    ora = ots.OracleTSurff(S, R, ks, 1.0, 0.0, 1.0, field3, dt)
    gpu = TSurff(PS, R, kg, lambda t: [_pulse(t)] + [0.0] * (dim - 1), dt)
    amp = np.zeros(int(np.prod([k[2] for k in kg])), complex)
    rng = np.random.default_rng(7)
    for i in range(8):
        t = 0.2 * i            # the last sample (t = 1.4) is after the pulse
        st = psi * np.exp(-0.3j * i) + 0.05 * (rng.standard_normal(S.ndof) + 1j * rng.standard_normal(S.ndof))
        amp = ora.add_flux(t, st, ks, amp)
        gpu.sample(t, torch.tensor(st, device=cuda))
    width = oo.cap_width(c["cap_kmin"])
    ref, nodes = ots.end_term(ora, st, A.M, A.H_total(), ks, cap_width=width, dp=dp)
    out, stats = gpu.end_term(op, torch.tensor(st, device=cuda), cap_width=width, dp=dp, rtol=1e-11)
    print(f"{name}: {stats}")
    assert stats["nodes"] == len(nodes)
    # exact preconditioners: the banded LU (1D) and the FP64 FDM inverse
    # with complex symmetric axis pencils (2D), so one or two iterations per node
    assert stats["eta"] == 0.0 and stats["max_its"] <= 3, stats
    err = np.abs(out - ref).max() / np.abs(ref).max()
    assert err < 1e-8, err
    # the flux part is unchanged by the end term
    assert np.abs(gpu.amplitudes() - amp).max() <= 1e-11 * np.abs(amp).max()


@pytest.mark.gpu
def test_end_term_end1d_on_the_gpu(cuda):
    """END1D of the reference's test_tsurff.py (p = 7, [-40, 40], CAP k_min
    0.5, Pade(2,2) dt 0.025 with the banded LU, R = 10, 181 momenta in
    [-1.5, 3], 0.2 sin^2(pi t/15) sin(1.3 t) for t < 15, T = 16): flux and
    end term on the GPU give the analytic spectrum to 2e-4 for |k| > 0.3 and
    the yield to 1e-3, while the flux alone misses a third of the packet."""
    import torch
    from oracle import bspline as ob
    from tdsez_gb300.operators import Operator, Physics, cap_width
    from tdsez_gb300.propagator import Propagator
    from tdsez_gb300.space import Space
    from tdsez_gb300.tsurff import TSurff
    p, L = 7, 40.0
    PS = Space([ob.uniform_knots(400, -L, L, p)], p, 10)
    op = Operator(PS, Physics(cap_kmin=0.5, bounds=[(-L, L)], coupled=(0,)))
    fld = lambda t: [0.2 * math.sin(math.pi * t / 15) ** 2 * math.sin(1.3 * t) if t < 15 else 0.0]
    w, k0 = 1.0, 0.8
    psi = op.separable_state([lambda x: (2 * np.pi * w * w) ** -0.25 * np.exp(-x * x / (4 * w * w) + 1j * k0 * x)])
    G = Propagator(op, "pade22", field=fld, pc="band", precision="fp64")
    ts = TSurff(PS, 10.0, [(-1.5, 3.0, 181)], fld, 0.025)
    G.evolve(psi, 0.025, 16.0, monitor=lambda step, t, ps: ts.sample(t, ps))
    amp = ts.amplitudes()
    end, stats = ts.end_term(op, psi, cap_width=cap_width(0.5))
    print(stats)
    ks = np.linspace(-1.5, 3.0, 181)
    ex = (2 * w * w / np.pi) ** 0.5 * np.exp(-2 * w * w * (ks - k0) ** 2)
    pes = np.abs(amp + end) ** 2
    fast = np.abs(ks) > 0.3
    err = np.abs(pes - ex)[fast].max() / ex.max()
    assert err < 2e-4, err
    assert abs(np.trapezoid(pes, ks) - 1.0) < 1e-3
    assert abs(np.trapezoid(np.abs(amp) ** 2, ks) - 1.0) > 0.2
    assert stats["nodes"] > 50


@pytest.mark.gpu
def test_end_term_end2d_on_the_gpu(cuda):
    """2D deck of the reference's end-term test (p = 4, 60 x 60 elements on
    [-20, 20]^2, CAP k_min 1, CN dt 0.02 to T = 2, packet k0 = (2, 1), R = 6,
    31 x 31 momenta on [-1, 5] x [-2, 4], no field): the packet is still inside
    the box at T; flux plus end term give the analytic spectrum to 1e-2."""
    import torch
    from oracle import bspline as ob
    from tdsez_gb300.operators import Operator, Physics, cap_width
    from tdsez_gb300.propagator import Propagator
    from tdsez_gb300.space import Space
    from tdsez_gb300.tsurff import TSurff
    p, L = 4, 20.0
    kn = ob.uniform_knots(60, -L, L, p)
    PS = Space([kn, kn], p, 6)
    op = Operator(PS, Physics(cap_kmin=1.0, bounds=[(-L, L), (-L, L)], coupled=(0,)))
    w, k0 = 1.0, (2.0, 1.0)
    psi = op.separable_state([lambda x, k=k: (2 * np.pi * w * w) ** -0.25 * np.exp(-x * x / (4 * w * w) + 1j * k * x)
                              for k in k0])
    G = Propagator(op, "cn", field=lambda t: [0.0], pc="fdm", precision="fp32", rtol=1e-12, guess_order=-1)
    ts = TSurff(PS, 6.0, [(-1.0, 5.0, 31), (-2.0, 4.0, 31)], lambda t: [0.0, 0.0], 0.02)
    G.evolve(psi, 0.02, 2.0, monitor=lambda step, t, ps: ts.sample(t, ps))
    end, stats = ts.end_term(op, psi, cap_width=cap_width(1.0))
    print(stats)
    b = (ts.amplitudes() + end).reshape(31, 31)
    kx, ky = np.linspace(-1, 5, 31), np.linspace(-2, 4, 31)
    ex = np.outer((2 * w * w / np.pi) ** 0.5 * np.exp(-2 * w * w * (kx - k0[0]) ** 2),
                  (2 * w * w / np.pi) ** 0.5 * np.exp(-2 * w * w * (ky - k0[1]) ** 2))
    err = np.abs(np.abs(b) ** 2 - ex).max() / ex.max()
    assert err < 1e-2, err
    assert stats["max_its"] <= 3 and stats["damped"] == 0, stats


@pytest.mark.gpu
def test_end_term_guards(cuda):
    import torch
    from tdsez_gb300 import _lib
    from tdsez_gb300.tsurff import TSurff
    c = CASES["1d_cap_free"]()
    PS, op = product_of(c)
    psi = torch.zeros(PS.ndof, dtype=torch.complex128, device=cuda)
    psi[PS.ndof // 2] = 1.0
    on = TSurff(PS, 5.0, [(-1.0, 1.0, 5)], lambda t: [0.05 * math.sin(t)], 0.1)
    on.sample(0.0, psi)
    on.sample(1.0, psi)
    with pytest.raises(_lib.TDZError, match="field is not over"):
        on.end_term(op, psi, cap_width=13.11)
    c2 = dict(c)
    c2.pop("cap_kmin")
    _, op_nocap = product_of(c2)
    off = TSurff(PS, 5.0, [(-1.0, 1.0, 5)], lambda t: [0.0], 0.1)
    off.sample(0.0, psi)
    with pytest.raises(_lib.TDZError, match="absorbing layer"):
        off.end_term(op_nocap, psi, cap_width=13.11)
