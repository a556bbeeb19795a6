"""Learned coarse correction inside the multigrid V-cycle, through the C ABI.

The network is trained on the GPU on pairs the solver generates. The test
checks three things:
* the network lowers the error of a cheap coarsest-level solve (a degree-2
  Chebyshev polynomial) on fresh right-hand sides, which is what it gains at
  its own task;
* the corrected preconditioner gives converged FP64 solves, with no more
  iterations than the same cheap V-cycle without the network;
* both reach the same solution.

With the default degree-12 coarse polynomial, the coarsest solve of this
hierarchy is already exact to FP32 rounding (relative error ~2e-9). There
the network has nothing left to correct, and its residual input is rounding
noise."""
import numpy as np
import pytest


@pytest.mark.gpu
def test_learned_coarse_correction(cuda):
    import torch
    from tdsez_gb300.operators import Operator
    from tdsez_gb300.propagator import Solver
    from tdsez_gb300.space import Space
    from tdsez_gb300.workloads import heterostructure
    w = heterostructure(nel=(16, 16, 32))           # same layering, 19 x 19 x 37 coefficients
    S = Space(w.knots, w.p, w.nq)
    op = Operator(S, w.phys)
    op.set_stage(1.0, 0.5j * w.dt, [w.phys.sign * 0.005])
    rng = np.random.default_rng(12)
    b = torch.tensor(rng.standard_normal(S.ndof) + 1j * rng.standard_normal(S.ndof), device=cuda)

    plain = Solver(op, pc="mg", precision="fp32", rtol=1e-10, maxit=200, mg_coarse_its=2)
    x0 = torch.zeros_like(b)
    its_plain, reason, _ = plain.solve(b, x0)
    assert reason > 0

    s = Solver(op, pc="mg", precision="fp32", rtol=1e-10, maxit=200, mg_coarse_its=2, mg_learned=True)
    loss = s.train_coarse(pairs=512, epochs=60, lr=1e-3, seed=3)
    assert np.isfinite(loss) and loss < 1.0
    e_plain, e_learned = s.coarse_gain(trials=16, seed=99)
    print(f"coarse solve error: Chebyshev {e_plain:.3e}, with the network {e_learned:.3e}; training loss {loss:.3e}")
    assert e_learned < e_plain, (e_plain, e_learned)

    x1 = torch.zeros_like(b)
    its_learned, reason, _ = s.solve(b, x1)
    print(f"FGMRES iterations to 1e-10: plain V-cycle {its_plain}, learned {its_learned}")
    assert reason > 0
    assert its_learned <= its_plain
    # both reach the same FP64 solution
    assert (torch.linalg.norm(x1 - x0) / torch.linalg.norm(x0)).item() < 1e-8


@pytest.mark.gpu
def test_learned_correction_trained_on_the_propagation(cuda):
    """The learned arm of the benchmark on a reduced heterostructure: the
    network is trained on the coarsest right-hand sides that the V-cycles of
    the propagation's own first CN steps produce (default coarse polynomial,
    a two-level hierarchy whose coarse level the polynomial does not solve
    exactly). Over the next steps the learned V-cycle needs no more FGMRES
    iterations than the same V-cycle without the network, and the three
    propagations (learned, plain, FDM-preconditioned) reach the same states."""
    import torch
    from tdsez_gb300.operators import Operator
    from tdsez_gb300.propagator import Propagator
    from tdsez_gb300.space import Space
    from tdsez_gb300.workloads import heterostructure
    w = heterostructure(nel=(32, 32, 64))
    S = Space(w.knots, w.p, w.nq)
    op = Operator(S, w.phys)
    kw = dict(pc="mg", precision="fp32", outer="df", rtol=1e-10, mg_levels=2)
    props = {"learned": Propagator(op, "cn", field=w.field, mg_learned=True, **kw),
             "plain": Propagator(op, "cn", field=w.field, **kw),
             "fdm": Propagator(op, "cn", field=w.field, pc="fdm", precision="fp32", outer="df", rtol=1e-10)}
    psi0 = op.separable_state(w.packet)
    t, dt = 0.0, w.dt
    x = {k: psi0.clone() for k in props}
    props["learned"].record_coarse(64)
    for _ in range(6):   # the same first steps for every arm (and the same guess history)
        for k, P in props.items():
            P.step(x[k], t, dt)
        t += dt
    props["learned"].record_coarse(0)
    loss, pairs = props["learned"].train_coarse(epochs=40, lr=1e-3)
    assert pairs >= 8 and np.isfinite(loss) and loss < 1.0, (loss, pairs)
    states, its = {}, {}
    for name, P in props.items():
        s0 = P.stats()
        for k in range(4):
            P.step(x[name], t + k * dt, dt)
        torch.cuda.synchronize()
        s1 = P.stats()
        its[name] = (s1["its"] - s0["its"]) / 4
        states[name] = x[name]
    print(f"training pairs {pairs}, loss {loss:.3e}; FGMRES its/step: learned {its['learned']}, "
          f"plain {its['plain']}, FDM {its['fdm']}")
    # each stage solve stops at a relative residual of 1e-10; with the stage
    # operator's conditioning (its spectrum spans |1 + i dt/2 lambda| up to a
    # few hundred) the states of independent solvers differ by up to ~1e-8 per
    # step, accumulated over ten steps
    for name in ("learned", "plain"):
        rel = (torch.linalg.norm(states[name] - states["fdm"]) / torch.linalg.norm(states["fdm"])).item()
        assert rel < 1e-6, (name, rel)
    assert its["learned"] <= its["plain"], its
