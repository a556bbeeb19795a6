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
