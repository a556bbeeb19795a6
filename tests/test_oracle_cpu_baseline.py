"""The oracle's C restatement of the reference's CPU solver (GMRES(30) with
block-Jacobi ILU(0), OpenMP; the CPU baseline of bench.py) against direct
sparse Crank-Nicolson solves of the same assembled matrices."""
import numpy as np
import pytest
import scipy.sparse.linalg as sla


@pytest.mark.parametrize("threads,blocks", [(1, 1), (3, 1), (3, 3)])
def test_c_port_matches_direct_cn(threads, blocks):
    from oracle.cpu_baseline import _problem, build_c, cn_steps_threads
    from tdsez_gb300.workloads import heterostructure
    try:
        build_c()
    except Exception as e:   # no gcc with OpenMP on this host
        pytest.skip(f"C port not buildable: {e}")
    w = heterostructure(nel=(5, 5, 10), dt=0.5)
    S, axes, M, H, T, psi = _problem(w)
    s = -w.phys.charge
    ref = psi.copy()
    for k in range(3):
        c = [s * e for e in w.field((k + 0.5) * w.dt)]
        A = (M + 0.5j * w.dt * (H + sum(ci * Ti for ci, Ti in zip(c, T)))).tocsc()
        X = sla.spsolve(A, M @ ref)
        ref = 2 * X - ref
    r = cn_steps_threads(w, seconds=0.0, min_steps=3, steps_max=3, threads=threads, blocks=blocks,
                         return_state=True)
    assert r["steps"] == 3 and r["blocks"] == blocks
    # rtol 1e-10 on the residual; the state error stays at the solve's accuracy
    assert np.linalg.norm(r["psi"] - ref) / np.linalg.norm(ref) < 1e-6
