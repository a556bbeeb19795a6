"""GPU parity of the fused matrix-free apply against the oracle's assembled
FP64 operators: M, H (+CAP), D_a and the stage operator, through the C ABI.
Bar: 1e-12 relative (max norm) in FP64 and in double-float (FP64 vectors,
FP32-pair arithmetic), 1e-6 in FP32 (FP32 vectors, and FP32 arithmetic on
FP64 vectors for the 3D operators without soft-core centres)."""
import numpy as np
import pytest

from tests.cases import CASES, oracle_of, product_of

TOL = {"fp64": 1e-12, "df": 1e-12, "fp32": 1e-6, "f32": 1e-6}


def _rel(y, ref):
    return np.abs(y - ref).max() / max(np.abs(ref).max(), 1e-300)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_apply_parity(cuda, name):
    import torch
    from tdsez_gb300 import _lib
    c = CASES[name]()
    S, ph, A = oracle_of(c)
    PS, op = product_of(c)
    assert PS.ndof == S.ndof
    rng = np.random.default_rng(11)
    x = rng.standard_normal(S.ndof) + 1j * rng.standard_normal(S.ndof)
    alpha, g = 1.0 + 0.1j, 0.013 + 0.04j
    cc = [0.021 * (k + 1) - 0.004j for k in range(len(c["coupled"]))]
    op.set_stage(alpha, g, cc)
    refs = {_lib.TDZ_MASS: A.M @ x, _lib.TDZ_HAMILTONIAN: A.H_total() @ x,
            _lib.TDZ_STAGE: alpha * (A.M @ x) + g * (A.H_total() @ x + sum(ck * (T @ x) for ck, T in zip(cc, A.terms())))}
    for a in range(S.dim):
        refs[_lib.TDZ_DIPOLE_X + a] = A.D[a] @ x
    precs = [("fp64", torch.complex128), ("df", torch.complex128), ("fp32", torch.complex64)]
    if S.dim == 3 and not c.get("soft"):   # FP32 arithmetic on FP64 vectors (TDZ_FP64_F32)
        precs.append(("f32", torch.complex128))
    for prec, dt in precs:
        xd = torch.tensor(x, dtype=dt, device=cuda)
        for which, ref in refs.items():
            yd = torch.full_like(xd, float("nan"))
            op.apply(which, xd, yd, df=prec == "df", f32=prec == "f32")
            torch.cuda.synchronize()
            err = _rel(yd.cpu().numpy().astype(np.complex128), ref)
            assert err < TOL[prec], (name, prec, which, err)
    assert op.launches >= 3 * len(refs)


@pytest.mark.gpu
def test_stage_change_needs_no_rebuild(cuda):
    """set_stage only changes scalars: two stages applied back to back both
    match the oracle (the CN / Pade stage update of propagator.cpp:374-551)."""
    import torch
    from tdsez_gb300 import _lib
    c = CASES["3d_heterostructure"]()
    S, ph, A = oracle_of(c)
    PS, op = product_of(c)
    x = np.random.default_rng(5).standard_normal(S.ndof) * (1 - 0.3j)
    xd = torch.tensor(x, dtype=torch.complex128, device=cuda)
    for alpha, g, c0 in [(1.0, 0.025j, 0.01), (1.0, (-np.sqrt(3) + 3j) / 12 * 0.02, -0.03)]:
        op.set_stage(alpha, g, [c0])
        yd = torch.empty_like(xd)
        op.apply(_lib.TDZ_STAGE, xd, yd)
        ref = alpha * (A.M @ x) + g * (A.H_total() @ x + c0 * (A.D[2] @ x))
        assert _rel(yd.cpu().numpy(), ref) < 1e-12


@pytest.mark.gpu
def test_vec_dot(cuda):
    """tdz_vec_dot (FP64 accumulation, deterministic) against numpy, FP32 and FP64."""
    import ctypes as C
    import torch
    from tdsez_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(2)
    n = 1_000_003
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    y = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    ref = np.vdot(x, y)
    out = torch.zeros(1, dtype=torch.complex128, device=cuda)
    for dt, prec, tol in ((torch.complex128, _lib.TDZ_FP64, 1e-13), (torch.complex64, _lib.TDZ_FP32, 1e-6)):
        xd, yd = torch.tensor(x, dtype=dt, device=cuda), torch.tensor(y, dtype=dt, device=cuda)
        vals = []
        for _ in range(2):
            _lib.check(lib.tdz_vec_dot(C.c_void_p(xd.data_ptr()), C.c_void_p(yd.data_ptr()), n, prec,
                                       C.c_void_p(out.data_ptr()), C.c_void_p(torch.cuda.current_stream().cuda_stream)))
            vals.append(out.item())
        assert vals[0] == vals[1]                      # bit-reproducible
        assert abs(vals[0] - ref) <= tol * np.sqrt(n) * 2


@pytest.mark.gpu
def test_vec_mdot(cuda):
    """tdz_vec_mdot (k = 20 > one 16-vector pass) against numpy."""
    import ctypes as C
    import torch
    from tdsez_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(5)
    n, k = 300_001, 20
    V = [torch.tensor(rng.standard_normal(n) + 1j * rng.standard_normal(n), device=cuda) for _ in range(k)]
    w = torch.tensor(rng.standard_normal(n) + 1j * rng.standard_normal(n), device=cuda)
    out = torch.zeros(k, dtype=torch.complex128, device=cuda)
    ptrs = (C.c_void_p * k)(*[v.data_ptr() for v in V])
    _lib.check(lib.tdz_vec_mdot(ptrs, k, C.c_void_p(w.data_ptr()), n, _lib.TDZ_FP64, C.c_void_p(out.data_ptr()),
                                C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    ref = np.array([np.vdot(v.cpu().numpy(), w.cpu().numpy()) for v in V])
    assert np.abs(out.cpu().numpy() - ref).max() <= 1e-12 * np.abs(ref).max() + 1e-9


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["3d_heterostructure", "2d_softcore", "3d_const_mass_cap"])
def test_observables(cuda, name):
    """Norm, energy and dipoles of a state in one call (the monitor
    expectation values), against the oracle's assembled matrices: 1e-12."""
    import torch
    c = CASES[name]()
    S, ph, A = oracle_of(c)
    PS, op = product_of(c)
    rng = np.random.default_rng(21)
    psi = rng.standard_normal(S.ndof) + 1j * rng.standard_normal(S.ndof)
    norm, energy, dip = op.observables(torch.tensor(psi, device=cuda))
    ref_n = np.vdot(psi, A.M @ psi)
    ref_e = np.vdot(psi, A.H_total() @ psi)
    assert abs(norm - ref_n.real) <= 1e-12 * abs(ref_n)
    assert abs(energy - ref_e) <= 1e-12 * abs(ref_e)
    for a in range(S.dim):
        ref_d = np.vdot(psi, A.D[a] @ psi)
        assert abs(dip[a] - ref_d) <= 1e-12 * max(abs(ref_d), 1e-3 * abs(ref_n)), (a, dip[a], ref_d)
