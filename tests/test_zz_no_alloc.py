"""tdz_vec_mdot_noalloc: the allocation-free multi-dot, for callers that
cannot allocate device memory (a host application that owns every device
allocation, or a time step that must not hit cudaMalloc). Its partial sums
live in a static device array of the library; the test checks, through the
C ABI, that two calls in a row give the same results as tdz_vec_mdot (which
uses library-allocated scratch), and that more dot products than the static
array holds are refused with an error instead of overrunning it.

Collected last (file name), so that a run stopping at the first failure has
run every other test; it also passes alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest


@pytest.mark.gpu
def test_mdot_noalloc_matches_mdot(cuda):
    import torch
    from tdsez_gb300 import _lib
    lib = _lib.load()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rng = np.random.default_rng(12)
    n = 500_003
    for dt, prec in ((torch.complex128, _lib.TDZ_FP64), (torch.complex64, _lib.TDZ_FP32)):
        for k in (1, 5, 8):
            V = [torch.tensor(rng.standard_normal(n) + 1j * rng.standard_normal(n), dtype=dt, device=cuda)
                 for _ in range(k)]
            w = torch.tensor(rng.standard_normal(n) + 1j * rng.standard_normal(n), dtype=dt, device=cuda)
            ptrs = (C.c_void_p * k)(*[v.data_ptr() for v in V])
            ref = torch.zeros(k, dtype=torch.complex128, device=cuda)
            _lib.check(lib.tdz_vec_mdot(ptrs, k, C.c_void_p(w.data_ptr()), n, prec, C.c_void_p(ref.data_ptr()),
                                        stream))
            for call in range(2):
                out = torch.full((k,), complex(float("nan"), float("nan")), dtype=torch.complex128, device=cuda)
                _lib.check(lib.tdz_vec_mdot_noalloc(ptrs, k, C.c_void_p(w.data_ptr()), n, prec,
                                                    C.c_void_p(out.data_ptr()), stream))
                torch.cuda.synchronize()
                o, r = out.cpu().numpy(), ref.cpu().numpy()
                assert np.all(np.isfinite(o))
                assert np.abs(o - r).max() <= 1e-12 * np.abs(r).max(), (k, call)


@pytest.mark.gpu
def test_mdot_noalloc_rejects_too_many(cuda):
    import torch
    from tdsez_gb300 import _lib
    lib = _lib.load()
    k, n = 9, 1000
    V = [torch.zeros(n, dtype=torch.complex128, device=cuda) for _ in range(k)]
    ptrs = (C.c_void_p * k)(*[v.data_ptr() for v in V])
    out = torch.zeros(k, dtype=torch.complex128, device=cuda)
    st = lib.tdz_vec_mdot_noalloc(ptrs, k, C.c_void_p(V[0].data_ptr()), n, _lib.TDZ_FP64,
                                  C.c_void_p(out.data_ptr()), C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 1 and b"static scratch holds" in lib.tdz_last_error()
