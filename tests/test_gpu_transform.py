"""Tensor-core plane transform (tcgen05, TF32 with a hi/lo split of both operands)
against numpy FP64, through the C ABI (the warp-specialised kernel; the
single-accumulator kernel with TDZ_TRANSFORM=split). Bar: FP32 class, i.e. a max-norm
relative error at most 4x that of the same contraction evaluated in FP32 by
numpy (about 1e-6 at K = 163), and never above 1e-5."""
import ctypes as C

import numpy as np
import pytest


def _run(K, N, planes, R, ldi, ldo, seed):
    import torch
    from tdsez_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(seed)
    B = rng.standard_normal((K, N))
    x = np.zeros((planes, R, 2, ldi), dtype=np.float32)
    x[..., :K] = rng.standard_normal((planes, R, 2, K)).astype(np.float32)
    ref = np.einsum("prck,kn->pncr", x[..., :K].astype(np.float64), B)
    ref32 = np.einsum("prck,kn->pncr", x[..., :K], B.astype(np.float32))
    err32 = np.abs(ref32 - ref).max() / np.abs(ref).max()
    xd = torch.tensor(x.reshape(-1), device="cuda")
    yd = torch.full((planes * N * 2 * ldo,), float("nan"), dtype=torch.float32, device="cuda")
    Bc = np.ascontiguousarray(B)
    s = torch.cuda.current_stream().cuda_stream
    _lib.check(lib.tdz_plane_transform(Bc.ctypes.data_as(C.POINTER(C.c_double)), K, N, C.c_void_p(xd.data_ptr()),
                                       planes, R, ldi, C.c_void_p(yd.data_ptr()), ldo, C.c_void_p(s)))
    y = yd.cpu().numpy().reshape(planes, N, 2, ldo)[..., :R]
    return np.abs(y - ref).max() / np.abs(ref).max(), err32


@pytest.mark.gpu
@pytest.mark.parametrize("K,N,planes,R,ldi,ldo", [
    (163, 163, 5, 163, 164, 164),     # heterostructure inner axis, 5 planes
    (163, 163, 130, 163, 164, 164),   # 331 row tiles: several per CTA, both TMEM accumulators in turn
    (7, 5, 3, 4, 8, 4),               # tiny, K < one 32-wide chunk, ragged tile
    (40, 256, 2, 70, 40, 72),         # widest N tile, K across two chunks
    (256, 16, 1, 300, 256, 300),      # narrowest N tile, K exactly 8 chunks, 5 M tiles
])
def test_plane_transform(cuda, K, N, planes, R, ldi, ldo):
    err, err32 = _run(K, N, planes, R, ldi, ldo, seed=K + N)
    assert err <= max(4 * err32, 1e-7) and err < 1e-5, (err, err32)


@pytest.mark.gpu
def test_plane_transform_rejects_bad_pitch(cuda):
    import torch
    from tdsez_gb300 import _lib
    lib = _lib.load()
    B = np.ones((6, 6))
    x = torch.zeros(64, device="cuda")
    y = torch.zeros(64, device="cuda")
    st = lib.tdz_plane_transform(B.ctypes.data_as(C.POINTER(C.c_double)), 6, 6, C.c_void_p(x.data_ptr()), 1, 2, 6,
                                 C.c_void_p(y.data_ptr()), 2, None)
    assert _lib.STATUS_NAMES[st] == "TDZ_ERR_ARG"
