"""ctypes binding of libtdz.so (the C ABI declared in include/tdz.h).

The library is built in-tree by ``tdsez_gb300.build``. Loading fails loudly
when it is missing: there is no CPU fallback for any operation.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "libtdz.so"

TDZ_OK = 0
TDZ_FP32, TDZ_FP64, TDZ_FP64_DF, TDZ_FP64_F32 = 0, 1, 2, 3
TDZ_MASS, TDZ_HAMILTONIAN, TDZ_DIPOLE_X, TDZ_DIPOLE_Y, TDZ_DIPOLE_Z, TDZ_STAGE = range(6)
TDZ_OBS_DIPOLES, TDZ_OBS_POPULATIONS, TDZ_OBS_ENERGIES, TDZ_OBS_CURRENTS, TDZ_OBS_AUTOCORRELATION = range(5)

STATUS_NAMES = {0: "TDZ_OK", 1: "TDZ_ERR_ARG", 2: "TDZ_ERR_CUDA", 3: "TDZ_ERR_NOT_CONVERGED",
                4: "TDZ_ERR_STATE", 5: "TDZ_ERR_UNSUPPORTED", 6: "TDZ_ERR_BREAKDOWN", 7: "TDZ_ERR_INTERNAL"}


class TDZError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


class tdz_physics(C.Structure):
    _fields_ = [
        ("charge", C.c_double),
        ("inv_mass", C.c_double),
        ("mass_axis", C.c_int),
        ("inv_mass_q", C.POINTER(C.c_double)),
        ("pot_q", C.POINTER(C.c_double) * 3),
        ("cap_q", C.POINTER(C.c_double) * 3),
        ("cap_inv_mass", C.c_double),
        ("coupled", C.c_int * 3),
        ("dirichlet", C.c_int),
        ("nsoft", C.c_int),
        ("soft", C.POINTER(C.c_double)),
    ]


class tdz_solver_opts(C.Structure):
    _fields_ = [
        ("restart", C.c_int),
        ("maxit", C.c_int),
        ("rtol", C.c_double),
        ("pc", C.c_int),
        ("pc_precision", C.c_int),
        ("mg_levels", C.c_int),
        ("mg_smooth", C.c_int),
        ("mg_coarse_its", C.c_int),
        ("outer_precision", C.c_int),
        ("mg_learned", C.c_int),
        ("relaxed", C.c_int),
        ("pc_refresh_its", C.c_int),
        ("mg_coarse", C.c_int),
    ]


class tdz_pc_refresh(C.Structure):
    _fields_ = [("base", C.c_int), ("rebuilds", C.c_int), ("cap", C.c_int)]


class tdz_tsurff_opts(C.Structure):
    _fields_ = [
        ("radius", C.c_double),
        ("nquad", C.c_int),
        ("nk", C.c_int * 3),
        ("kmin", C.c_double * 3),
        ("kmax", C.c_double * 3),
        ("mass", C.c_double),
        ("v0", C.c_double),
        ("charge", C.c_double),
        ("dt", C.c_double),
    ]


class tdz_tsurff_end_opts(C.Structure):
    _fields_ = [
        ("dp", C.c_double),
        ("cap_width", C.c_double),
        ("eta", C.c_double),
        ("rtol", C.c_double),
        ("maxit", C.c_int),
    ]


FIELD_FN = C.CFUNCTYPE(C.c_double, C.c_int, C.c_double, C.c_void_p)

TDZ_PC_NONE, TDZ_PC_MASS, TDZ_PC_MG, TDZ_PC_FDM, TDZ_PC_BAND = 0, 1, 2, 3, 4
TDZ_CN, TDZ_PADE22, TDZ_MAGNUS4 = 0, 1, 2

_lib = None

VP = C.c_void_p
PP = C.POINTER(C.c_void_p)
I = C.c_int
D = C.c_double
LL = C.c_longlong

# name -> (restype, argtypes); every symbol declared in include/tdz.h
SIGNATURES = {
    "tdz_last_error": (C.c_char_p, []),
    "tdz_version": (C.c_char_p, []),
    "tdz_launch_count": (LL, []),
    "tdz_space_create": (I, [I, C.POINTER(I), C.POINTER(I), C.POINTER(C.POINTER(D)), I, PP]),
    "tdz_space_axis": (I, [VP, I, C.POINTER(I), C.POINTER(I), C.POINTER(I)]),
    "tdz_space_ndof": (I, [VP, C.POINTER(LL)]),
    "tdz_space_quadrature": (I, [VP, I, C.POINTER(D), C.POINTER(D)]),
    "tdz_space_project": (I, [VP, I, C.POINTER(D), C.POINTER(D)]),
    "tdz_space_destroy": (None, [VP]),
    "tdz_operator_create": (I, [VP, C.POINTER(tdz_physics), PP]),
    "tdz_operator_set_stage": (I, [VP, D, D, D, D, I, C.POINTER(D)]),
    "tdz_operator_apply": (I, [VP, I, I, VP, VP, VP]),
    "tdz_operator_mass_solve": (I, [VP, I, VP, VP]),
    "tdz_operator_launches": (LL, [VP]),
    "tdz_operator_destroy": (None, [VP]),
    "tdz_vec_dot": (I, [VP, VP, LL, I, VP, VP]),
    "tdz_vec_mdot": (I, [C.POINTER(VP), I, VP, LL, I, VP, VP]),
    "tdz_vec_mdot_noalloc": (I, [C.POINTER(VP), I, VP, LL, I, VP, VP]),
    "tdz_solver_create": (I, [VP, C.c_void_p, VP, PP]),
    "tdz_solver_solve": (I, [VP, VP, VP, VP, C.POINTER(I), C.POINTER(I), C.POINTER(D)]),
    "tdz_solver_precondition": (I, [VP, VP, VP, VP]),
    "tdz_solver_destroy": (None, [VP]),
    "tdz_prop_create": (I, [VP, I, C.c_void_p, I, VP, PP]),
    "tdz_prop_step": (I, [VP, VP, D, C.POINTER(D), C.POINTER(D), VP]),
    "tdz_prop_stats": (I, [VP, C.POINTER(LL), C.POINTER(LL), C.POINTER(LL), C.POINTER(LL), C.POINTER(I),
                           C.POINTER(D)]),
    "tdz_prop_destroy": (None, [VP]),
    "tdz_tsurff_create": (I, [VP, C.c_void_p, FIELD_FN, VP, PP]),
    "tdz_tsurff_sample": (I, [VP, D, VP, VP]),
    "tdz_tsurff_amplitudes": (I, [VP, C.POINTER(D), VP]),
    "tdz_tsurff_volkov": (I, [VP, C.POINTER(D)]),
    "tdz_tsurff_interior": (I, [VP, VP, C.POINTER(D), VP]),
    "tdz_tsurff_end_term": (I, [VP, VP, C.c_void_p, C.c_void_p, VP, C.POINTER(D), C.POINTER(D), VP]),
    "tdz_tsurff_destroy": (None, [VP]),
    "tdz_solver_train_coarse": (I, [VP, I, I, C.c_float, C.c_ulonglong, C.POINTER(C.c_float), VP]),
    "tdz_solver_coarse_gain": (I, [VP, I, C.c_ulonglong, C.POINTER(C.c_double), C.POINTER(C.c_double), VP]),
    "tdz_set_autotune": (None, [I]),
    "tdz_set_apply3d_shape": (None, [I, I]),
    "tdz_eigen_solve": (I, [VP, I, D, D, I, C.c_void_p, VP, C.POINTER(D), C.POINTER(D), C.POINTER(I), VP]),
    "tdz_prop_refreshes": (I, [VP, C.POINTER(LL)]),
    "tdz_prop_record_coarse": (I, [VP, I]),
    "tdz_prop_train_coarse": (I, [VP, I, C.c_float, C.c_ulonglong, C.POINTER(C.c_float), C.POINTER(I), VP]),
    "tdz_pc_refresh_stale": (I, [C.POINTER(tdz_pc_refresh), I]),
    "tdz_strong_field_ratio": (I, [VP, I, D, D, FIELD_FN, VP, C.POINTER(D)]),
    "tdz_prop_step_batch": (I, [I, C.POINTER(VP), C.POINTER(VP), C.c_double, C.POINTER(C.POINTER(C.c_double)),
                                C.POINTER(C.POINTER(C.c_double)), C.POINTER(VP), I]),
    "tdz_observables": (I, [VP, VP, C.POINTER(C.c_double), VP]),
    "tdz_plane_transform": (I, [C.POINTER(C.c_double), I, I, VP, I, I, I, VP, I, VP]),
    "tdz_cnn_create": (I, [I, I, I, I, I, I, I, I, C.c_ulonglong, PP]),
    "tdz_cnn_forward": (I, [VP, VP, VP, I, VP]),
    "tdz_cnn_train_step": (I, [VP, VP, VP, I, C.c_float, VP]),
    "tdz_cnn_loss": (I, [VP, C.POINTER(C.c_float), VP]),
    "tdz_cnn_num_params": (I, [VP, C.POINTER(LL)]),
    "tdz_cnn_get_params": (I, [VP, C.POINTER(C.c_float)]),
    "tdz_cnn_set_params": (I, [VP, C.POINTER(C.c_float)]),
    "tdz_cnn_get_grads": (I, [VP, C.POINTER(C.c_float)]),
    "tdz_cnn_destroy": (None, [VP]),
    "tdz_tsurff_info": (I, [VP, C.POINTER(D)]),
    "tdz_h5_write": (I, [C.c_char_p, I, C.POINTER(C.c_char_p), C.POINTER(I), C.POINTER(LL),
                         C.POINTER(C.POINTER(D)), I, C.POINTER(C.c_char_p), C.POINTER(LL), C.POINTER(C.POINTER(D))]),
    "tdz_obsfile_open": (I, [C.c_char_p, I, I, LL, PP]),
    "tdz_obsfile_columns": (I, [VP, I]),
    "tdz_obsfile_record": (I, [VP, D, C.POINTER(C.POINTER(D))]),
    "tdz_obsfile_rows": (I, [VP, C.POINTER(LL), C.POINTER(LL)]),
    "tdz_obsfile_flush": (I, [VP]),
    "tdz_obsfile_close": (I, [VP]),
}


def load():
    """Load libtdz.so (building it first when it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        from . import build as _build
        _build.build()
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int):
    if status != TDZ_OK:
        msg = load().tdz_last_error().decode(errors="replace")
        raise TDZError(status, msg)


def dptr(arr):
    """POINTER(c_double) of a contiguous float64 numpy array (or None)."""
    if arr is None:
        return None
    return arr.ctypes.data_as(C.POINTER(C.c_double))
