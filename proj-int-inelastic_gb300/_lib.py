"""ctypes binding of ``libpii_gb300.so`` (the C ABI in ``include/pii_gb300.h``).

The shared library is built in-tree by ``build.py``.  Loading fails loudly if
it is missing: there is no CPU fallback for any operator of this package.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpii_gb300.so")

PII_OK = 0
PII_ERR_ARG = -1
PII_ERR_CUDA = -2
PII_ERR_SIZE = -3
PII_ERR_NONFINITE = -4
PII_ERR_STALL = -5

PREC_FP32 = 0
PREC_FP64 = 1

BC_EXTRAP = 1
BC_PERIODIC = 2

INT_EULER = 0
INT_PFE = 1
INT_TPI2 = 2
INT_TPI3 = 3
INT_CONSP = 4
INT_CONSP_M = 5

_c_int, _c_i64, _c_dbl, _vp = ctypes.c_int, ctypes.c_int64, ctypes.c_double, ctypes.c_void_p
_pdbl = ctypes.POINTER(ctypes.c_double)
_pint = ctypes.POINTER(ctypes.c_int)

# name -> (restype, argtypes): exactly the declarations of include/pii_gb300.h
SIGNATURES = {
    "pii_last_error": (ctypes.c_char_p, []),
    "pii_version": (ctypes.c_char_p, []),
    "pii_plan_create": (_c_int, [ctypes.POINTER(_vp), _c_int, _c_int, _c_int, _pdbl, _pdbl, _pdbl, _c_dbl, _c_dbl,
                                 _c_dbl, _c_dbl, _c_dbl, _c_dbl, _c_int, _c_i64, _c_int]),
    "pii_plan_create_nd": (_c_int, [ctypes.POINTER(_vp), _c_int, _c_int, _c_int, _c_int, _pdbl, _pdbl, _pdbl, _c_dbl,
                                    _c_dbl, _c_dbl, _c_dbl, _c_dbl, _c_dbl, _c_int, _c_i64, _c_int]),
    "pii_plan_dim": (_c_int, [_vp]),
    "pii_plan_set_restitution": (_c_int, [_vp, _pdbl, _pdbl, _c_i64]),
    "pii_plan_destroy": (_c_int, [_vp]),
    "pii_plan_workspace_bytes": (_c_i64, [_vp]),
    "pii_plan_set_gain_path": (_c_int, [_vp, _c_int]),
    "pii_plan_autotune": (_c_int, [_vp, _c_i64, _pdbl, _vp]),
    "pii_plan_get_tuning": (_c_int, [_vp, _pint, _pint, ctypes.POINTER(ctypes.c_int64)]),
    "pii_plan_set_tuning": (_c_int, [_vp, _c_int, _c_int, _c_i64]),
    "pii_plan_set_dft_path": (_c_int, [_vp, _c_int]),
    "pii_plan_get_dft_path": (_c_int, [_vp, _pint, _pint]),
    "pii_plan_set_fused_split": (_c_int, [_vp, ctypes.c_double]),
    "pii_plan_get_fused_split": (ctypes.c_double, [_vp]),
    "pii_plan_dft_test_hooks": (_c_int, [_vp, ctypes.c_uint32, _c_int]),
    "pii_plan_set_nyquist_path": (_c_int, [_vp, _c_int]),
    "pii_plan_get_nyquist_path": (_c_int, [_vp]),
    "pii_collide": (_c_int, [_vp, _vp, _vp, _c_i64, _c_int, _c_dbl, _c_int, _vp]),
    "pii_laplacian": (_c_int, [_vp, _vp, _vp, _c_i64, _vp]),
    "pii_transport_df": (_c_int, [_vp, _vp, _vp, _c_i64, _c_dbl, _c_dbl, _pdbl, _c_int, _c_int, _vp]),
    "pii_boltzmann_df": (_c_int, [_vp, _vp, _vp, _c_i64, _c_dbl, _c_dbl, _pdbl, _c_int, _c_int, _c_dbl, _c_int,
                                  _c_int, _vp]),
    "pii_step": (_c_int, [_vp, _c_int, _vp, _c_i64, _c_dbl, _pint, _pdbl, _c_int, _c_dbl, _pdbl, _c_int, _c_int,
                          _c_dbl, _c_int, _c_int, _c_int, _vp]),
    "pii_step_splitting": (_c_int, [_vp, _c_int, _vp, _c_i64, _c_dbl, _c_dbl, _pdbl, _c_int, _c_int, _c_dbl, _c_dbl,
                                    _c_dbl, _c_dbl, _c_int, _c_int, _c_int, _vp]),
    "pii_state_check": (_c_int, [_vp, _vp, _vp, _c_i64, _pdbl, _c_dbl, _vp]),
    "pii_moments": (_c_int, [_vp, _vp, _vp, _c_i64, _pdbl, _c_dbl, _vp]),
    "pii_fast_sweep": (_c_int, [_vp, _vp, _vp, _c_i64, _c_dbl, _c_dbl, _pdbl, _pdbl, _vp]),
    "pii_axpby": (_c_int, [_vp, _vp, _c_dbl, _c_dbl, _c_i64, _vp]),
    "pii_collide_noalloc": (_c_int, [_vp, _vp, _c_i64, _c_int, _c_int, _c_int, _pdbl, _pdbl, _pdbl, _c_dbl, _c_dbl,
                                     _c_dbl, _c_dbl, _c_dbl, _c_dbl, _c_int, _vp]),
    "pii_kernel_launches": (_c_i64, []),
    "pii_plan_graph_count": (_c_i64, [_vp]),
    "pii_plan_profile": (_c_int, [_vp, _c_int]),
    "pii_plan_profile_read": (_c_int, [_vp, _pdbl, ctypes.POINTER(ctypes.c_int64)]),
}

NSTAGES = 15
STAGES = ["fwd_plane", "col_fwd", "col_pstart", "pair_plane", "col_pend", "reduce", "col_iprep", "finish", "df",
          "axpy", "massfix", "gain_cluster", "gain_parity", "nyq_corr", "gain_fused"]

_lib = None


def load():
    """Load the library once; raise ImportError if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build it with `python -c \"import __graft_entry__ as g; g.build()\"` "
                "(the operator has no CPU fallback)"
            )
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def last_error():
    return load().pii_last_error().decode()


def check(status, what):
    """Raise the Python exception the reference would raise for a failing call."""
    if status == PII_OK:
        return
    msg = f"{what}: {last_error()}"
    if status in (PII_ERR_ARG, PII_ERR_SIZE):
        raise ValueError(msg)
    if status == PII_ERR_NONFINITE:
        raise FloatingPointError(msg)
    raise RuntimeError(msg)


def dptr(x):
    """Double-array pointer for a host numpy array (kept alive by the caller)."""
    return x.ctypes.data_as(_pdbl)


def iptr(x):
    return x.ctypes.data_as(_pint)
