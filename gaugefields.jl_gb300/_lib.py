"""ctypes binding of libgfgb300.so (the C-ABI declared in include/gaugefields_gb300.h).

There is no CPU fallback: if the library is missing or cannot be loaded, every
entry point raises.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgfgb300.so")

GF_OK = 0
GF_EINVAL = -1
GF_ENOMEM = -2
GF_ECUDA = -3
GF_ENAN = -4
GF_ESTATE = -5

GF_LINK64, GF_LINK32, GF_MOM64, GF_MAT64, GF_MAT32 = 1, 2, 3, 4, 5
GF_FP64, GF_MIXED, GF_DFLOAT = 0, 1, 2
GF_QPQ, GF_PQP, GF_OMELYAN = 0, 1, 2
GF_MAX_STOUT = 4


class GFError(RuntimeError):
    """A CUDA-side failure reported by the library."""

    def __init__(self, code, msg):
        super().__init__("%s (status %d)" % (msg, code))
        self.code = code


class GFNonFinite(GFError):
    """A non-finite Delta H (the trajectory is rejected)."""


class MDParams(ctypes.Structure):
    _fields_ = [
        ("beta", ctypes.c_double),
        ("tau", ctypes.c_double),
        ("steps", ctypes.c_int),
        ("integrator", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("nstout", ctypes.c_int),
        ("rho", ctypes.c_double * GF_MAX_STOUT),
        ("reunitarize", ctypes.c_int),
        ("stout_recompute", ctypes.c_int),
        ("lam", ctypes.c_double),
        ("c_rect", ctypes.c_double),
    ]


_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double
_U64 = ctypes.c_uint64
_DP = ctypes.POINTER(ctypes.c_double)

# name -> argument types (all return int status, except gf_last_error)
SIGNATURES = {
    "gf_ctx_create": [ctypes.POINTER(ctypes.c_int), _I, ctypes.POINTER(_P)],
    "gf_ctx_destroy": [_P],
    "gf_ctx_set_stream": [_P, _P],
    "gf_ctx_synchronize": [_P],
    "gf_ctx_volume": [_P, ctypes.POINTER(ctypes.c_int64)],
    "gf_field_alloc": [_P, _I, ctypes.POINTER(_P)],
    "gf_field_free": [_P],
    "gf_field_kind": [_P, ctypes.POINTER(ctypes.c_int)],
    "gf_field_bytes": [_P, ctypes.POINTER(ctypes.c_size_t)],
    "gf_field_device_ptr": [_P, ctypes.POINTER(_P)],
    "gf_field_copy": [_P, _P, _P],
    "gf_field_zero": [_P, _P],
    "gf_upload_links": [_P, _P, _P],
    "gf_download_links": [_P, _P, _P],
    "gf_upload_mom": [_P, _P, _P],
    "gf_download_mom": [_P, _P, _P],
    "gf_cold_start": [_P, _P],
    "gf_hot_start": [_P, _P, _U64],
    "gf_gaussian_momenta": [_P, _P, _U64, _U64],
    "gf_mom_scale": [_P, _P, _D],
    "gf_reunitarize": [_P, _P],
    "gf_plaquette": [_P, _P, _DP],
    "gf_action": [_P, _P, _D, _DP],
    "gf_rectangle": [_P, _P, _DP],
    "gf_action_loops": [_P, _P, _D, _D, _DP],
    "gf_kinetic": [_P, _P, _DP],
    "gf_staple": [_P, _P, _I, _P],
    "gf_force": [_P, _P, _D, _P],
    "gf_force_loops": [_P, _P, _D, _D, _P],
    "gf_mom_update": [_P, _P, _P, _D, _D],
    "gf_link_update": [_P, _P, _P, _D, _I],
    "gf_hamiltonian": [_P, _P, _P, ctypes.POINTER(MDParams), _DP],
    "gf_md_trajectory": [_P, _P, _P, ctypes.POINTER(MDParams), _DP],
    "gf_md_mom_update": [_P, _P, _P, _D, ctypes.POINTER(MDParams)],
    "gf_md_link_update": [_P, _P, _P, _D, ctypes.POINTER(MDParams)],
    "gf_hmc_update": [_P, _P, _P, ctypes.POINTER(MDParams), _U64, _U64, _D, _DP],
    "gf_stout_create": [_P, _I, _DP, _I, _I, ctypes.POINTER(_P)],
    "gf_stout_destroy": [_P],
    "gf_stout_forward": [_P, _P, _P, _P],
    "gf_stout_backward": [_P, _P, _P, _P],
    "gf_stout_mom_update": [_P, _P, _P, _P, _D, _D],
    "gf_stout_param_derivatives": [_P, _P, _P, _P, _P],
    "gf_field_axpy": [_P, _P, _D, _P],
    "gf_flow": [_P, _P, _D, _I],
    "gf_flow_precision": [_P, _P, _D, _I, _I],
    "gf_flow_loops": [_P, _P, _D, _I, _D, _D],
    "gf_flow_force": [_P, _P, _P, _D],
    "gf_prof_enable": [_P, _I],
    "gf_prof_read": [_P, _I, _DP, ctypes.POINTER(ctypes.c_longlong)],
    "gf_launch_count": [ctypes.POINTER(ctypes.c_longlong)],
    "gf_plaquette_noalloc": [_P, ctypes.POINTER(ctypes.c_int), _P, _P],
    "gf_polyakov_loop": [_P, _P, _DP],
}

KERNEL_CLASSES = ["plaquette", "force", "link_update", "stout_fwd", "bwd_local", "bwd_gather", "stout_fwd64",
                  "bwd_local64", "bwd_gather64", "other", "link_update_df", "stout_fwd_df", "force_df",
                  "bwd_local_df", "bwd_gather_df", "rect", "rect_df"]
# arithmetic precision of each class (the force class follows its links)
KERNEL_PRECISION = {"plaquette": "fp64", "force": "fp32", "link_update": "fp64", "stout_fwd": "fp32",
                    "bwd_local": "fp32", "bwd_gather": "fp32", "stout_fwd64": "fp64", "bwd_local64": "fp64",
                    "bwd_gather64": "fp64", "other": "fp64", "link_update_df": "df", "stout_fwd_df": "df",
                    "force_df": "df", "bwd_local_df": "df", "bwd_gather_df": "df",
                    "rect": "fp64", "rect_df": "df"}

_lib = None


def load(path=LIB_PATH):
    """Load the CUDA library (raises if it is absent: there is no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError("libgfgb300.so not found at %s: build it with __graft_entry__.build()" % path)
    lib = ctypes.CDLL(path)
    for name, args in SIGNATURES.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = ctypes.c_int
    lib.gf_last_error.argtypes = [_P]
    lib.gf_last_error.restype = ctypes.c_char_p
    _lib = lib
    return lib


def exported_symbols():
    return list(SIGNATURES) + ["gf_last_error"]


def check(rc, ctx=None):
    if rc == GF_OK:
        return
    lib = load()
    msg = lib.gf_last_error(ctx).decode(errors="replace") if lib else ""
    if rc == GF_EINVAL:
        raise ValueError(msg)
    if rc == GF_ENAN:
        raise GFNonFinite(rc, msg)
    raise GFError(rc, msg)


def call(name, *args, ctx=None):
    rc = getattr(load(), name)(*args)
    check(rc, ctx)
