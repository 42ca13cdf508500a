"""ctypes binding of libgffm (include/gffm.h).

This is the Python counterpart of the ``ccall`` stubs a Julia binding of the
library would declare: plain pointers, sizes and a stream handle.  Loading
fails loudly when the library has not been built -- there is no fallback.
"""
import ctypes
import os

from . import build as _build

_I64 = ctypes.c_int64
_P = ctypes.c_void_p
_D = ctypes.c_double
_F = ctypes.c_float
_INT = ctypes.c_int
_SZ = ctypes.c_size_t
_PI64 = ctypes.POINTER(ctypes.c_int64)
_PSZ = ctypes.POINTER(ctypes.c_size_t)

# name -> (restype, argtypes)
SIGNATURES = {
    "gffm_version": (ctypes.c_char_p, []),
    "gffm_last_error_string": (ctypes.c_char_p, []),
    "gffm_device_status": (_INT, [_P]),
    "gffm_profile_next_kernel": (_INT, [_P, _P]),
    "gffm_find_max_stripe_ops": (_INT, [_INT, _I64, _PI64]),
    "gffm_matmul_plain_f64": (_INT, [_I64, _I64, _I64, _P, _I64, _P, _I64, _P, _I64, _I64, _I64, _P]),
    "gffm_matmul_plain_f32": (_INT, [_I64, _I64, _I64, _P, _I64, _P, _I64, _P, _I64, _I64, _I64, _P]),
    "gffm_matvec_plain_f64": (_INT, [_I64, _I64, _P, _I64, _P, _P, _I64, _I64, _P]),
    "gffm_matvec_plain_f32": (_INT, [_I64, _I64, _P, _I64, _P, _P, _I64, _I64, _P]),
    "gffm_matmul_limb_workspace_size": (_INT, [_I64, _I64, _I64, _I64, _PSZ]),
    "gffm_matmul_limb_f64": (_INT, [_I64, _I64, _I64, _P, _I64, _P, _I64, _P, _I64, _I64, _P, _SZ, _P]),
    "gffm_matmul_limb_f32": (_INT, [_I64, _I64, _I64, _P, _I64, _P, _I64, _P, _I64, _I64, _P, _SZ, _P]),
    "gffm_elim_workspace_size": (_INT, [_I64, _I64, _I64, _PSZ]),
    "gffm_pluq_f64": (_INT, [_I64, _I64, _P, _I64, _P, _I64, _P, _I64, _I64, _I64, _P, _P, _P, _P, _P, _P, _SZ, _P]),
    "gffm_pluq_plain_f64": (_INT, [_I64, _I64, _P, _I64, _P, _I64, _P, _I64, _I64, _I64, _P, _P, _P, _P, _P, _P, _SZ,
                                   _P]),
    "gffm_pluq_f32": (_INT, [_I64, _I64, _P, _I64, _P, _I64, _P, _I64, _I64, _I64, _P, _P, _P, _P, _P, _P, _SZ, _P]),
    "gffm_lu_f64": (_INT, [_I64, _I64, _P, _I64, _P, _I64, _P, _I64, _I64, _P, _P, _P, _SZ, _P]),
    "gffm_lu_f32": (_INT, [_I64, _I64, _P, _I64, _P, _I64, _P, _I64, _I64, _P, _P, _P, _SZ, _P]),
    "gffm_rref_f64": (_INT, [_I64, _I64, _P, _I64, _P, _I64, _I64, _P, _P, _P, _SZ, _P]),
    "gffm_rref_f32": (_INT, [_I64, _I64, _P, _I64, _P, _I64, _I64, _P, _P, _P, _SZ, _P]),
    "gffm_apply_row_swaps_f64": (_INT, [_P, _I64, _I64, _I64, _P, _I64, _INT, _P]),
    "gffm_apply_row_swaps_f32": (_INT, [_P, _I64, _I64, _I64, _P, _I64, _INT, _P]),
    "gffm_apply_col_swaps_f64": (_INT, [_P, _I64, _I64, _I64, _P, _I64, _INT, _P]),
    "gffm_apply_col_swaps_f32": (_INT, [_P, _I64, _I64, _I64, _P, _I64, _INT, _P]),
    "gffm_matmul_limb_static_max_bytes": (_INT, [_PSZ]),
    "gffm_matmul_limb_static_scratch_size": (_INT, [_I64, _I64, _I64, _I64, _PSZ]),
    "gffm_matmul_limb_static_f64": (_INT, [_I64, _I64, _I64, _P, _I64, _P, _I64, _P, _I64, _I64, _P]),
    "gffm_matmul_host_workspace_size": (_INT, [_I64, _I64, _I64, _I64, _PSZ]),
    "gffm_div_scalar_f64": (_INT, [_P, _P, _I64, _I64, _I64, _P]),
    "gffm_div_scalar_f32": (_INT, [_P, _P, _I64, _I64, _I64, _P]),
    "gffm_trunc_div_f64": (_INT, [_P, _P, _I64, _I64, _P]),
    "gffm_trunc_div_f32": (_INT, [_P, _P, _I64, _I64, _P]),
    "gffm_mod_inv": (_INT, [_I64, _I64, ctypes.POINTER(ctypes.c_int64)]),
    "gffm_tri_sub32_f64": (_INT, [ctypes.c_int, _I64, _I64, _P, _I64, _I64, _I64, _P, _I64, _I64, _P]),
    "gffm_tri_sub32_f32": (_INT, [ctypes.c_int, _I64, _I64, _P, _I64, _I64, _I64, _P, _I64, _I64, _P]),
    "gffm_triangular_inverse_workspace_size": (_INT, [ctypes.c_int, _I64, _I64, _I64, _PSZ]),
    "gffm_triangular_inverse_f64": (_INT, [ctypes.c_int, _I64, _I64, _P, _I64, _P, _I64, _I64, _P, _SZ, _P]),
    "gffm_triangular_inverse_f32": (_INT, [ctypes.c_int, _I64, _I64, _P, _I64, _P, _I64, _I64, _P, _SZ, _P]),
    "gffm_matmul_host_f64": (_INT, [_I64, _I64, _I64, _P, _I64, _P, _I64, _P, _I64, _I64, _P, _SZ, _P]),
}
for _op in ("add", "sub", "mul_elementwise"):
    SIGNATURES["gffm_%s_f64" % _op] = (_INT, [_P, _P, _P, _I64, _I64, _P])
    SIGNATURES["gffm_%s_f32" % _op] = (_INT, [_P, _P, _P, _I64, _I64, _P])
for _op in ("scalar_add", "scalar_sub", "rscalar_sub", "scalar_mul"):
    SIGNATURES["gffm_%s_f64" % _op] = (_INT, [_P, _P, _D, _I64, _I64, _P])
    SIGNATURES["gffm_%s_f32" % _op] = (_INT, [_P, _P, _F, _I64, _I64, _P])
SIGNATURES["gffm_mod_f64"] = (_INT, [_P, _P, _I64, _I64, _P])
SIGNATURES["gffm_mod_f32"] = (_INT, [_P, _P, _I64, _I64, _P])
SIGNATURES.update({
    "gffm_karatsuba_workspace_size": (_INT, [_I64, _I64, _I64, _I64, _I64, _PSZ]),
    "gffm_karatsuba_matmul_f64": (_INT, [_I64, _I64, _I64, _P, _P, _I64, _P, _P, _I64, _P, _P, _I64, _I64, _I64,
                                         _P, _SZ, _P]),
    "gffm_karatsuba_poly_workspace_size": (_INT, [_I64, _I64, _I64, _I64, _PSZ]),
    "gffm_karatsuba_poly_matmul_f64": (_INT, [_I64, _I64, _I64, _P, _P, _I64, _P, _P, _I64, _P, _P, _P, _I64, _I64,
                                              _P, _SZ, _P]),
    "gffm_karatsuba_add_f64": (_INT, [_P, _P, _P, _P, _P, _P, _I64, _I64, _I64, _P]),
    "gffm_karatsuba_sub_f64": (_INT, [_P, _P, _P, _P, _P, _P, _I64, _I64, _I64, _P]),
    "gffm_karatsuba_negate_f64": (_INT, [_P, _P, _P, _P, _I64, _I64, _I64, _P]),
    "gffm_karatsuba_scalar_mul_f64": (_INT, [_P, _P, _P, _P, _I64, _I64, _I64, _I64, _P]),
    "gffm_karatsuba_from_values_f64": (_INT, [_P, _P, _P, _I64, _I64, _I64, _P]),
    "gffm_karatsuba_to_values_f64": (_INT, [_P, _P, _P, _I64, _I64, _I64, _P]),
    "gffm_tune_table_set": (_INT, [_P, _I64]),
    "gffm_tune_table_size": (_INT, [_PI64]),
    "gffm_matmul_limb_tuned_workspace_size": (_INT, [_I64, _I64, _I64, _I64, _P, _PSZ]),
    "gffm_matmul_limb_tuned_f64": (_INT, [_I64, _I64, _I64, _P, _I64, _P, _I64, _P, _I64, _I64, _P, _P, _SZ, _P]),
    "gffm_inverse_workspace_size": (_INT, [_I64, _PSZ]),
    "gffm_inverse_f64": (_INT, [_I64, _P, _I64, _P, _I64, _I64, _P, _P, _SZ, _P]),
    "gffm_inverse_f32": (_INT, [_I64, _P, _I64, _P, _I64, _I64, _P, _P, _SZ, _P]),
    "gffm_batched_plan_create": (_INT, [_P, _I64, _P, _P]),
    "gffm_batched_plan_info": (_INT, [_P, _PI64]),
    "gffm_batched_run": (_INT, [_P, _P]),
    "gffm_batched_plan_destroy": (_INT, [_P]),
})

STATUS = {
    0: "GFFM_OK", 1: "GFFM_ERR_ARG", 2: "GFFM_ERR_SIZE", 3: "GFFM_ERR_MODULUS", 4: "GFFM_ERR_STRIPE",
    5: "GFFM_ERR_WORKSPACE", 6: "GFFM_ERR_CUDA", 7: "GFFM_ERR_TIMEOUT", 8: "GFFM_ERR_BOUNDS",
    9: "GFFM_ERR_NOT_PRIME", 10: "GFFM_ERR_UNSUPPORTED",
}

_lib = None


class GFFMError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s: %s" % (STATUS.get(status, str(status)), message))
        self.status = status


def lib_path():
    return _build.LIB_PATH


def load(path=None):
    """Load libgffm.so (built in-tree by gffm.build / __graft_entry__.build())."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or _build.LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError("libgffm.so is not built (%s); run __graft_entry__.build()" % path)
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    # install the shipped autotune table (gffm/tuning.json) as the library's tune table
    from . import autotune
    autotune.apply()
    return L


def call(name, *args):
    """Call a gffm entry point and raise GFFMError on a non-zero status."""
    L = load()
    st = getattr(L, name)(*args)
    if st != 0:
        msg = L.gffm_last_error_string()
        raise GFFMError(st, msg.decode() if msg else "")
    return st
