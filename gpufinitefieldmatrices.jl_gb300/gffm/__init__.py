"""gffm -- GB300-native drop-in for the hot path of GPUFiniteFieldMatrices.jl.

Host-side mirror of the reference's CuModMatrix / KaratsubaMatrix interface
over the C ABI of libgffm (include/gffm.h).  Every operation runs a CUDA
kernel of libgffm; there is no CPU fallback.
"""
from ._lib import GFFMError, load as load_library, lib_path  # noqa: F401
from .build import build  # noqa: F401
from .cumod import (  # noqa: F401
    TILE_WIDTH, DEFAULT_TYPE, CuModArray, CuModMatrix, CuModVector, wrap, zeros, eye, rand, similar, copy,
    add_, sub_, elementwise_multiply_, scalar_add_, scalar_sub_, rscalar_sub_, scalar_mul_, negate_,
    mod_, mod_elements_, fill_, zero_, copy_, change_modulus, change_modulus_no_alloc_, div_,
    mul_, stripe_mul_, mat_mul_gpu_type, mat_mul_type_inplace_, find_max_stripe_ops, limbs_for, LimbTuning,
    matmul_host, host_matrix,
    CuModArraySizeMismatchException, CuModArrayModulusMismatchException, CuModMatrixNotSquareException,
    CuModMatrixModulusNotPrimeException,
)
from .elimination import (  # noqa: F401,E402
    pluq_gpu_kernel, lu_gpu_type, rref_gpu_type, apply_col_perm_, apply_col_inv_perm_, apply_col_perm,
    apply_row_perm_, apply_row_inv_perm_, apply_row_perm, perm_array_to_matrix,
    inverse, is_invertible, is_invertible_with_inverse, MatrixNotInvertibleException,
)
from . import cumod as _cumod, karatsuba as _karatsuba  # noqa: E402
from .karatsuba import (  # noqa: F401,E402
    KaratsubaArray, KaratsubaMatrix, KaratsubaVector, KaratsubaZeros, KaratsubaMatrix_from, Karatsubacopy,
    initialize_plan_, KMatMul_, KMatMul_gemv_, MatToKMat, KMatToMat, poly_karatsuba_matmul, scalar_multiply_,
    find_max_ops, find_max_ops_karatsuba, nKMuls, divide_elements_,
)


def _dispatch(name):
    """Julia's multiple dispatch for the names both types define (add!, sub!, negate!, zero!, copy!)."""
    on_mod, on_k = getattr(_cumod, name), getattr(_karatsuba, name)

    def f(*args, **kw):
        return (on_k if isinstance(args[0], KaratsubaArray) else on_mod)(*args, **kw)

    f.__name__ = name
    f.__doc__ = "%s for CuModArray (%s) or KaratsubaArray (%s)" % (name, on_mod.__doc__, on_k.__doc__)
    return f


add_ = _dispatch("add_")
sub_ = _dispatch("sub_")
negate_ = _dispatch("negate_")
zero_ = _dispatch("zero_")
copy_ = _dispatch("copy_")
from .batched import BatchPlan, Tuning as BatchTuning, batched_plan  # noqa: F401,E402
from . import autotune  # noqa: F401,E402
from .triangular import (  # noqa: F401,E402
    InverseNotDefinedException, mod_inv, forward_sub_gpu_type_32, backward_sub_gpu_type_32,
    upper_triangular_inverse_no_copy, lower_triangular_inverse_no_copy, triangular_inverse_into_,
    hensel_pseudoinverse,
)
