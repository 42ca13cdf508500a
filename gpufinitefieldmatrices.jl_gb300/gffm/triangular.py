"""Triangular inverses and substitutions (src/CuModMatrix/triangular/), and the
reference's mod_inv.

``upper_triangular_inverse_no_copy`` / ``lower_triangular_inverse_no_copy``
(triangular_inverse_no_copy.jl:197-245, 450-477) and ``forward_sub_gpu_type_32``
/ ``backward_sub_gpu_type_32`` (substitution_inplace.jl:37-61) return a new
CuModMatrix of size (cols, rows), as the reference does; the work is libgffm's
``gffm_triangular_inverse_*`` (the reference's block recursion, 32-blocks by
substitution and the off-diagonal blocks on the limb tensor-core GEMM) and
``gffm_tri_sub32_*``.
"""
import ctypes

from . import cumod
from ._lib import GFFMError, call
from .cumod import _ptr, _stream


class InverseNotDefinedException(Exception):
    """InverseNotDefinedException (src/CuModMatrix/CuModMatrix.jl:29)."""


def mod_inv(p, P):
    """mod_inv(p, P) (src/CuModMatrix/rref_lu_pluq/pluq_kernels.jl:11-31): the extended
    Euclid result, 0 for p = 0 and a non-inverse when gcd(p, P) > 1."""
    out = ctypes.c_int64(0)
    call("gffm_mod_inv", int(p), int(P), ctypes.byref(out))
    return out.value


def _sfx(A):
    return cumod._sfx(A.dtype)


def _sub32(A, row_shift, col_shift, upper):
    m, n = A.rows(), A.cols()
    X = cumod.zeros(A.dtype, n, m, A.N)
    call("gffm_tri_sub32_%s" % _sfx(A), 1 if upper else 0, m, n, _ptr(A.data), A.ld, int(row_shift), int(col_shift),
         _ptr(X.data), X.ld, A.N, _stream())
    return X


def forward_sub_gpu_type_32(A, row_shift, col_shift):
    """forward_sub_gpu_type_32(A, row_shift, col_shift): the inverse of the 32 x 32
    lower-triangular window of A at (row_shift, col_shift), in the top-left of a
    new (cols x rows) CuModMatrix."""
    return _sub32(A, row_shift, col_shift, False)


def backward_sub_gpu_type_32(A, row_shift, col_shift):
    """backward_sub_gpu_type_32(A, row_shift, col_shift): the upper-triangular
    counterpart of forward_sub_gpu_type_32."""
    return _sub32(A, row_shift, col_shift, True)


def _inverse(A, upper):
    m, n = A.rows(), A.cols()
    X = cumod.zeros(A.dtype, n, m, A.N)
    try:
        call("gffm_triangular_inverse_%s" % _sfx(A), 1 if upper else 0, m, n, _ptr(A.data), A.ld, _ptr(X.data), X.ld,
             A.N, None, 0, _stream())
    except GFFMError as e:
        if e.status == 2:
            raise InverseNotDefinedException("(Right) pseudoinverse not defined for tall lower triangular matrices")
        raise
    return X


def upper_triangular_inverse_no_copy(A, debug=False):
    """upper_triangular_inverse_no_copy(A): the inverse of an upper-triangular
    CuModMatrix as a new (cols x rows) CuModMatrix; tall and wide inputs give the
    inverse of their leading square block.  ``debug`` (printing) is accepted and
    ignored."""
    return _inverse(A, True)


def lower_triangular_inverse_no_copy(A, debug=False):
    """lower_triangular_inverse_no_copy(A): the lower-triangular counterpart;
    InverseNotDefinedException for tall input wider than 32 columns."""
    return _inverse(A, False)


def triangular_inverse_into_(X, A, upper):
    """The same into a caller's (cols x rows) CuModMatrix X (no allocation of the result)."""
    if (X.rows(), X.cols()) != (A.cols(), A.rows()):
        raise cumod.CuModArraySizeMismatchException("Output matrix has incorrect dimensions")
    call("gffm_triangular_inverse_%s" % _sfx(A), 1 if upper else 0, A.rows(), A.cols(), _ptr(A.data), A.ld,
         _ptr(X.data), X.ld, A.N, None, 0, _stream())
    return X


def hensel_pseudoinverse(N, precision, A, T):
    """hensel_pseudoinverse(N, precision, A, T) (src/CuModMatrix/triangular/hensel.jl:13-20):
    the Newton iteration T <- 2T - T(AT), doubling the precision, that lifts a
    solution of AT = I mod N to one mod N^precision.  A and T are CuModMatrices;
    all arithmetic is mod M = N^precision (2 <= M < 2^26 for the exact GEMM).
    The reference returns a Nemo matrix over ZZ/M; here the result is a
    CuModMatrix with modulus M."""
    M = int(N) ** int(precision)
    i = 1
    T = cumod.change_modulus(T, M) if T.N != M else T
    while i < precision:
        AT = cumod.mat_mul_gpu_type(A, T, M)
        TAT = cumod.mat_mul_gpu_type(T, AT, M)
        T2 = cumod.similar(T, M)
        cumod.scalar_mul_(T2, T, 2, M)
        cumod.sub_(T2, T2, TAT, M)
        T = T2
        i *= 2
    return T


__all__ = ["InverseNotDefinedException", "mod_inv", "forward_sub_gpu_type_32", "backward_sub_gpu_type_32",
           "upper_triangular_inverse_no_copy", "lower_triangular_inverse_no_copy", "triangular_inverse_into_",
           "hensel_pseudoinverse"]
