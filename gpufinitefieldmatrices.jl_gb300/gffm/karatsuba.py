"""KaratsubaArray / KaratsubaMatrix / KaratsubaVector: the reference's two-digit
type (src/KaratsubaMatrix/KaratsubaMatrix.jl) over libgffm.

An element is the pair of digits (d1, d2) of the value d1 + N1*d2 in
Z/(N1*N2) (KaratsubaMatrix.jl:304,318-336); ``data1`` and ``data2`` are
CuModArrays (both carrying modulus N1, as the reference constructs them).
``M`` is the tag the reference compares between operands ("Matrices must have
the same modulus m").  Products and digit arithmetic are exact in Z/(N1*N2);
they equal the reference's kernels whenever N2 divides N1, which holds for
every modulus pair the reference builds (MatToKMat uses N1 = N2 = M).
"""
import ctypes

import numpy as np
import torch

from . import cumod
from ._lib import call
from .cumod import CuModArray, _ptr, _stream

nKMuls = 3   # component products per Karatsuba product (KaratsubaMatrix.jl:211)

_BITS = {torch.float64: 51, torch.float32: 22, torch.float16: 9}   # get_bits (CuModMatrix.jl:188-206)


def get_bits(dtype):
    if dtype not in _BITS:
        raise TypeError("Input type is not recognized.")
    return _BITS[dtype]


def find_max_ops(dtype, N):
    """find_max_ops(type, N) (CuModMatrix.jl:208-216)."""
    return (2 ** get_bits(dtype) - 1) // (int(N) ** 2) - 1


def find_max_ops_karatsuba(dtype, N):
    """find_max_ops_karatsuba(type, N) (KaratsubaMatrix.jl:104-131)."""
    return find_max_ops(dtype, N)


class KaratsubaArray:
    """KaratsubaArray{T,D}(A, B[, N1, N2, M]) (KaratsubaMatrix.jl:1-52)."""

    def __init__(self, data1, data2, N1=None, N2=None, M=None):
        if data1.size != data2.size:
            raise ValueError("Dimensions of matrices must match")
        if N1 is None:
            M = find_max_ops(data1.dtype, max(data1.size + data2.size))
            N1 = N2 = M
        elif M >= 2 ** get_bits(data1.dtype):
            raise ValueError("Modulus too large")
        self.data1 = data1
        self.data2 = data2
        self.plan = None
        self.N1, self.N2, self.M = int(N1), int(N2), int(M)

    @property
    def size(self):
        return self.data1.size

    @property
    def ndim(self):
        return self.data1.ndim

    def __len__(self):
        return len(self.data1)

    def __getitem__(self, idx):
        """getindex: d1 + N1*d2 (KaratsubaMatrix.jl:304-305), 1-based like the reference."""
        if isinstance(idx, tuple):
            i, j = idx
            return int(self.data1.Array()[i - 1, j - 1]) + self.N1 * int(self.data2.Array()[i - 1, j - 1])
        a1 = self.data1.Array().reshape(-1, order="F")
        a2 = self.data2.Array().reshape(-1, order="F")
        return int(a1[idx - 1]) + self.N1 * int(a2[idx - 1])

    def __setitem__(self, idx, v):
        """setindex!: d1 = rem(v, N1), d2 = div(v, N1) (KaratsubaMatrix.jl:307-315)."""
        v = int(v)
        q = abs(v) // self.N1 * (1 if v >= 0 else -1)        # Julia div truncates
        r = v - q * self.N1
        for arr, val in ((self.data1, r), (self.data2, q)):
            if isinstance(idx, tuple):
                i, j = idx
                arr.data[j - 1, i - 1] = float(val)
            else:
                if arr.ndim == 1:
                    arr.data[idx - 1] = float(val)
                else:
                    rows = arr.rows()
                    arr.data[(idx - 1) // rows, (idx - 1) % rows] = float(val)

    def Array(self):
        """Array(K): the values d1 + N1*d2 as int64 (KaratsubaMatrix.jl:318-336)."""
        return self.data1.Array().astype(np.int64) + self.N1 * self.data2.Array().astype(np.int64)

    def __add__(self, other):
        K = _like(self)
        initialize_plan_(K)
        return add_(K, self, other)

    def __sub__(self, other):
        K = _like(self)
        return sub_(K, self, other)

    def __neg__(self):
        K = _like(self)
        return negate_(K, self)

    def __mul__(self, other):
        if isinstance(other, KaratsubaArray):
            rows = self.data1.rows()
            if other.ndim == 1:
                K = KaratsubaZeros(self.data1.dtype, rows, self.N1, self.N2, self.M, True)
            else:
                K = KaratsubaZeros(self.data1.dtype, rows, other.data1.cols(), self.N1, self.N2, self.M, True)
            for X in (self, other, K):
                if X.plan is None:
                    initialize_plan_(X)
            return KMatMul_(K, self, other)
        K = _like(self)
        return scalar_multiply_(K, self, other)

    def __rmul__(self, s):
        return self.__mul__(s)

    def __matmul__(self, other):
        return self.__mul__(other)


KaratsubaMatrix_t = KaratsubaArray
KaratsubaVector_t = KaratsubaArray


def _zeros_like_digits(A, N):
    if A.ndim == 1:
        return cumod.zeros(A.dtype, A.size[0], N)
    return cumod.zeros(A.dtype, A.size[0], A.size[1], N)


def _like(K):
    return KaratsubaArray(_zeros_like_digits(K.data1, K.data1.N), _zeros_like_digits(K.data2, K.data1.N),
                          K.N1, K.N2, K.M)


def KaratsubaMatrix(A, B=None, N1=None, N2=None, M=None, elem_type=torch.float64):
    """KaratsubaMatrix(A, B[, M] | [, N1, N2, M]) (KaratsubaMatrix.jl:61-71).

    A and B are the digit matrices: CuModArrays, or host arrays that become
    CuModMatrices of modulus N1 (the reference's tests pass CuModMatrix digits)."""
    if N1 is not None and N2 is None and M is None:          # KaratsubaMatrix(A, B, M)
        N1 = N2 = M = N1
    if not isinstance(A, CuModArray):
        mod = N1 if N1 is not None else 2 ** 52
        A = cumod.CuModMatrix(A, mod, mod=False, elem_type=elem_type)
        B = cumod.CuModMatrix(B, mod, mod=False, elem_type=elem_type)
    return KaratsubaArray(A, B, N1, N2, M)


def KaratsubaVector(x, y, N1=None, N2=None, M=None, elem_type=torch.float64):
    """KaratsubaVector(A, B[, N1, N2, M]) (KaratsubaMatrix.jl:73-79)."""
    if not isinstance(x, CuModArray):
        mod = N1 if N1 is not None else 2 ** 52
        x = cumod.CuModVector(x, mod, mod=False, elem_type=elem_type)
        y = cumod.CuModVector(y, mod, mod=False, elem_type=elem_type)
    return KaratsubaArray(x, y, N1, N2, M)


def KaratsubaZeros(dtype, rows, cols_or_N1, *rest):
    """KaratsubaZeros(T, rows, cols, N1, N2, M, use_gpu) / KaratsubaZeros(T, length, N1, N2, M, use_gpu)
    (KaratsubaMatrix.jl:404-420).  Only device storage exists here."""
    if len(rest) == 4:
        cols, (N1, N2, M, _use_gpu) = cols_or_N1, rest
        return KaratsubaArray(cumod.zeros(dtype, rows, cols, N1), cumod.zeros(dtype, rows, cols, N1), N1, N2, M)
    N1, (N2, M, _use_gpu) = cols_or_N1, rest
    return KaratsubaArray(cumod.zeros(dtype, rows, N1), cumod.zeros(dtype, rows, N1), N1, N2, M)


def initialize_plan_(K):
    """initialize_plan!(K) (KaratsubaMatrix.jl:422-424)."""
    K.plan = _zeros_like_digits(K.data1, K.N1)
    return K.plan


def _check_f64(*Ks):
    for K in Ks:
        if K.data1.dtype != torch.float64 or K.data2.dtype != torch.float64:
            raise NotImplementedError("Not implemented for non-Float64 entries")


def _check_elementwise(K, *others):
    for X in others:
        if X.M != K.M:
            raise ValueError("Matrices must have the same modulus m")
        if X.data1.size != K.data1.size:
            raise ValueError("Matrix dimensions must match")
    _check_f64(K, *others)
    for X in (K,) + others:
        if X.data1.padded_len != K.data1.padded_len or X.data2.padded_len != K.data1.padded_len:
            raise ValueError("digit arrays must share one padded layout")


def add_(K, A, B):
    """add!(K, A, B) (KaratsubaMatrix.jl:505-536; karatsuba_add_kernel!, KaratsubaKernels.jl:2-50)."""
    _check_elementwise(K, A, B)
    if K.plan is None:
        raise ValueError("Must initialize plan first before using fallback implementation")
    call("gffm_karatsuba_add_f64", _ptr(K.data1.data), _ptr(K.data2.data), _ptr(A.data1.data), _ptr(A.data2.data),
         _ptr(B.data1.data), _ptr(B.data2.data), A.data1.padded_len, A.N1, A.N2, _stream())
    return K


def sub_(K, A, B):
    """sub!(K, A, B) (KaratsubaMatrix.jl:583-629; karatsuba_sub_kernel!, KaratsubaKernels.jl:113-125)."""
    _check_elementwise(K, A, B)
    call("gffm_karatsuba_sub_f64", _ptr(K.data1.data), _ptr(K.data2.data), _ptr(A.data1.data), _ptr(A.data2.data),
         _ptr(B.data1.data), _ptr(B.data2.data), A.data1.padded_len, A.N1, A.N2, _stream())
    return K


def negate_(K, A):
    """negate!(K, A) (KaratsubaMatrix.jl:691-731; karatsuba_negate_kernel!, KaratsubaKernels.jl:79-111)."""
    _check_elementwise(K, A)
    call("gffm_karatsuba_negate_f64", _ptr(K.data1.data), _ptr(K.data2.data), _ptr(A.data1.data),
         _ptr(A.data2.data), A.data1.padded_len, A.N1, A.N2, _stream())
    return K


def scalar_multiply_(B, A, s):
    """scalar_multiply!(B, A, s) (KaratsubaMatrix.jl:631-666; KaratsubaKernels.jl:52-77)."""
    _check_elementwise(B, A)
    call("gffm_karatsuba_scalar_mul_f64", _ptr(B.data1.data), _ptr(B.data2.data), _ptr(A.data1.data),
         _ptr(A.data2.data), int(s), A.data1.padded_len, A.N1, A.N2, _stream())
    return B


def KMatMul_(C, A, B):
    """KMatMul!(C, A, B) (KaratsubaMatrix.jl:133-204): C = A*B in Z/(N1*N2); B may be a KaratsubaVector."""
    if A.M != B.M or A.M != C.M:
        raise ValueError("Matrices must have the same modulus m")
    if A.data1.cols() != B.data1.rows():
        raise ValueError("Matrix dimensions don't work for multiplication")
    if A.plan is None or B.plan is None or C.plan is None:
        raise ValueError("Must initialize plans first")
    _check_f64(A, B, C)
    m, k = A.data1.rows(), A.data1.cols()
    n = B.data1.cols()
    if C.data1.rows() != m or C.data1.cols() != n:
        raise ValueError("Output matrix C has incorrect dimensions")
    if A.data2.ld != A.data1.ld or B.data2.ld != B.data1.ld or C.data2.ld != C.data1.ld:
        raise ValueError("digit arrays must share one leading dimension")
    call("gffm_karatsuba_matmul_f64", m, n, k, _ptr(A.data1.data), _ptr(A.data2.data), A.data1.ld,
         _ptr(B.data1.data), _ptr(B.data2.data), B.data1.ld, _ptr(C.data1.data), _ptr(C.data2.data), C.data1.ld,
         A.N1, A.N2, None, 0, _stream())
    return C


def KMatMul_gemv_(C, A, B):
    """KMatMul_gemv!(C, A, B) (KaratsubaMatrix.jl:238-300): the matrix-vector product."""
    return KMatMul_(C, A, B)


def poly_karatsuba_matmul(A0, A1, B0, B1, p=None):
    """(A0 + A1 x)(B0 + B1 x) mod p -> (C0, C1, C2), three limb products
    (C1 = (A0 + A1)(B0 + B1) - C0 - C2 fused into the last one)."""
    p = int(p if p is not None else A0.N)
    for X in (A1, B0, B1):
        if X.dtype != A0.dtype:
            raise TypeError("mismatched element types")
    if A0.dtype != torch.float64:
        raise NotImplementedError("Not implemented for non-Float64 entries")
    if A0.size != A1.size or B0.size != B1.size:
        raise ValueError("Dimensions of matrices must match")
    if A0.ld != A1.ld or B0.ld != B1.ld:
        raise ValueError("components must share one leading dimension")
    m, k = A0.rows(), A0.cols()
    n = B0.cols()
    if B0.rows() != k:
        raise ValueError("Matrix dimensions don't work for multiplication")
    C = [cumod.zeros(A0.dtype, m, n, p) for _ in range(3)]
    call("gffm_karatsuba_poly_matmul_f64", m, n, k, _ptr(A0.data), _ptr(A1.data), A0.ld, _ptr(B0.data),
         _ptr(B1.data), B0.ld, _ptr(C[0].data), _ptr(C[1].data), _ptr(C[2].data), C[0].ld, p, None, 0, _stream())
    return tuple(C)


def MatToKMat(A, M=None, dtype=None):
    """MatToKMat(A[, M]) / MatToKMat(T, A, M) (KaratsubaMatrix.jl:358-402): digits of A in base N1 = N2 = M."""
    if M is None:
        M = find_max_ops(A.dtype, max(A.size))
    return KaratsubaMatrix_from(A, M, M, M)


def KaratsubaMatrix_from(A, N1, N2, M):
    """KaratsubaMatrix(T, A, N1, N2, M) (KaratsubaMatrix.jl:372-397): d1 = a mod N1, d2 = div(a, N1) mod N2."""
    if A.dtype != torch.float64:
        raise NotImplementedError("Not implemented for non-Float64 entries")
    K = KaratsubaArray(_zeros_like_digits(A, N1), _zeros_like_digits(A, N1), N1, N2, M)
    call("gffm_karatsuba_from_values_f64", _ptr(K.data1.data), _ptr(K.data2.data), _ptr(A.data), A.padded_len,
         int(N1), int(N2), _stream())
    return K


def KMatToMat(K, dtype=torch.float64):
    """KMatToMat(T, K) (KaratsubaMatrix.jl:352-356): the values d1 + N1*d2 as a CuModArray mod N1*N2.

    The reference evaluates K.data1 + K.N1*K.data2 with CuModArray arithmetic
    modulo data2's modulus N1, which drops the second digit; this returns the
    value the expression denotes."""
    if dtype != torch.float64:
        raise NotImplementedError("Not implemented for non-Float64 entries")
    R = _zeros_like_digits(K.data1, K.N1 * K.N2)
    call("gffm_karatsuba_to_values_f64", _ptr(R.data), _ptr(K.data1.data), _ptr(K.data2.data), K.data1.padded_len,
         K.N1, K.N2, _stream())
    return R


def zero_(K):
    """zero!(K) (KaratsubaMatrix.jl:347-350)."""
    cumod.zero_(K.data1)
    cumod.zero_(K.data2)
    return K


def copy_(B, A):
    """copy!(B, A) (KaratsubaMatrix.jl:338-345)."""
    cumod.copy_(B.data1, A.data1)
    cumod.copy_(B.data2, A.data2)
    if A.plan is not None and B.plan is None:
        initialize_plan_(B)
    return B


def divide_elements_(B, A, N):
    """divide_elements!(B, A, N) (KaratsubaMatrix.jl:733-736): B.data = div.(A.data, N),
    truncating integer division over the padded data; returns A, as the reference does."""
    call("gffm_trunc_div_%s" % cumod._sfx(B.dtype), _ptr(B.data), _ptr(A.data), A.padded_len, int(N), _stream())
    return A


def Karatsubacopy(A):
    """Karatsubacopy(A) (KaratsubaMatrix.jl:738-744)."""
    B = KaratsubaArray(cumod.copy(A.data1), cumod.copy(A.data2), A.N1, A.N2, A.N1 * A.N2)
    if A.plan is not None:
        initialize_plan_(B)
    return B


def workspace_size(m, n, k, N1, N2):
    out = ctypes.c_size_t(0)
    call("gffm_karatsuba_workspace_size", m, n, k, int(N1), int(N2), ctypes.byref(out))
    return out.value
