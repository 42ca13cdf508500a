"""CPU oracle for GPUFiniteFieldMatrices.jl's hot path -- TEST INFRASTRUCTURE ONLY.

This package wraps ``gffm_oracle.c`` (an exact integer restatement of the
reference's algorithms; each C routine cites the reference function it
follows) with numpy/ctypes.  Only ``tests/``, ``__graft_entry__.smoke()`` and
the CPU-baseline / reference arm of ``bench.py`` may import it, and only as
the checker or the timed CPU baseline.  The product library never calls it.

All matrices are numpy int64 arrays holding residues; they are passed to C in
column-major (Fortran) order, matching CuModArray.data in the reference.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "gffm_oracle.c")
_LIB_PATH = os.path.join(_HERE, "liboracle.so")
_lib = None

_i64 = ctypes.c_int64
_p = ctypes.c_void_p


def build(force=False):
    """Compile the oracle with gcc (portable flags: runs on x86-64 and aarch64)."""
    if (not force and os.path.exists(_LIB_PATH)
            and os.path.getmtime(_LIB_PATH) >= os.path.getmtime(_SRC)):
        return _LIB_PATH
    tmp = _LIB_PATH + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-std=gnu11", _SRC, "-o", tmp]
    subprocess.check_call(cmd)
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        L.or_mod_inv.restype = _i64
        L.or_mod_inv.argtypes = [_i64, _i64]
        L.or_find_max_stripe_ops.restype = _i64
        L.or_find_max_stripe_ops.argtypes = [ctypes.c_int, _i64]
        L.or_matmul.restype = None
        L.or_matmul.argtypes = [_i64, _i64, _i64, _p, _i64, _p, _i64, _p, _i64, _i64, ctypes.c_int]
        L.or_pluq.restype = ctypes.c_int
        L.or_pluq.argtypes = [_i64, _i64, _p, _i64, _p, _i64, _i64, _i64, _p, _p, _p, _p, _p]
        L.or_lu.restype = ctypes.c_int
        L.or_lu.argtypes = [_i64, _i64, _p, _i64, _p, _i64, _i64, _p, _p]
        L.or_rref.restype = ctypes.c_int
        L.or_rref.argtypes = [_i64, _i64, _p, _i64, _i64, _p, _p]
        L.or_karatsuba_matmul.restype = None
        L.or_karatsuba_matmul.argtypes = [_i64, _i64, _i64, _p, _p, _i64, _p, _p, _i64, _p, _p, _i64,
                                          _i64, _i64, ctypes.c_int]
        L.or_karatsuba_addsub.restype = None
        L.or_karatsuba_addsub.argtypes = [_i64, _p, _p, _p, _p, _p, _p, _i64, _i64, ctypes.c_int]
        L.or_karatsuba_scale.restype = None
        L.or_karatsuba_scale.argtypes = [_i64, _p, _p, _i64, ctypes.c_int, _p, _p, _i64, _i64]
        L.or_tri_window.restype = None
        L.or_tri_window.argtypes = [ctypes.c_int, _i64, _i64, _p, _i64, _i64, _i64, _i64, _p]
        L.or_tri_inverse.restype = ctypes.c_int
        L.or_tri_inverse.argtypes = [ctypes.c_int, _i64, _i64, _p, _i64, _i64, _p]
        _lib = L
    return _lib


def _f(a):
    return np.asfortranarray(np.asarray(a, dtype=np.int64))


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def mod_inv(p, N):
    """mod_inv (src/CuModMatrix/rref_lu_pluq/pluq_kernels.jl:11-31)."""
    return int(lib().or_mod_inv(int(p), int(N)))


def find_max_stripe_ops(bits, N):
    """find_max_stripe_ops (src/CuModMatrix/kernel_mul/stripe_mul.jl:13-27)."""
    return int(lib().or_find_max_stripe_ops(int(bits), int(N)))


def matmul(A, B, N, threads=0):
    """Exact A*B mod N (stripe_mul!, src/CuModMatrix/kernel_mul/stripe_mul.jl:175-244)."""
    A = _f(A)
    B = _f(B)
    m, k = A.shape
    k2, n = B.shape
    assert k == k2
    C = np.zeros((m, n), dtype=np.int64, order="F")
    lib().or_matmul(m, n, k, _ptr(A), max(m, 1), _ptr(B), max(k, 1), _ptr(C), max(m, 1), int(N), int(threads))
    return C


def pluq(A, N, l_cols=None):
    """Restated pluq_gpu_kernel (src/CuModMatrix/rref_lu_pluq/pluq_kernels.jl:46-157).

    Returns (U, L, row_swaps, col_swaps, rank).  U is m x n, L is m x l_cols
    (l_cols = m + 32 is the reference's padded width; only the first m columns
    are part of L's logical size).  Swap stacks are lists of 1-based tuples.
    """
    U = _f(A).copy(order="F")
    m, n = U.shape
    if l_cols is None:
        l_cols = m + 32
    L = np.zeros((m, l_cols), dtype=np.int64, order="F")
    rs = np.zeros((max(m, 1), 2), dtype=np.int64)
    cs = np.zeros((max(n, 1), 2), dtype=np.int64)
    nr = ctypes.c_int64(0)
    nc = ctypes.c_int64(0)
    rk = ctypes.c_int64(0)
    st = lib().or_pluq(m, n, _ptr(U), max(m, 1), _ptr(L), max(m, 1), l_cols, int(N), _ptr(rs),
                       ctypes.byref(nr), _ptr(cs), ctypes.byref(nc), ctypes.byref(rk))
    if st != 0:
        raise IndexError("pluq: the reference would index L out of bounds (status %d)" % st)
    rows = [tuple(int(v) for v in rs[i]) for i in range(nr.value)]
    cols = [tuple(int(v) for v in cs[i]) for i in range(nc.value)]
    return U, L, rows, cols, rk.value


def lu(A, N):
    """lu_gpu_type semantics (no column swaps): returns (U, L (m x m), perm (1-based), rank)."""
    U = _f(A).copy(order="F")
    m, n = U.shape
    L = np.zeros((m, m), dtype=np.int64, order="F")
    perm = np.zeros(max(m, 1), dtype=np.int64)
    rk = ctypes.c_int64(0)
    lib().or_lu(m, n, _ptr(U), max(m, 1), _ptr(L), max(m, 1), int(N), _ptr(perm), ctypes.byref(rk))
    return U, L, [int(p) + 1 for p in perm[:m]], rk.value


def rref(A, N):
    """Canonical reduced row echelon form mod prime N; returns (R, rank, pivot_cols)."""
    R = _f(A).copy(order="F")
    m, n = R.shape
    rk = ctypes.c_int64(0)
    piv = np.zeros(max(min(m, n), 1), dtype=np.int64)
    lib().or_rref(m, n, _ptr(R), max(m, 1), int(N), ctypes.byref(rk), _ptr(piv))
    return R, rk.value, [int(c) for c in piv[:rk.value]]


def karatsuba_matmul(A1, A2, B1, B2, N1, N2, threads=0):
    """Digit-form product in Z/(N1*N2) (KMatMul!, src/KaratsubaMatrix/KaratsubaMatrix.jl:133-204)."""
    A1, A2, B1, B2 = _f(A1), _f(A2), _f(B1), _f(B2)
    m, k = A1.shape
    n = B1.shape[1]
    C1 = np.zeros((m, n), dtype=np.int64, order="F")
    C2 = np.zeros((m, n), dtype=np.int64, order="F")
    lib().or_karatsuba_matmul(m, n, k, _ptr(A1), _ptr(A2), max(m, 1), _ptr(B1), _ptr(B2), max(k, 1),
                              _ptr(C1), _ptr(C2), max(m, 1), int(N1), int(N2), int(threads))
    return C1, C2


def karatsuba_addsub(A1, A2, B1, B2, N1, N2, sub=False):
    """Digit-form (A +- B) mod N1*N2 (karatsuba_add_kernel!/karatsuba_sub_kernel!)."""
    A1, A2, B1, B2 = (np.ascontiguousarray(np.asarray(x, dtype=np.int64)) for x in (A1, A2, B1, B2))
    C1 = np.zeros_like(A1)
    C2 = np.zeros_like(A1)
    lib().or_karatsuba_addsub(A1.size, _ptr(A1), _ptr(A2), _ptr(B1), _ptr(B2), _ptr(C1), _ptr(C2),
                              int(N1), int(N2), 1 if sub else 0)
    return C1, C2


def karatsuba_scale(A1, A2, N1, N2, s=0, negate=False):
    """Digit-form (s*A) or (-A) mod N1*N2 (karatsuba_scalar_multiply_kernel!, karatsuba_negate_kernel!)."""
    A1, A2 = (np.ascontiguousarray(np.asarray(x, dtype=np.int64)) for x in (A1, A2))
    C1 = np.zeros_like(A1)
    C2 = np.zeros_like(A1)
    lib().or_karatsuba_scale(A1.size, _ptr(A1), _ptr(A2), int(s), 1 if negate else 0, _ptr(C1), _ptr(C2),
                             int(N1), int(N2))
    return C1, C2


def poly_karatsuba_matmul(A0, A1, B0, B1, p, threads=0):
    """(A0 + A1 x)(B0 + B1 x) mod p as (C0, C1, C2) -- the polynomial reading of a
    two-component Karatsuba product: C0 = A0B0, C2 = A1B1, C1 = A0B1 + A1B0."""
    C0 = matmul(A0, B0, p, threads)
    C2 = matmul(A1, B1, p, threads)
    C1 = (matmul(A0, B1, p, threads) + matmul(A1, B0, p, threads)) % p
    return C0, C1, C2


def apply_row_swaps(M, swaps, inverse=False):
    """apply_row_perm! / apply_row_inv_perm! (src/CuModMatrix/rref_lu_pluq/permutations.jl:73-89)."""
    M = np.array(M, copy=True)
    seq = list(reversed(swaps)) if inverse else list(swaps)
    for (i, j) in seq:
        M[[i - 1, j - 1], :] = M[[j - 1, i - 1], :]
    return M


def apply_col_swaps(M, swaps, inverse=False):
    """apply_col_perm! / apply_col_inv_perm! (src/CuModMatrix/rref_lu_pluq/permutations.jl:11-27)."""
    M = np.array(M, copy=True)
    seq = list(reversed(swaps)) if inverse else list(swaps)
    for (i, j) in seq:
        M[:, [i - 1, j - 1]] = M[:, [j - 1, i - 1]]
    return M


def tri_window(A, N, row_shift, col_shift, upper):
    """forward_sub_kernel_32 / backward_sub_kernel_32 (src/CuModMatrix/triangular/
    substitution_inplace.jl:6-35, 63-88): the 32 x 32 window inverse (exact)."""
    A = _f(A)
    m, n = A.shape
    W = np.zeros((32, 32), dtype=np.int64, order="F")
    lib().or_tri_window(1 if upper else 0, m, n, _ptr(A), max(m, 1), int(row_shift), int(col_shift), int(N), _ptr(W))
    return W


def tri_sub32(A, N, row_shift, col_shift, upper):
    """forward_sub_gpu_type_32 / backward_sub_gpu_type_32: the window inverse in the
    top-left of an (n x m) zero matrix."""
    m, n = np.asarray(A).shape
    X = np.zeros((n, m), dtype=np.int64)
    W = tri_window(A, N, row_shift, col_shift, upper)
    r, c = min(32, n), min(32, m)
    X[:r, :c] = W[:r, :c]
    return X


def tri_inverse(A, N, upper):
    """upper_triangular_inverse_no_copy / lower_triangular_inverse_no_copy
    (src/CuModMatrix/triangular/triangular_inverse_no_copy.jl:197-245, 450-477):
    returns (X (n x m), status); status 2 is the reference's InverseNotDefinedException."""
    A = _f(A)
    m, n = A.shape
    X = np.zeros((n, m), dtype=np.int64, order="F")
    st = lib().or_tri_inverse(1 if upper else 0, m, n, _ptr(A), max(m, 1), int(N), _ptr(X))
    return X, st
