"""PLUQ / LU / RREF and swap-stack permutations over libgffm.

Mirrors src/CuModMatrix/rref_lu_pluq/pluq_kernels.jl (pluq_gpu_kernel),
src/CuModMatrix/rref_lu_pluq/permutations.jl and the intended rref_gpu_type /
lu_gpu_type API of test/Experiments/rref_gpu_type.jl.  Outputs keep the
reference's layout: U has A's padded data shape with size (rows, cols), L is
(rows+32) x (rows+32) with size (rows, rows), swap stacks are lists of 1-based
(i, j) tuples.
"""
import ctypes

import numpy as np
import torch

from ._lib import GFFMError, call
from .cumod import CuModArray, CuModMatrixModulusNotPrimeException, TILE_WIDTH, _ptr, _sfx, _stream, zeros


def _call_prime(name, *args):
    """A call defined over prime fields: status 9 becomes CuModMatrixModulusNotPrimeException."""
    try:
        return call(name, *args)
    except GFFMError as e:
        if e.status == 9:
            raise CuModMatrixModulusNotPrimeException(str(e)) from None
        raise


def _swaps_buf(P):
    arr = np.ascontiguousarray(np.asarray(P, dtype=np.int64).reshape(-1, 2))
    return arr, arr.ctypes.data_as(ctypes.c_void_p), arr.shape[0]


def pluq_gpu_kernel(A, debug=False, method="limb"):
    """pluq_gpu_kernel(A) -> (U, L, Perm_rows, Perm_cols) (pluq_kernels.jl:46-157).

    method="plain" runs the trailing products on the reference's plain Float64
    arithmetic instead of the limb tensor-core GEMM (Float64 storage only)."""
    if method not in ("limb", "plain"):
        raise ValueError("method must be 'limb' or 'plain'")
    entry = "gffm_pluq_" + _sfx(A.dtype)
    if method == "plain":
        if A.dtype != torch.float64:
            raise TypeError("the plain form takes Float64 storage")
        entry = "gffm_pluq_plain_f64"
    rows, cols = A.data.shape[1] - TILE_WIDTH, A.data.shape[0] - TILE_WIDTH   # size(A.data) .- 32 (:82-84)
    U = CuModArray(torch.zeros_like(A.data), (rows, cols), A.N)
    L = CuModArray(torch.zeros((rows + TILE_WIDTH, rows + TILE_WIDTH), dtype=A.dtype, device=A.data.device),
                   (rows, rows), A.N)
    rs = np.zeros((max(rows, 1), 2), dtype=np.int64)
    cs = np.zeros((max(cols, 1), 2), dtype=np.int64)
    nr, nc, rk = ctypes.c_int64(0), ctypes.c_int64(0), ctypes.c_int64(0)
    call(entry, rows, cols, _ptr(A.data), A.ld, _ptr(U.data), U.ld, _ptr(L.data), L.ld,
         rows + TILE_WIDTH, A.N, rs.ctypes.data_as(ctypes.c_void_p), ctypes.byref(nr),
         cs.ctypes.data_as(ctypes.c_void_p), ctypes.byref(nc), ctypes.byref(rk), None, 0, _stream())
    Prows = [tuple(int(v) for v in rs[i]) for i in range(nr.value)]
    Pcols = [tuple(int(v) for v in cs[i]) for i in range(nc.value)]
    if debug:
        print("rank", rk.value, "Perm_rows", Prows, "Perm_cols", Pcols)
    return U, L, Prows, Pcols


def pluq_rank(A):
    """Rank found by the elimination (number of pivots)."""
    rows, cols = A.size
    U = CuModArray(torch.zeros_like(A.data), (rows, cols), A.N)
    L = CuModArray(torch.zeros((rows + TILE_WIDTH, rows + TILE_WIDTH), dtype=A.dtype, device=A.data.device),
                   (rows, rows), A.N)
    rs = np.zeros((max(rows, 1), 2), dtype=np.int64)
    cs = np.zeros((max(cols, 1), 2), dtype=np.int64)
    nr, nc, rk = ctypes.c_int64(0), ctypes.c_int64(0), ctypes.c_int64(0)
    call("gffm_pluq_" + _sfx(A.dtype), rows, cols, _ptr(A.data), A.ld, _ptr(U.data), U.ld, _ptr(L.data), L.ld,
         rows + TILE_WIDTH, A.N, rs.ctypes.data_as(ctypes.c_void_p), ctypes.byref(nr),
         cs.ctypes.data_as(ctypes.c_void_p), ctypes.byref(nc), ctypes.byref(rk), None, 0, _stream())
    return rk.value


def lu_gpu_type(A, mod_N=-1):
    """lu_gpu_type(A, mod_N) -> (U, L, Perm) (test/Experiments/rref_gpu_type.jl:60-103)."""
    N = mod_N if mod_N > 0 else A.N
    rows, cols = A.size
    U = CuModArray(torch.zeros_like(A.data), (rows, cols), N)
    L = zeros(A.dtype, rows, rows, N)
    perm = np.zeros(max(rows, 1), dtype=np.int64)
    rk = ctypes.c_int64(0)
    call("gffm_lu_" + _sfx(A.dtype), rows, cols, _ptr(A.data), A.ld, _ptr(U.data), U.ld, _ptr(L.data), L.ld, N,
         perm.ctypes.data_as(ctypes.c_void_p), ctypes.byref(rk), None, 0, _stream())
    return U, L, [int(p) for p in perm[:rows]]


def rref_gpu_type(A, mod_N=-1, return_pivots=False):
    """rref_gpu_type(A, mod_N) (test/Experiments/rref_gpu_type.jl:8-51): the reduced row echelon form."""
    N = mod_N if mod_N > 0 else A.N
    rows, cols = A.size
    R = CuModArray(torch.zeros_like(A.data), (rows, cols), N)
    piv = np.zeros(max(min(rows, cols), 1), dtype=np.int64)
    rk = ctypes.c_int64(0)
    _call_prime("gffm_rref_" + _sfx(A.dtype), rows, cols, _ptr(A.data), A.ld, _ptr(R.data), R.ld, N, ctypes.byref(rk),
         piv.ctypes.data_as(ctypes.c_void_p), None, 0, _stream())
    if return_pivots:
        return R, rk.value, [int(p) for p in piv[:rk.value]]
    return R


# -- inverse / invertibility (CuModMatrix.jl:335-502) ---------------------------
class MatrixNotInvertibleException(Exception):
    pass


def _inverse(A):
    from .cumod import CuModMatrixNotSquareException
    if A.ndim != 2 or A.rows() != A.cols():
        raise CuModMatrixNotSquareException("Matrix must be square to be inverted")
    n = A.rows()
    Ainv = zeros(A.dtype, n, n, A.N)
    ok = ctypes.c_int(0)
    _call_prime("gffm_inverse_" + _sfx(A.dtype), n, _ptr(A.data), A.ld, _ptr(Ainv.data), Ainv.ld, A.N,
                ctypes.byref(ok), None, 0, _stream())
    return bool(ok.value), Ainv


def is_invertible_with_inverse(A, debug=False):
    """is_invertible_with_inverse(A) -> (true, A^-1) or (false, None) (CuModMatrix.jl:356-422).

    Invertibility is decided by the elimination's exact pivot count (the reference
    computes a floating-point rank of U on the host)."""
    ok, Ainv = _inverse(A)
    return (True, Ainv) if ok else (False, None)


def is_invertible(A):
    """is_invertible(A) (CuModMatrix.jl:460-465): full rank mod N."""
    if A.ndim == 2 and A.rows() == A.cols():
        return _inverse(A)[0]
    return pluq_rank(A) == min(A.size)


def inverse(A):
    """inverse(A) (CuModMatrix.jl:480-502): A^-1 mod N, or MatrixNotInvertibleException."""
    ok, Ainv = _inverse(A)
    if not ok:
        raise MatrixNotInvertibleException("Matrix is not invertible mod %d" % A.N)
    return Ainv


# -- permutations.jl -----------------------------------------------------------
def _apply(P, A, rows, inverse):
    if len(P) == 0:
        return A
    arr, ptr, n = _swaps_buf(P)
    nrows, ncols = A.data.shape[1], A.data.shape[0]      # the padded data, as the reference's kernels index it
    name = ("gffm_apply_row_swaps_" if rows else "gffm_apply_col_swaps_") + _sfx(A.dtype)
    call(name, _ptr(A.data), A.ld, nrows, ncols, ptr, n, 1 if inverse else 0, _stream())
    torch.cuda.current_stream().synchronize()            # arr must outlive the launch
    return A


def apply_col_perm_(P, A):
    """apply_col_perm!(P, A): A <- A * P (permutations.jl:11-18)."""
    return _apply(P, A, rows=False, inverse=False)


def apply_col_inv_perm_(P, A):
    """apply_col_inv_perm!(P, A) (permutations.jl:20-27)."""
    return _apply(P, A, rows=False, inverse=True)


def apply_col_perm(P, A):
    """apply_col_perm(P, A): permuted copy (permutations.jl:29-37)."""
    return _apply(P, CuModArray(A.data.clone(), A.size, A.N), rows=False, inverse=False)


def apply_row_perm_(P, A):
    """apply_row_perm!(P, A) (permutations.jl:73-80)."""
    return _apply(P, A, rows=True, inverse=False)


def apply_row_inv_perm_(P, A):
    """apply_row_inv_perm!(P, A) (permutations.jl:82-89)."""
    return _apply(P, A, rows=True, inverse=True)


def apply_row_perm(P, A):
    """apply_row_perm(P, A): permuted copy (permutations.jl:91-100)."""
    return _apply(P, CuModArray(A.data.clone(), A.size, A.N), rows=True, inverse=False)


def perm_array_to_matrix(perm, N, new_size, perm_stack=False, elem_type=torch.float32):
    """perm_array_to_matrix(perm, N, new_size; perm_stack) (permutations.jl:141-157), built on the host."""
    from .cumod import CuModMatrix
    n = len(perm)
    if perm_stack:
        P = np.eye(n, dtype=np.int64)
        for (i, j) in perm:
            P[[i - 1, j - 1], :] = P[[j - 1, i - 1], :]
    else:
        P = np.zeros((n, n), dtype=np.int64)
        for i in range(n):
            P[perm[i] - 1, i] = 1
    return CuModMatrix(P, N, new_size=new_size, elem_type=elem_type)


# -- benchmark helper used by bench.py -----------------------------------------
def bench_pluq(size, stream_ptr, dev, reps=2, method="limb", warmup=1, outputs=False):
    """Time pluq on a full-rank size x size matrix mod 67108859 (seeded uniform residues)
    through the C ABI; returns a dict for the benchmark line.  method "plain" times the
    plain Float64 trailing products.  With outputs=True also returns the last run's
    (A, U, L, Perm_rows, Perm_cols) for checking."""
    import time
    p = 67108859
    if size is None or size < 0:
        size = 16384
    g = torch.Generator(device=dev)
    g.manual_seed(4321)
    from .cumod import rand
    A = rand(torch.float64, size, size, p, generator=g)
    U = CuModArray(torch.zeros_like(A.data), A.size, p)
    L = CuModArray(torch.zeros((size + 32, size + 32), dtype=torch.float64, device=A.data.device), (size, size), p)
    ws = ctypes.c_size_t(0)
    call("gffm_elim_workspace_size", size, size, size + 32, ctypes.byref(ws))
    buf = torch.empty(ws.value, dtype=torch.uint8, device=A.data.device)
    rs = np.zeros((size, 2), dtype=np.int64)
    cs = np.zeros((size, 2), dtype=np.int64)
    nr, nc, rk = ctypes.c_int64(0), ctypes.c_int64(0), ctypes.c_int64(0)

    entry = "gffm_pluq_f64" if method == "limb" else "gffm_pluq_plain_f64"

    def run():
        call(entry, size, size, _ptr(A.data), A.ld, _ptr(U.data), U.ld, _ptr(L.data), L.ld, size + 32, p,
             rs.ctypes.data_as(ctypes.c_void_p), ctypes.byref(nr), cs.ctypes.data_as(ctypes.c_void_p),
             ctypes.byref(nc), ctypes.byref(rk), ctypes.c_void_p(buf.data_ptr()), ws.value, stream_ptr)

    for _ in range(warmup):
        run()
    torch.cuda.synchronize()
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        run()
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    best = min(times)
    ops = 2.0 / 3.0 * size ** 3
    out = {"size": size, "modulus": p, "method": method, "seconds": round(best, 4), "rank": rk.value,
           "gops": round(ops / best / 1e9, 1), "ops": "2/3 n^3 modular multiply-adds"}
    if not outputs:
        return out
    Prows = [tuple(int(v) for v in rs[i]) for i in range(nr.value)]
    Pcols = [tuple(int(v) for v in cs[i]) for i in range(nc.value)]
    return out, (A, U, L, Prows, Pcols)
