"""Exact host-side checks of large outputs -- TEST INFRASTRUCTURE ONLY.

Used by ``tests/`` and by ``bench.py`` after its timed regions, never by the
product library.  Every check is exact arithmetic mod N on the host (the
oracle's matmul), so a passing check is a proof up to Freivalds' error
probability (at most 1/N per random vector for a wrong result).

* ``freivalds_product``: C == A*B mod N, tested as C x == A (B x).
* ``freivalds_pluq``: L U == P A mod N for a factorization without column
  swaps, tested as L (U x) == P (A x), P the row swap stack applied in order
  (apply_row_perm!, src/CuModMatrix/rref_lu_pluq/permutations.jl:73-80).
* ``pluq_leading_block``: the first ``width`` pivot steps of
  pluq_gpu_kernel (src/CuModMatrix/rref_lu_pluq/pluq_kernels.jl:82-141)
  depend only on the first ``width`` columns, so the oracle's factorization
  of that column block fixes the first row swaps, U's leading square and L's
  first columns (after the later row swaps, which move whole rows of L
  inside its swap width).
"""
import numpy as np

from . import apply_row_swaps, matmul, pluq


def freivalds_product(A, B, C, N, rng, vectors=2):
    """C == A*B mod N for int64 residue arrays, by Freivalds' test."""
    A, B, C = (np.asarray(x, dtype=np.int64) for x in (A, B, C))
    if A.shape[1] == 0:
        return bool((C == 0).all())
    for _ in range(vectors):
        x = rng.integers(0, N, size=(B.shape[1], 1))
        if not np.array_equal(matmul(C, x, N), matmul(A, matmul(B, x, N), N)):
            return False
    return True


def freivalds_pluq(A, U, L, row_swaps, N, rng, vectors=2):
    """L U == P A mod N (no column swaps) for int64 residue arrays: L is m x m, U m x n."""
    A, U, L = (np.asarray(x, dtype=np.int64) for x in (A, U, L))
    for _ in range(vectors):
        x = rng.integers(0, N, size=(A.shape[1], 1))
        lhs = matmul(L, matmul(U, x, N), N)
        rhs = apply_row_swaps(matmul(A, x, N), row_swaps)
        if not np.array_equal(lhs, rhs):
            return False
    return True


def pluq_leading_block(A_block, U, L_first, row_swaps, N):
    """Compare a factorization's first ``w`` pivot steps with the oracle's factorization
    of the leading m x w column block ``A_block`` (full column rank expected).

    ``U`` is the factorization's leading w x w block of U, ``L_first`` the first w
    columns of L (m x w), ``row_swaps`` its whole row swap stack.  Returns a dict of
    booleans, one per compared part."""
    A_block = np.asarray(A_block, dtype=np.int64)
    m, w = A_block.shape
    U0, L0, rs0, cs0, rk0 = pluq(A_block, N)
    early = [s for s in row_swaps if s[0] <= w]
    late = [s for s in row_swaps if s[0] > w]
    L0w = apply_row_swaps(L0[:, :w], late)
    return {
        "block_full_rank": rk0 == w and cs0 == [],
        "row_swaps": early == rs0,
        "U_block": bool(np.array_equal(np.asarray(U, dtype=np.int64), U0[:w, :w])),
        "L_columns": bool(np.array_equal(np.asarray(L_first, dtype=np.int64), L0w)),
    }
