"""The host checks that the config-size tests and the bench run on large outputs
(oracle/checks.py) accept correct results and reject results with one planted
mistake.  Everything runs on the CPU; the mistakes are planted in the oracle's own
results."""
import numpy as np

import oracle
from oracle import checks

P = 65521


def test_freivalds_product_accepts_and_rejects():
    rng = np.random.default_rng(1)
    A, B = rng.integers(0, P, size=(40, 30)), rng.integers(0, P, size=(30, 20))
    C = oracle.matmul(A, B, P)
    assert checks.freivalds_product(A, B, C, P, np.random.default_rng(2))
    for i, j in ((0, 0), (39, 19), (17, 5)):
        bad = C.copy()
        bad[i, j] = (bad[i, j] + 1) % P
        assert not checks.freivalds_product(A, B, bad, P, np.random.default_rng(2))
    z = np.zeros
    assert checks.freivalds_product(z((3, 0), np.int64), z((0, 4), np.int64), z((3, 4), np.int64), P, rng)
    assert not checks.freivalds_product(z((3, 0), np.int64), z((0, 4), np.int64), np.ones((3, 4), np.int64), P, rng)


def test_freivalds_pluq_accepts_and_rejects():
    rng = np.random.default_rng(3)
    m = 48
    A = rng.integers(0, P, size=(m, m))
    U, L, rs, cs, rank = oracle.pluq(A, P)
    assert cs == [] and rank == m and len(rs) > 0
    Lm = L[:, :m]
    assert checks.freivalds_pluq(A, U, Lm, rs, P, np.random.default_rng(4))
    bad_u = U.copy()
    bad_u[3, 10] = (bad_u[3, 10] + 1) % P
    assert not checks.freivalds_pluq(A, bad_u, Lm, rs, P, np.random.default_rng(4))
    bad_l = Lm.copy()
    bad_l[20, 5] = (bad_l[20, 5] + 7) % P
    assert not checks.freivalds_pluq(A, U, bad_l, rs, P, np.random.default_rng(4))
    assert not checks.freivalds_pluq(A, U, Lm, rs[1:], P, np.random.default_rng(4))   # a row swap dropped


def test_pluq_leading_block_matches_the_full_factorization():
    """The first w pivot steps of a factorization depend only on the first w columns:
    the oracle's factorization of the whole matrix agrees with its factorization of the
    leading column block, and a planted change in U or in the swap stack is caught."""
    rng = np.random.default_rng(5)
    m, n, w = 64, 80, 16
    A = rng.integers(0, P, size=(m, n))
    U, L, rs, cs, rank = oracle.pluq(A, P)
    got = checks.pluq_leading_block(A[:, :w], U[:w, :w], L[:, :w], rs, P)
    assert all(got.values()), got
    bad_u = U[:w, :w].copy()
    bad_u[2, 7] = (bad_u[2, 7] + 1) % P
    assert not checks.pluq_leading_block(A[:, :w], bad_u, L[:, :w], rs, P)["U_block"]
    early = [s for s in rs if s[0] <= w]
    assert early, "the leading block has row swaps"
    dropped = [s for s in rs if s != early[0]]
    assert not checks.pluq_leading_block(A[:, :w], U[:w, :w], L[:, :w], dropped, P)["row_swaps"]
