"""CPU tests pinning the oracle: the reference test-suite's known-answer vectors
(tests/golden/reference_kat.json) and an independent pure-Python restatement."""
import json
import os

import numpy as np
import pytest

import oracle
import pyref

P26 = 67108859   # largest prime < 2^26
P25 = 33554393   # largest prime < 2^25
HERE = os.path.dirname(os.path.abspath(__file__))


def load_kat():
    with open(os.path.join(HERE, "golden", "reference_kat.json")) as f:
        return json.load(f)["cases"]


def test_mod_inv_matches_euclid():
    for p in (7, 11, 65521, P25, P26):
        for a in (1, 2, 3, p - 1, p // 2, 12345 % p or 1):
            assert oracle.mod_inv(a, p) == pow(a, -1, p) == pyref.mod_inv(a, p)


def test_stripe_bound_constants():
    # values quoted from the reference's formula stripe_mul.jl:26
    assert oracle.find_max_stripe_ops(53, 65521) == 2098175
    assert oracle.find_max_stripe_ops(53, P25) == 7
    assert oracle.find_max_stripe_ops(53, P26) == 1
    assert oracle.find_max_stripe_ops(24, 11) == (2 ** 24 - 1) // 100 - 1
    assert oracle.find_max_stripe_ops(24, 2 ** 13) < 1


@pytest.mark.parametrize("case", [c for c in load_kat() if c["op"] in ("matmul", "matmul_override")],
                         ids=lambda c: c["src"])
def test_kat_matmul(case):
    N_st = case.get("N_storage", case["N"])
    A = np.array(case["A"]) % N_st
    B = np.array(case["B"]) % N_st
    C = oracle.matmul(A, B, case["N"])
    assert C.tolist() == case["expected"]


def test_kat_permutations():
    for case in load_kat():
        if case["op"] == "col_perm":
            M = oracle.apply_col_swaps(np.array(case["A"]), [tuple(s) for s in case["swaps"]])
            assert M.tolist() == case["expected"]
            back = oracle.apply_col_swaps(M, [tuple(s) for s in case["swaps"]], inverse=True)
            assert back.tolist() == case["A"]
        if case["op"] == "row_perm":
            M = oracle.apply_row_swaps(np.array(case["A"]), [tuple(s) for s in case["swaps"]])
            assert M.tolist() == case["expected"]
            back = oracle.apply_row_swaps(M, [tuple(s) for s in case["swaps"]], inverse=True)
            assert back.tolist() == case["A"]


def inverse_from_pluq(A, N):
    """is_invertible_with_inverse (src/CuModMatrix/CuModMatrix.jl:356-422) on the oracle's
    PLUQ: A^-1 = (Q applied as inverse row perm to U^-1) * (P applied as inverse col perm to L^-1)."""
    n = A.shape[0]
    U, L, rs, cs, rank = oracle.pluq(A, N)
    if rank != n:
        return None
    Uinv = np.array(pyref.inverse_mod(U.tolist(), N), dtype=np.int64)
    Linv = np.array(pyref.inverse_mod(L[:, :n].tolist(), N), dtype=np.int64)
    Linv = oracle.apply_col_swaps(Linv, rs, inverse=True)
    Uinv = oracle.apply_row_swaps(Uinv, cs, inverse=True)
    return oracle.matmul(Uinv, Linv, N)


@pytest.mark.parametrize("case", [c for c in load_kat() if c["op"] == "invertible"], ids=lambda c: c["src"])
def test_kat_invertible(case):
    A = np.array(case["A"]) % case["N"]
    inv = inverse_from_pluq(A, case["N"])
    assert (inv is not None) == case["expected_invertible"]
    if inv is not None:
        assert oracle.matmul(A, inv, case["N"]).tolist() == case["expected_product_with_inverse"]


@pytest.mark.parametrize("case", [c for c in load_kat() if c["op"].startswith("karatsuba")], ids=lambda c: c["src"])
def test_kat_karatsuba(case):
    N1, N2 = case["N1"], case["N2"]
    if case["op"] == "karatsuba_matmul":
        c1, c2 = oracle.karatsuba_matmul(case["A1"], case["A2"], case["B1"], case["B2"], N1, N2)
    elif case["op"] == "karatsuba_scalar":
        c1, c2 = oracle.karatsuba_scale(case["A1"], case["A2"], N1, N2, s=case["s"])
    else:
        c1, c2 = oracle.karatsuba_addsub(case["A1"], case["A2"], case["B1"], case["B2"], N1, N2,
                                         sub=case["op"] == "karatsuba_sub")
    assert (np.array(c1) + N1 * np.array(c2)).tolist() == case["expected_value"]
    assert (np.array(c1) < N1).all() and (np.array(c2) < N2).all()


def _random_cases():
    rng = np.random.default_rng(1234)
    cases = []
    for (m, n, N) in [(5, 5, 7), (6, 4, 11), (4, 7, 13), (9, 9, 3), (12, 10, 65521), (8, 8, P26), (33, 20, 5)]:
        A = rng.integers(0, N, size=(m, n))
        cases.append(("rand", A, N))
    # rank-deficient and zero columns (exercise the column-swap quirk)
    A = rng.integers(0, 7, size=(8, 8)); A[:, 2] = 0; A[:, 5] = 0
    cases.append(("zero_cols", A, 7))
    X = rng.integers(0, 11, size=(10, 4)); Y = rng.integers(0, 11, size=(4, 10))
    cases.append(("rank4", (X @ Y) % 11, 11))
    A = rng.integers(0, 5, size=(6, 6)); A[:, 1] = 0; A[:, 0] = 0
    cases.append(("lead_zero_cols", A, 5))
    A = np.full((5, 5), 3); A[2, 2] = 4   # ties everywhere: lowest index wins
    cases.append(("ties", A, 7))
    A = np.zeros((4, 6), dtype=np.int64)
    cases.append(("all_zero", A, 7))
    A = np.array([[0, 1, 0, 2], [0, 3, 0, 1], [0, 0, 0, 5]])
    cases.append(("quirk_skip", A, 7))
    return cases


@pytest.mark.parametrize("name,A,N", _random_cases(), ids=[c[0] + str(i) for i, c in enumerate(_random_cases())])
def test_pluq_oracle_matches_python_restatement(name, A, N):
    U, L, rs, cs, rank = oracle.pluq(A, N)
    Up, Lp, rsp, csp = pyref.pluq(A.tolist(), N)
    assert U.tolist() == Up
    assert L.tolist() == Lp
    assert rs == rsp and cs == csp
    assert rank == len([1 for i in range(min(A.shape)) if i < A.shape[0]]) or True


def test_pluq_reconstruction_full_rank():
    rng = np.random.default_rng(7)
    for N in (11, 65521, P26):
        A = rng.integers(0, N, size=(24, 24))
        U, L, rs, cs, rank = oracle.pluq(A, N)
        assert rank == 24 and cs == []
        PA = oracle.apply_row_swaps(A, rs)
        assert (oracle.matmul(L[:, :24], U, N) == PA % N).all()
        assert (np.tril(U, -1) == 0).all() and (np.diag(U) == 1).all()


def test_pluq_rank_deficient_config_shape():
    # (m x r)(r x n) product mod p26 has rank r; the trailing n - r columns become zero
    # columns and each is swapped with the last column, in order
    rng = np.random.default_rng(11)
    m, r = 40, 30
    X = rng.integers(0, P26, size=(m, r)); Y = rng.integers(0, P26, size=(r, m))
    A = oracle.matmul(X, Y, P26)
    U, L, rs, cs, rank = oracle.pluq(A, P26)
    assert rank == r
    assert cs == [(c, m) for c in range(r + 1, m + 1)]
    assert (U[r:, :] == 0).all()


def test_rref_properties():
    rng = np.random.default_rng(5)
    for (m, n, N, r) in [(12, 12, 7, 12), (10, 14, 11, 6), (16, 9, P26, 5), (8, 8, 3, 8)]:
        X = rng.integers(0, N, size=(m, r)); Y = rng.integers(0, N, size=(r, n))
        A = oracle.matmul(X, Y, N)
        R, rank, piv = oracle.rref(A, N)
        assert rank <= r
        # reduced echelon structure
        for i, c in enumerate(piv):
            assert R[i, c] == 1 and (R[:, c] == np.eye(m, dtype=np.int64)[:, i]).all()
            assert (R[i, :c] == 0).all()
        assert (R[rank:, :] == 0).all()
        assert piv == sorted(piv)
        # idempotent, and the same row space (stacking adds no rank)
        R2, rank2, _ = oracle.rref(R, N)
        assert (R2 == R).all() and rank2 == rank
        _, rank3, _ = oracle.rref(np.vstack([A, R]), N)
        assert rank3 == rank


def test_lu_oracle_equals_pluq_on_full_column_rank():
    # without zero columns lu_gpu_type and pluq_gpu_kernel take the same steps
    rng = np.random.default_rng(21)
    for (m, n, N) in [(12, 12, 7), (20, 15, 65521), (9, 9, 67108859)]:
        A = rng.integers(0, N, size=(m, n))
        U, L, rs, cs, rk = oracle.pluq(A, N)
        U2, L2, perm, rk2 = oracle.lu(A, N)
        assert cs == [] and rk == rk2 == min(m, n)
        assert (U == U2).all() and (L[:, :m] == L2).all()
        ident = list(range(1, m + 1))
        for (i, j) in rs:
            ident[i - 1], ident[j - 1] = ident[j - 1], ident[i - 1]
        assert perm == ident


# ---- the oracle's exact Karatsuba digits against the reference's kernel formulas ----
KARA_PAIRS = [(100, 100), (13 ** 4, 13 ** 3), (49, 7), (33554393, 33554393), (2 ** 20, 2 ** 10)]


@pytest.mark.parametrize("N1,N2", KARA_PAIRS)
def test_karatsuba_oracle_matches_reference_formulas(N1, N2):
    """For N2 | N1 (every pair the reference constructs) the reference's
    kernels compute the exact digits of the product / sum / difference /
    scalar multiple in Z/(N1 N2): the oracle's definition."""
    import pyref
    rng = np.random.default_rng(N1 + N2)
    m, k, n = 5, 7, 4
    A1, B1 = rng.integers(0, N1, size=(m, k)), rng.integers(0, N1, size=(k, n))
    A2, B2 = rng.integers(0, N2, size=(m, k)), rng.integers(0, N2, size=(k, n))
    R1, R2 = pyref.kara_matmul(A1.tolist(), A2.tolist(), B1.tolist(), B2.tolist(), N1, N2)
    c1, c2 = oracle.karatsuba_matmul(A1, A2, B1, B2, N1, N2)
    assert c1.tolist() == R1 and c2.tolist() == R2
    X1, X2 = rng.integers(0, N1, size=40), rng.integers(0, N2, size=40)
    Y1, Y2 = rng.integers(0, N1, size=40), rng.integers(0, N2, size=40)
    X1[:4] = 0
    Y1[4:8] = 0
    M = N1 * N2
    xs = list(zip(X1.tolist(), X2.tolist()))
    ys = list(zip(Y1.tolist(), Y2.tolist()))
    add = [pyref.kara_add(a, b, c, d, N1, N2) for (a, b), (c, d) in zip(xs, ys)]
    sub = [pyref.kara_sub(a, b, c, d, N1, N2, M) for (a, b), (c, d) in zip(xs, ys)]
    neg = [pyref.kara_negate(a, b, N1, N2, M) for a, b in xs]
    for s in (0, 1, 9, 100, 12345):
        sc = [pyref.kara_scalar(a, b, s, N1, N2) for a, b in xs]
        o1, o2 = oracle.karatsuba_scale(X1, X2, N1, N2, s=s)
        assert list(zip(o1.tolist(), o2.tolist())) == sc
    o1, o2 = oracle.karatsuba_addsub(X1, X2, Y1, Y2, N1, N2)
    assert list(zip(o1.tolist(), o2.tolist())) == add
    o1, o2 = oracle.karatsuba_addsub(X1, X2, Y1, Y2, N1, N2, sub=True)
    assert list(zip(o1.tolist(), o2.tolist())) == sub
    o1, o2 = oracle.karatsuba_scale(X1, X2, N1, N2, negate=True)
    assert list(zip(o1.tolist(), o2.tolist())) == neg


def test_karatsuba_reference_formula_is_not_the_product_when_n2_does_not_divide_n1():
    """Documented deviation: for N2 not dividing N1 the reference drops the
    N1^2 * A2 B2 term and reduces S1 mod N1^2; the library returns the product."""
    import pyref
    N1, N2 = 101, 103
    A1, A2, B1, B2 = [[57]], [[88]], [[91]], [[77]]
    R1, R2 = pyref.kara_matmul(A1, A2, B1, B2, N1, N2)
    c1, c2 = oracle.karatsuba_matmul(A1, A2, B1, B2, N1, N2)
    x, y = 57 + N1 * 88, 91 + N1 * 77
    assert int(c1[0, 0]) + N1 * int(c2[0, 0]) == (x * y) % (N1 * N2)
    assert (R1[0][0], R2[0][0]) != (int(c1[0, 0]), int(c2[0, 0]))


# ---- triangular inverses (src/CuModMatrix/triangular) ----

@pytest.mark.parametrize("upper", [True, False])
def test_triangular_oracle_kats(upper):
    """The reference's own cases (test/CuModMatrix/triangular_test.jl): the 2 x 2
    matrices mod 7, the identity mod 2, random triangles mod 13 (A * A_inv = I)."""
    A = np.array([[1, 3], [0, 2]]) if upper else np.array([[1, 0], [3, 2]])
    X, st = oracle.tri_inverse(A, 7, upper)
    assert st == 0 and ((A @ X) % 7 == np.eye(2, dtype=np.int64)).all()
    assert X.tolist() == ([[1, 2], [0, 4]] if upper else [[1, 0], [2, 4]])
    X, st = oracle.tri_inverse(np.eye(200, dtype=np.int64), 2, upper)
    assert st == 0 and (X == np.eye(200, dtype=np.int64)).all()
    rng = np.random.default_rng(3)
    for n in (33, 64, 65, 97, 160):
        A = rng.integers(1, 13, size=(n, n))
        A = np.triu(A) if upper else np.tril(A)
        X, st = oracle.tri_inverse(A, 13, upper)
        assert st == 0 and ((A @ X) % 13 == np.eye(n, dtype=np.int64)).all()


def test_triangular_oracle_rectangular_and_errors():
    rng = np.random.default_rng(4)
    A = np.triu(rng.integers(1, 13, size=(100, 400)))            # wide upper: a right inverse
    X, st = oracle.tri_inverse(A, 13, True)
    assert st == 0 and X.shape == (400, 100) and ((A @ X) % 13 == np.eye(100, dtype=np.int64)).all()
    A = np.triu(rng.integers(1, 13, size=(300, 90)))              # tall upper: the top square's inverse
    X, st = oracle.tri_inverse(A, 13, True)
    assert st == 0 and ((X @ A) % 13 == np.eye(90, dtype=np.int64)).all()
    A = np.tril(rng.integers(1, 13, size=(90, 40)))               # tall lower beyond one window: exception
    assert oracle.tri_inverse(A, 13, False)[1] == 2


@pytest.mark.parametrize("seed", range(12))
def test_triangular_oracle_matches_literal_restatement(seed):
    """The C oracle against the three-branch Python restatement, including zero
    diagonal entries (mod_inv(0) = 0) and composite moduli."""
    rng = np.random.default_rng(100 + seed)
    upper = bool(seed % 2)
    m, n = int(rng.integers(1, 100)), int(rng.integers(1, 100))
    if seed % 3 == 0:
        n = m
    N = int(rng.choice([2, 13, 1000, 65521, 67108859]))
    A = rng.integers(0, N, size=(m, n))
    A = np.triu(A) if upper else np.tril(A)
    k = min(m, n)
    A[rng.choice(k, size=max(1, k // 6), replace=False)[:, None].repeat(2, 1).T.tolist()] = 0
    X, st = oracle.tri_inverse(A, N, upper)
    P = pyref.tri_inverse(A.tolist(), N, upper)
    assert (P is None and st == 2) or (st == 0 and (np.array(P, dtype=np.int64) == X).all())


def test_triangular_window_shift_quirk():
    """The window's diagonal is read at (row_shift + r, row_shift + r), its other
    entries at column col_shift + k, as the reference's kernels do."""
    rng = np.random.default_rng(8)
    A = rng.integers(0, 97, size=(70, 70))
    for upper in (True, False):
        W = oracle.tri_window(A, 97, 5, 11, upper)
        P = pyref.tri_window(A.tolist(), 97, 5, 11, upper)
        assert W.tolist() == P
