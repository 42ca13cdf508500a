"""GPU parity tests of the elimination: PLUQ (U, L, both swap stacks, rank),
LU, RREF and the swap-stack permutations, bit-exact against the oracle's
restatement of pluq_gpu_kernel and the reference's known answers."""
import json
import os

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

HERE = os.path.dirname(os.path.abspath(__file__))
P26 = 67108859
P25 = 33554393


def as_int(M):
    return np.rint(M.Array()).astype(np.int64)


def status_ok(gffm):
    assert gffm.load_library().gffm_device_status(None) == 0


def make(kind, m, n, N, rng):
    if kind == "uniform":
        return rng.integers(0, N, size=(m, n))
    if kind.startswith("rank"):
        r = int(kind[4:])
        X = rng.integers(0, N, size=(m, r))
        Y = rng.integers(0, N, size=(r, n))
        return oracle.matmul(X, Y, N)
    if kind == "zero_cols":            # interior zero columns with a non-zero last column: the skip quirk
        A = rng.integers(0, N, size=(m, n))
        for c in range(1, n - 1, 3):
            A[:, c] = 0
        return A
    if kind == "lead_zero":
        A = rng.integers(0, N, size=(m, n))
        A[:, :min(5, n - 1)] = 0
        return A
    if kind == "ties":
        return rng.integers(0, 2, size=(m, n)) * (N - 1)
    if kind == "zeros":
        return np.zeros((m, n), dtype=np.int64)
    if kind == "tall_low":             # rows below the pivot are zero early
        A = np.triu(rng.integers(0, N, size=(m, n)))
        return A
    if kind == "wide_quirk":           # 32 leading zero columns: pivots land past L's row-swap width
        A = rng.integers(0, N, size=(m, n))
        A[:, :32] = 0
        return A
    raise ValueError(kind)


CASES = [
    ("uniform", 1, 1, 7), ("uniform", 5, 5, 7), ("uniform", 33, 20, 3), ("uniform", 64, 64, 65521),
    ("uniform", 65, 65, P26), ("uniform", 130, 129, 2080639), ("uniform", 200, 300, P25), ("uniform", 300, 100, 11),
    ("uniform", 257, 257, 2 ** 20), ("uniform", 100, 100, 1000), ("uniform", 90, 90, 255255),
    ("uniform", 20, 20, 2), ("uniform", 150, 150, 3),
    ("rank30", 96, 96, P26), ("rank70", 150, 140, 7), ("rank1", 40, 40, 5),
    ("zero_cols", 40, 40, 13), ("zero_cols", 100, 130, 65521), ("lead_zero", 70, 80, 7),
    ("ties", 70, 70, 3), ("ties", 130, 90, 11), ("zeros", 10, 12, 7), ("tall_low", 90, 90, P26),
    ("wide_quirk", 3, 40, 7), ("wide_quirk", 5, 45, 11), ("wide_quirk", 4, 38, 65521),
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: "%s-%dx%d-%d" % c)
def test_pluq_matches_oracle(gffm, case):
    kind, m, n, N = case
    rng = np.random.default_rng(m * 1000 + n + N % 997)
    A = make(kind, m, n, N, rng)
    Ag = gffm.CuModMatrix(A, N, elem_type=torch.float64)
    try:
        U0, L0, rs0, cs0, rk0 = oracle.pluq(A, N)
    except IndexError:
        # the reference indexes L past its padded width here (a BoundsError): so must we
        with pytest.raises(gffm.GFFMError) as ei:
            gffm.pluq_gpu_kernel(Ag)
        assert ei.value.status == 8
        status_ok(gffm)
        return
    U, L, rs, cs = gffm.pluq_gpu_kernel(Ag)
    assert rs == rs0 and cs == cs0
    assert np.array_equal(as_int(U), U0)
    Ld = np.rint(L.data.cpu().numpy().T).astype(np.int64)     # padded (m+32) x (m+32) data
    assert np.array_equal(Ld[:m, :m + 32], L0)
    assert (Ld[m:, :] == 0).all()
    status_ok(gffm)


# Sizes where the next panel factors beside the previous panel's trailing update
# (at least 1024 rows below the panel and more than one panel of columns left).
LOOKAHEAD = [("uniform", 1400, 1400, P26), ("uniform", 1500, 700, 65521), ("uniform", 1300, 2000, P25),
             ("rank1200", 1400, 1400, P26), ("zero_cols", 1300, 1350, 13), ("ties", 1200, 1200, 3)]


@pytest.mark.parametrize("case", LOOKAHEAD, ids=lambda c: "%s-%dx%d-%d" % c)
def test_pluq_lookahead_sizes_match_oracle(gffm, case):
    test_pluq_matches_oracle(gffm, case)


# Well over 512 rows below the first pivot: the cooperative left-looking panel
# (128 columns over several CTAs) -- zero-column stops inside a panel and at its
# start, a rank drop mid-panel, ties across CTAs, a narrow last panel.
MULTI_CTA = [("uniform", 1700, 1700, P26), ("rank200", 1800, 1800, P26), ("zero_cols", 1700, 1750, 13),
             ("ties", 1700, 1700, 3), ("uniform", 2500, 300, 65521), ("uniform", 1600, 2600, P25),
             ("lead_zero", 1700, 1720, 7), ("rank100", 2000, 400, 65521)]


@pytest.mark.parametrize("case", MULTI_CTA, ids=lambda c: "%s-%dx%d-%d" % c)
def test_pluq_multi_cta_panel_matches_oracle(gffm, case):
    test_pluq_matches_oracle(gffm, case)


def test_rref_multi_cta_panel_matches_oracle(gffm):
    rng = np.random.default_rng(77)
    A = make("rank1700", 1800, 1900, P26, rng)
    R, rank, piv = gffm.rref_gpu_type(gffm.CuModMatrix(A, P26, elem_type=torch.float64), return_pivots=True)
    R0, rank0, piv0 = oracle.rref(A, P26)
    assert rank == rank0 == 1700 and piv == [c + 1 for c in piv0]
    np.testing.assert_array_equal(as_int(R), R0)
    status_ok(gffm)


def test_rref_lookahead_size_matches_oracle(gffm):
    rng = np.random.default_rng(77)
    A = make("rank1100", 1300, 1400, P26, rng)
    R, rank, piv = gffm.rref_gpu_type(gffm.CuModMatrix(A, P26, elem_type=torch.float64), return_pivots=True)
    R0, rank0, piv0 = oracle.rref(A, P26)
    assert rank == rank0 == 1100 and piv == [c + 1 for c in piv0]
    assert np.array_equal(as_int(R), R0)
    status_ok(gffm)


def test_pluq_config2_rank900(gffm):
    """1024 x 1024 of rank 900 mod the largest prime below 2^26: (1024x900)(900x1024)."""
    rng = np.random.default_rng(900)
    X = rng.integers(0, P26, size=(1024, 900))
    Y = rng.integers(0, P26, size=(900, 1024))
    A = oracle.matmul(X, Y, P26)
    U0, L0, rs0, cs0, rk0 = oracle.pluq(A, P26)
    assert rk0 == 900 and cs0 == [(c, 1024) for c in range(901, 1025)]
    Ag = gffm.CuModMatrix(A, P26, elem_type=torch.float64)
    U, L, rs, cs = gffm.pluq_gpu_kernel(Ag)
    assert rs == rs0 and cs == cs0
    assert np.array_equal(as_int(U), U0)
    Ld = np.rint(L.data.cpu().numpy().T).astype(np.int64)
    assert np.array_equal(Ld[:1024, :1056], L0)
    # RREF of the same matrix
    R, rank, piv = gffm.rref_gpu_type(Ag, return_pivots=True)
    R0, rank0, piv0 = oracle.rref(A, P26)
    assert rank == rank0 == 900 and piv == [c + 1 for c in piv0]
    assert np.array_equal(as_int(R), R0)
    status_ok(gffm)


def test_pluq_float32_storage(gffm):
    rng = np.random.default_rng(32)
    N = 4093
    A = rng.integers(0, N, size=(80, 70))
    U0, L0, rs0, cs0, _ = oracle.pluq(A, N)
    U, L, rs, cs = gffm.pluq_gpu_kernel(gffm.CuModMatrix(A, N, elem_type=torch.float32))
    assert rs == rs0 and cs == cs0 and np.array_equal(as_int(U), U0)
    status_ok(gffm)


@pytest.mark.parametrize("case", [("uniform", 50, 50, 7), ("rank20", 60, 70, 11), ("zero_cols", 40, 45, 13),
                                  ("uniform", 150, 100, P26), ("lead_zero", 70, 70, 65521),
                                  ("zero_cols", 1700, 1650, 65521)],
                         ids=lambda c: "%s-%dx%d-%d" % c)
def test_lu_matches_oracle(gffm, case):
    kind, m, n, N = case
    A = make(kind, m, n, N, np.random.default_rng(m + n))
    U0, L0, perm0, rk0 = oracle.lu(A, N)
    U, L, perm = gffm.lu_gpu_type(gffm.CuModMatrix(A, N, elem_type=torch.float64))
    assert perm == perm0
    assert np.array_equal(as_int(U), U0)
    assert np.array_equal(as_int(L), L0)
    status_ok(gffm)


@pytest.mark.parametrize("case", [("uniform", 30, 30, 7), ("rank20", 60, 70, 11), ("zero_cols", 40, 45, 13),
                                  ("rank100", 200, 260, P26), ("uniform", 130, 70, 65521), ("zeros", 5, 6, 3),
                                  ("rank64", 64, 200, P25)],
                         ids=lambda c: "%s-%dx%d-%d" % c)
def test_rref_matches_oracle(gffm, case):
    kind, m, n, N = case
    A = make(kind, m, n, N, np.random.default_rng(m * n))
    R0, rk0, piv0 = oracle.rref(A, N)
    R, rk, piv = gffm.rref_gpu_type(gffm.CuModMatrix(A, N, elem_type=torch.float64), return_pivots=True)
    assert rk == rk0 and piv == [c + 1 for c in piv0]
    assert np.array_equal(as_int(R), R0)
    status_ok(gffm)


def inverse_from_gpu_pluq(gffm, A, N):
    """is_invertible_with_inverse (CuModMatrix.jl:356-422) from the GPU factors."""
    import pyref
    n = A.shape[0]
    U, L, rs, cs = gffm.pluq_gpu_kernel(gffm.CuModMatrix(A, N, elem_type=torch.float64))
    Uh = as_int(U)
    Lh = np.rint(L.data.cpu().numpy().T).astype(np.int64)[:n, :n]
    if np.linalg.matrix_rank(np.diag(np.diag(Uh)).astype(float)) < n:
        return None
    Uinv = np.array(pyref.inverse_mod(Uh.tolist(), N), dtype=np.int64)
    Linv = np.array(pyref.inverse_mod(Lh.tolist(), N), dtype=np.int64)
    Linv = oracle.apply_col_swaps(Linv, rs, inverse=True)
    Uinv = oracle.apply_row_swaps(Uinv, cs, inverse=True)
    return oracle.matmul(Uinv, Linv, N)


def test_kat_invertible_from_gpu_factors(gffm):
    with open(os.path.join(HERE, "golden", "reference_kat.json")) as f:
        cases = [c for c in json.load(f)["cases"] if c["op"] == "invertible"]
    for c in cases:
        A = np.array(c["A"]) % c["N"]
        inv = inverse_from_gpu_pluq(gffm, A, c["N"])
        assert (inv is not None) == c["expected_invertible"], c["src"]
        if inv is not None:
            assert oracle.matmul(A, inv, c["N"]).tolist() == c["expected_product_with_inverse"]
    status_ok(gffm)


def test_kat_permutations(gffm):
    with open(os.path.join(HERE, "golden", "reference_kat.json")) as f:
        cases = [c for c in json.load(f)["cases"] if c["op"] in ("col_perm", "row_perm")]
    for c in cases:
        A = gffm.CuModMatrix(c["A"], c["N"])
        swaps = [tuple(s) for s in c["swaps"]]
        if c["op"] == "col_perm":
            gffm.apply_col_perm_(swaps, A)
            assert as_int(A).tolist() == c["expected"]
            gffm.apply_col_inv_perm_(swaps, A)
        else:
            gffm.apply_row_perm_(swaps, A)
            assert as_int(A).tolist() == c["expected"]
            gffm.apply_row_inv_perm_(swaps, A)
        assert as_int(A).tolist() == c["A"]
    status_ok(gffm)


def test_permutations_long_stacks(gffm):
    rng = np.random.default_rng(17)
    m, n = 300, 5000
    A = rng.integers(0, 97, size=(m, n))
    rows = [(int(a), int(b)) for a, b in rng.integers(1, m + 1, size=(3000, 2))]
    cols = [(int(a), int(b)) for a, b in rng.integers(1, n + 1, size=(4500, 2))]
    G = gffm.CuModMatrix(A, 97)
    gffm.apply_row_perm_(rows, G)
    gffm.apply_col_perm_(cols, G)
    want = oracle.apply_col_swaps(oracle.apply_row_swaps(A, rows), cols)
    assert np.array_equal(as_int(G), want)
    status_ok(gffm)


def test_pluq_8192_reconstruction(gffm):
    """Full-rank 8192 x 8192 mod p26: rank, no column swaps, unit upper U, and
    Freivalds' check of L U = P A on two random vectors (exact on the host)."""
    n = 8192
    g = torch.Generator(device="cuda")
    g.manual_seed(8192)
    A = gffm.rand(torch.float64, n, n, P26, generator=g)
    U, L, rs, cs = gffm.pluq_gpu_kernel(A)
    assert cs == []
    Ah, Uh = as_int(A), as_int(U)
    Lh = np.rint(L.data.cpu().numpy().T).astype(np.int64)[:n, :n]
    assert (np.diag(Uh) == 1).all()
    rng = np.random.default_rng(1)
    for _ in range(2):
        x = rng.integers(0, P26, size=(n, 1))
        lhs = oracle.matmul(Lh, oracle.matmul(Uh, x, P26), P26)
        rhs = oracle.apply_row_swaps(oracle.matmul(Ah, x, P26), rs)
        assert np.array_equal(lhs, rhs)
    # the rows of L above the diagonal and U below it are zero (sampled)
    idx = rng.integers(0, n, size=64)
    for i in idx:
        assert (Uh[i, :i] == 0).all() and (Lh[i, i + 1:] == 0).all()
    status_ok(gffm)


# ---- inverse / is_invertible / is_invertible_with_inverse (CuModMatrix.jl:335-502) ----
def test_kat_inverse(gffm):
    """The reference's known answers: de Rham 10 x 10 mod 7, the 6 x 6 identity mod 11, a singular 3 x 3."""
    with open(os.path.join(HERE, "golden", "reference_kat.json")) as f:
        cases = [c for c in json.load(f)["cases"] if c["op"] == "invertible"]
    for c in cases:
        A = gffm.CuModMatrix(np.array(c["A"]) % c["N"], c["N"], elem_type=torch.float64)
        ok, Ainv = gffm.is_invertible_with_inverse(A)
        assert ok == c["expected_invertible"], c["src"]
        assert gffm.is_invertible(A) == c["expected_invertible"]
        if ok:
            prod = oracle.matmul(np.array(c["A"]) % c["N"], as_int(Ainv), c["N"])
            assert prod.tolist() == c["expected_product_with_inverse"]
        else:
            with pytest.raises(gffm.MatrixNotInvertibleException):
                gffm.inverse(A)
    status_ok(gffm)


@pytest.mark.parametrize("n,N", [(1, 7), (5, 7), (64, 65521), (130, 1000003), (300, P26), (1024, P25)])
def test_inverse_random(gffm, n, N):
    import pyref
    rng = np.random.default_rng(n + N % 1000)
    A = rng.integers(0, N, size=(n, n))
    while n <= 64 and pyref.inverse_mod(A.tolist(), N) is None:      # small fields: draw an invertible one
        A = rng.integers(0, N, size=(n, n))
    Ag = gffm.CuModMatrix(A, N, elem_type=torch.float64)
    Ainv = gffm.inverse(Ag)
    Ah = as_int(Ainv)
    x = rng.integers(0, N, size=(n, 2))
    assert np.array_equal(oracle.matmul(A, oracle.matmul(Ah, x, N), N), x)   # A A^-1 x = x
    if n <= 64:
        assert Ah.tolist() == pyref.inverse_mod(A.tolist(), N)
    # the negative power goes through the same inverse (CuModMatrix.jl:307-329)
    if n <= 130:
        assert np.array_equal(as_int(Ag ** -1), Ah)
    status_ok(gffm)


@pytest.mark.parametrize("kind,n,N", [("rank30", 40, 13), ("zeros", 5, 7), ("rank1", 64, P26)])
def test_inverse_singular(gffm, kind, n, N):
    A = make(kind, n, n, N, np.random.default_rng(n))
    Ag = gffm.CuModMatrix(A, N, elem_type=torch.float64)
    assert gffm.is_invertible_with_inverse(Ag) == (False, None)
    assert not gffm.is_invertible(Ag)
    with pytest.raises(gffm.MatrixNotInvertibleException):
        gffm.inverse(Ag)
    status_ok(gffm)


def test_rref_and_inverse_need_a_prime(gffm):
    """Over a composite modulus the echelon form and the inverse are not defined: the
    reference's CuModMatrixModulusNotPrimeException, raised before any launch."""
    A = gffm.CuModMatrix(np.eye(4, dtype=np.int64), 2080639, elem_type=torch.float64)   # 11 * 189149
    with pytest.raises(gffm.CuModMatrixModulusNotPrimeException):
        gffm.rref_gpu_type(A)
    with pytest.raises(gffm.CuModMatrixModulusNotPrimeException):
        gffm.inverse(A)
    status_ok(gffm)


def test_pluq_taller_than_the_cooperative_panel(gffm):
    """More rows than the cooperative panel keeps in shared memory (min(SMs, 160) * 288):
    the first panels factor as 32-column tall panels in global memory, exact against the
    oracle -- a 50,000 x 64 matrix, and one row over the capacity."""
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    cap = min(sms, 160) * 288
    rng = np.random.default_rng(50000)
    for (m, n, N, kind) in [(50000, 64, P26, "uniform"), (cap + 1, 40, 65521, "ties"), (50000, 70, 13, "zero_cols")]:
        A = make(kind, m, n, N, rng)
        U0, L0, rs0, cs0, rk0 = oracle.pluq(A, N, l_cols=n + 32)
        U, L, rs, cs = gffm.pluq_gpu_kernel(gffm.CuModMatrix(A, N, elem_type=torch.float64))
        assert rs == rs0 and cs == cs0
        assert np.array_equal(np.rint(U.data[:n, :m].cpu().numpy().T).astype(np.int64), U0)
        # L is the reference's (m+32) x (m+32): its first n + 32 columns hold every non-zero
        # (the oracle's L is truncated there; its swap width is capped the same way)
        Ld = L.data[:n + 32, :m].cpu().numpy().T
        assert np.array_equal(np.rint(Ld).astype(np.int64), L0)
        assert not bool(L.data[n + 32:, :].any()) and not bool(L.data[:, m:].any())
        status_ok(gffm)
    # RREF (zero columns skipped, not swapped) through the same tall panels
    A = make("rank50", 46000, 60, P26, rng)
    R0, rank0, piv0 = oracle.rref(A, P26)
    R, rank, piv = gffm.rref_gpu_type(gffm.CuModMatrix(A, P26, elem_type=torch.float64), return_pivots=True)
    assert rank == rank0 == 50 and piv == [c + 1 for c in piv0]
    assert np.array_equal(as_int(R), R0)
    status_ok(gffm)
