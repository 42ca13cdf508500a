"""GPU parity tests: triangular inverses and substitutions (src/CuModMatrix/
triangular), mod_inv, scalar division and truncating division, against the
oracle.  Bar: bit-exact equality on every output element."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
P26 = 67108859


def tri(rng, m, n, N, upper, zero_diag=0):
    A = rng.integers(0, N, size=(m, n))
    A = np.triu(A) if upper else np.tril(A)
    k = min(m, n)
    if zero_diag:
        idx = rng.choice(k, size=min(k, zero_diag), replace=False)
        A[idx, idx] = 0
    else:
        d = np.arange(k)
        A[d, d] = rng.integers(1, N, size=k)
    return A


def as_int(M):
    return np.rint(M.Array()).astype(np.int64)


@pytest.mark.parametrize("dtype", ["f64", "f32"])
@pytest.mark.parametrize("upper", [True, False])
@pytest.mark.parametrize("n,N", [(1, 7), (2, 7), (5, 13), (31, 97), (32, 13), (33, 65521), (64, P26), (65, 13),
                                 (96, 1000), (100, 65521), (200, P26), (257, 8388593)])
def test_square_inverse_matches_oracle(gffm, dtype, upper, n, N):
    if dtype == "f32" and N > (1 << 24):
        pytest.skip("Float32 storage holds residues below 2^24")
    rng = np.random.default_rng(n * 31 + N % 1000 + upper)
    A = tri(rng, n, n, N, upper)
    T = torch.float64 if dtype == "f64" else torch.float32
    Ag = gffm.CuModMatrix(A, N, elem_type=T)
    X = (gffm.upper_triangular_inverse_no_copy if upper else gffm.lower_triangular_inverse_no_copy)(Ag)
    want, st = oracle.tri_inverse(A, N, upper)
    assert st == 0 and X.size == (n, n)
    np.testing.assert_array_equal(as_int(X), want)
    if N in (7, 13, 97, 65521, P26, 8388593) and n <= 100:      # primes: a true inverse
        assert ((A.astype(object) @ want.astype(object)) % N == np.eye(n, dtype=object)).all()


@pytest.mark.parametrize("upper", [True, False])
@pytest.mark.parametrize("n,N", [(40, 13), (100, 1000), (150, P26)])
def test_singular_diagonal_matches_oracle(gffm, upper, n, N):
    """Zero diagonal entries: the reference's mod_inv(0) = 0 block result."""
    rng = np.random.default_rng(n + upper)
    A = tri(rng, n, n, N, upper, zero_diag=max(1, n // 7))
    X = (gffm.upper_triangular_inverse_no_copy if upper else gffm.lower_triangular_inverse_no_copy)(
        gffm.CuModMatrix(A, N, elem_type=torch.float64))
    np.testing.assert_array_equal(as_int(X), oracle.tri_inverse(A, N, upper)[0])


@pytest.mark.parametrize("upper,m,n", [(True, 100, 400), (True, 300, 90), (True, 20, 70), (True, 70, 20),
                                       (False, 90, 300), (False, 70, 20), (False, 20, 70)])
def test_rectangular_inverse_matches_oracle(gffm, upper, m, n):
    rng = np.random.default_rng(m * 3 + n)
    N = 65521
    A = tri(rng, m, n, N, upper)
    X = (gffm.upper_triangular_inverse_no_copy if upper else gffm.lower_triangular_inverse_no_copy)(
        gffm.CuModMatrix(A, N, elem_type=torch.float64))
    want, st = oracle.tri_inverse(A, N, upper)
    assert st == 0 and X.size == (n, m)
    np.testing.assert_array_equal(as_int(X), want)


def test_tall_lower_raises(gffm):
    A = np.tril(np.ones((90, 40), dtype=np.int64))
    with pytest.raises(gffm.InverseNotDefinedException):
        gffm.lower_triangular_inverse_no_copy(gffm.CuModMatrix(A, 13, elem_type=torch.float64))


@pytest.mark.parametrize("upper", [True, False])
@pytest.mark.parametrize("m,n,rs,cs", [(32, 32, 0, 0), (70, 70, 5, 11), (50, 80, 32, 32), (10, 40, 0, 0),
                                       (100, 100, 90, 90)])
def test_substitution_window_matches_oracle(gffm, upper, m, n, rs, cs):
    """forward_sub_gpu_type_32 / backward_sub_gpu_type_32, shifts included (the
    diagonal read at the row shift on both axes, as the reference does)."""
    rng = np.random.default_rng(m + n + rs + cs)
    A = rng.integers(0, 97, size=(m, n))
    Ag = gffm.CuModMatrix(A, 97, elem_type=torch.float64)
    X = (gffm.backward_sub_gpu_type_32 if upper else gffm.forward_sub_gpu_type_32)(Ag, rs, cs)
    assert X.size == (n, m)
    np.testing.assert_array_equal(as_int(X), oracle.tri_sub32(A, 97, rs, cs, upper))


def test_mod_inv_matches_oracle(gffm):
    rng = np.random.default_rng(2)
    for P in (7, 1000, 65521, P26, 2 ** 52):
        for p in list(rng.integers(0, P, size=20)) + [0, 1, P - 1, -3, P + 5]:
            assert gffm.mod_inv(int(p), P) == oracle.mod_inv(int(p), P)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_div_and_truediv(gffm, dtype):
    rng = np.random.default_rng(6)
    N = 65521
    A = rng.integers(0, N, size=(50, 40))
    Ag = gffm.CuModMatrix(A, N, elem_type=dtype)
    for s in (3, 12345, N - 1, -7):
        inv = oracle.mod_inv(s, N)
        want = (A.astype(np.int64) * (inv % N)) % N
        np.testing.assert_array_equal(as_int(Ag / s), want)
        C = gffm.zeros(dtype, 50, 40, N)
        gffm.div_(C, Ag, s)
        np.testing.assert_array_equal(as_int(C), want)
    # mod_N override: the inverse taken modulo the override
    C = gffm.zeros(dtype, 50, 40, N)
    gffm.div_(C, Ag, 5, 1009)
    np.testing.assert_array_equal(as_int(C), (A % 1009 * oracle.mod_inv(5, 1009)) % 1009)


def test_divide_elements(gffm):
    """divide_elements!(B, A, N): truncating division over the padded data; returns A."""
    A = gffm.CuModMatrix(np.array([[0, 7, 13], [20, 6, 1]]), 1000, elem_type=torch.float64)
    B = gffm.zeros(torch.float64, 2, 3, 1000)
    out = gffm.divide_elements_(B, A, 7)
    assert out is A
    assert as_int(B).tolist() == [[0, 1, 1], [2, 0, 0]]


@pytest.mark.parametrize("p,k,n", [(13, 4, 70), (101, 3, 40), (5, 9, 33)])
def test_hensel_pseudoinverse(gffm, p, k, n):
    """hensel_pseudoinverse (triangular/hensel.jl:13-20): lift A T = I mod p to mod p^k."""
    M = p ** k
    rng = np.random.default_rng(p + k + n)
    Lo = np.tril(rng.integers(0, p, size=(n, n)))
    Up = np.triu(rng.integers(0, p, size=(n, n)))
    d = np.arange(n)
    Lo[d, d] = rng.integers(1, p, size=n)
    Up[d, d] = rng.integers(1, p, size=n)
    A = oracle.matmul(Lo, Up, M)                                   # invertible mod p
    T0 = oracle.matmul(oracle.tri_inverse(Up % p, p, True)[0], oracle.tri_inverse(Lo % p, p, False)[0], p)
    assert (oracle.matmul(A % p, T0, p) == np.eye(n, dtype=np.int64)).all()
    want, i = T0 % M, 1
    while i < k:                                                   # the iteration itself, on the oracle's GEMM
        want = (2 * want - oracle.matmul(want, oracle.matmul(A, want, M), M)) % M
        i *= 2
    got = gffm.hensel_pseudoinverse(p, k, gffm.CuModMatrix(A, M, elem_type=torch.float64),
                                    gffm.CuModMatrix(T0, M, elem_type=torch.float64))
    assert got.N == M
    np.testing.assert_array_equal(as_int(got), want)
    assert (oracle.matmul(A, want, M) == np.eye(n, dtype=np.int64)).all()
