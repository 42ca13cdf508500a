"""GPU parity tests of the KaratsubaArray type: the digit-form product
(KMatMul!), its polynomial reading, and the elementwise digit kernels,
bit-exact against the oracle and the reference's known answers."""
import json
import os

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

HERE = os.path.dirname(os.path.abspath(__file__))
P25 = 33554393
P26 = 67108859


def status_ok(gffm):
    assert gffm.load_library().gffm_device_status(None) == 0


def digits(gffm, D, N):
    return gffm.CuModMatrix(np.asarray(D), N, mod=False, elem_type=torch.float64)


def tag(N1, N2):
    """The modulus tag M: N1*N2 where the reference's constructor accepts it (M < 2^51), else N1."""
    return N1 * N2 if N1 * N2 < 2 ** 51 else N1


def kmat(gffm, A1, A2, N1, N2, plan=True):
    K = gffm.KaratsubaMatrix(digits(gffm, A1, N1), digits(gffm, A2, N1), N1, N2, tag(N1, N2))
    if plan:
        gffm.initialize_plan_(K)
    return K


def as_int(M):
    return np.rint(M.Array()).astype(np.int64)


def test_kat_karatsuba(gffm):
    """test/KaratsubaMatrix/basic_operations_test.jl:51-65 through the mirror."""
    with open(os.path.join(HERE, "golden", "reference_kat.json")) as f:
        cases = [c for c in json.load(f)["cases"] if c["op"].startswith("karatsuba")]
    assert len(cases) == 7
    for c in cases:
        N1, N2 = c["N1"], c["N2"]
        A = kmat(gffm, c["A1"], c["A2"], N1, N2)
        if c["op"] == "karatsuba_scalar":
            R = c["s"] * A
        else:
            B = kmat(gffm, c["B1"], c["B2"], N1, N2)
            R = {"karatsuba_matmul": lambda: A * B, "karatsuba_add": lambda: A + B,
                 "karatsuba_sub": lambda: A - B}[c["op"]]()
        assert R.Array().tolist() == c["expected_value"], c["src"]
    status_ok(gffm)


def test_kat_mat_to_kmat(gffm):
    """MatToKMat(CuModMatrix([1 2; 3 4], 100), 100) + MatToKMat(B, 100) == A + B (basic_operations_test.jl:51-62)."""
    A = gffm.CuModMatrix([[1, 2], [3, 4]], 100, elem_type=torch.float64)
    B = gffm.CuModMatrix([[5, 6], [7, 8]], 100, elem_type=torch.float64)
    AK, BK = gffm.MatToKMat(A, 100), gffm.MatToKMat(B, 100)
    assert (AK + BK).Array().tolist() == [[6, 8], [10, 12]]
    assert (AK - BK).Array().tolist() == [[9996, 9996], [9996, 9996]]
    assert (9 * AK).Array().tolist() == [[9, 18], [27, 36]]
    assert (AK * BK).Array().tolist() == [[19, 22], [43, 50]]
    status_ok(gffm)


# (m, k, n, N1, N2): all four raw digit counts of N1, N2 dividing N1 and not,
# long K (several exact chunks), n = 1 (KaratsubaVector)
MM_CASES = [
    (5, 7, 4, 100, 100), (33, 20, 17, 49, 7), (130, 200, 70, 13 ** 4, 13 ** 3), (64, 64, 64, 50, 61),
    (129, 300, 65, 8000, 8000), (200, 150, 190, 1000003, 999983), (300, 257, 190, P25, P25),
    (96, 5000, 80, P26, P26), (70, 1100, 3, P26 - 2, 17), (150, 640, 1, 13 ** 4, 13 ** 3),
    (1, 1, 1, 2, 2), (40, 2200, 40, 2 ** 26 - 1, 2 ** 26 - 1),
]


@pytest.mark.parametrize("case", MM_CASES, ids=lambda c: "%dx%dx%d-%d-%d" % c)
@pytest.mark.parametrize("pattern", ["uniform", "max"])
def test_karatsuba_matmul_matches_oracle(gffm, case, pattern):
    m, k, n, N1, N2 = case
    rng = np.random.default_rng(m * 7 + k + n + N1 % 1000)
    if pattern == "max":     # every digit at its largest value: the exactness bounds
        A1, B1 = np.full((m, k), N1 - 1), np.full((k, n), N1 - 1)
        A2, B2 = np.full((m, k), N2 - 1), np.full((k, n), N2 - 1)
    else:
        A1, B1 = rng.integers(0, N1, size=(m, k)), rng.integers(0, N1, size=(k, n))
        A2, B2 = rng.integers(0, N2, size=(m, k)), rng.integers(0, N2, size=(k, n))
    c1, c2 = oracle.karatsuba_matmul(A1, A2, B1, B2, N1, N2)
    A, B = kmat(gffm, A1, A2, N1, N2), kmat(gffm, B1, B2, N1, N2)
    C = gffm.KaratsubaZeros(torch.float64, m, n, N1, N2, tag(N1, N2), True)
    gffm.initialize_plan_(C)
    gffm.KMatMul_(C, A, B)
    assert np.array_equal(as_int(C.data1), c1)
    assert np.array_equal(as_int(C.data2), c2)
    status_ok(gffm)


def test_karatsuba_gemv_reference_test(gffm):
    """test/KaratsubaMatrix/basic_operations_test.jl:75-127: n = 500, N1 = 13^4,
    N2 = 13^3, KMatMul!(yK, AK, xK) == mod(A x, N1 N2) (a few seeded draws)."""
    n, N1, N2 = 500, 13 ** 4, 13 ** 3
    rng = np.random.default_rng(500)
    for _ in range(3):
        A1, A2 = rng.integers(0, N1, size=(n, n)), rng.integers(0, N2, size=(n, n))
        x1, x2 = rng.integers(0, N1, size=n), rng.integers(0, N2, size=n)
        AK = kmat(gffm, A1, A2, N1, N2)
        xK = gffm.KaratsubaVector(gffm.CuModVector(x1, N1, elem_type=torch.float64),
                                  gffm.CuModVector(x2, N1, elem_type=torch.float64), N1, N2, N1 * N2)
        yK = gffm.KaratsubaVector(gffm.CuModVector(np.zeros(n, dtype=np.int64), N1, elem_type=torch.float64),
                                  gffm.CuModVector(np.zeros(n, dtype=np.int64), N1, elem_type=torch.float64),
                                  N1, N2, N1 * N2)
        for K in (AK, xK, yK):
            gffm.initialize_plan_(K)
        gffm.KMatMul_(yK, AK, xK)
        Acpu = A1 + N1 * A2
        xcpu = (x1 + N1 * x2).reshape(n, 1)
        want = oracle.matmul(Acpu, xcpu, N1 * N2).reshape(-1)
        assert np.array_equal(yK.Array(), want)
    status_ok(gffm)


def test_karatsuba_4096_freivalds(gffm):
    """4096 x 4096 x 4096 digits mod p25 (N1 = N2 = p25): the values X = A1 + N1 A2
    satisfy C v = X (Y v) mod p25^2 for random v (exact 128-bit host products)."""
    n, N = 4096, P25
    g = torch.Generator(device="cuda")
    g.manual_seed(4096)
    A = gffm.KaratsubaArray(gffm.rand(torch.float64, n, n, N, generator=g),
                            gffm.rand(torch.float64, n, n, N, generator=g), N, N, N * N)
    B = gffm.KaratsubaArray(gffm.rand(torch.float64, n, n, N, generator=g),
                            gffm.rand(torch.float64, n, n, N, generator=g), N, N, N * N)
    C = A * B
    X, Y, Cv = A.Array(), B.Array(), C.Array()
    assert (C.data1.Array() < N).all() and (C.data2.Array() < N).all()
    rng = np.random.default_rng(2)
    for _ in range(2):
        v = rng.integers(0, N * N, size=(n, 1))
        lhs = oracle.matmul(Cv, v, N * N)
        rhs = oracle.matmul(X, oracle.matmul(Y, v, N * N), N * N)
        assert np.array_equal(lhs, rhs)
    status_ok(gffm)


POLY_CASES = [(5, 7, 4, 7), (70, 130, 90, 65521), (300, 257, 190, P25), (128, 4100, 64, P26), (33, 64, 1, 3)]


@pytest.mark.parametrize("case", POLY_CASES, ids=lambda c: "%dx%dx%d-%d" % c)
def test_poly_karatsuba_matches_oracle(gffm, case):
    m, k, n, p = case
    rng = np.random.default_rng(m + k + n)
    A0, A1 = rng.integers(0, p, size=(m, k)), rng.integers(0, p, size=(m, k))
    B0, B1 = rng.integers(0, p, size=(k, n)), rng.integers(0, p, size=(k, n))
    want = oracle.poly_karatsuba_matmul(A0, A1, B0, B1, p)
    got = gffm.poly_karatsuba_matmul(*(digits(gffm, X, p) for X in (A0, A1, B0, B1)), p)
    for g_, w in zip(got, want):
        assert np.array_equal(as_int(g_), w)
    status_ok(gffm)


def test_poly_karatsuba_4096_identity(gffm):
    """4096^2 mod p25, the polynomial reading: (A0 + t A1)(B0 + t B1) v =
    (C0 + t C1 + t^2 C2) v mod p at random t and v."""
    n, p = 4096, P25
    g = torch.Generator(device="cuda")
    g.manual_seed(25)
    Ms = [gffm.rand(torch.float64, n, n, p, generator=g) for _ in range(4)]
    C0, C1, C2 = gffm.poly_karatsuba_matmul(*Ms, p)
    A0, A1, B0, B1 = (as_int(M) for M in Ms)
    H0, H1, H2 = (as_int(C) for C in (C0, C1, C2))
    rng = np.random.default_rng(3)
    for _ in range(2):
        t = int(rng.integers(1, p))
        v = rng.integers(0, p, size=(n, 1))
        Bt = (B0 + t * B1) % p
        At = (A0 + t * A1) % p
        lhs = oracle.matmul(At, oracle.matmul(Bt, v, p), p)
        Ct = (H0 + t * H1 % p + (t * t % p) * H2 % p) % p
        rhs = oracle.matmul(Ct, v, p)
        assert np.array_equal(lhs, rhs)
    status_ok(gffm)


ELT_PAIRS = [(100, 100), (13 ** 4, 13 ** 3), (P25, P25), (101, 103), (2 ** 26, 2 ** 26), (3, 2 ** 40)]


@pytest.mark.parametrize("N1,N2", ELT_PAIRS)
def test_karatsuba_elementwise_matches_oracle(gffm, N1, N2):
    rng = np.random.default_rng(N1 % 977 + N2 % 991)
    m, n = 67, 45
    X1, X2 = rng.integers(0, N1, size=(m, n)), rng.integers(0, N2, size=(m, n))
    Y1, Y2 = rng.integers(0, N1, size=(m, n)), rng.integers(0, N2, size=(m, n))
    X1[:5, :] = 0
    Y1[:, :3] = X1[:, :3]
    A, B = kmat(gffm, X1, X2, N1, N2), kmat(gffm, Y1, Y2, N1, N2)
    for got, want in [(A + B, oracle.karatsuba_addsub(X1, X2, Y1, Y2, N1, N2)),
                      (A - B, oracle.karatsuba_addsub(X1, X2, Y1, Y2, N1, N2, sub=True)),
                      (-A, oracle.karatsuba_scale(X1, X2, N1, N2, negate=True))] + \
                     [(s * A, oracle.karatsuba_scale(X1, X2, N1, N2, s=s))
                      for s in (0, 1, 9, -5, 2 ** 40 + 3, N1 * N2 - 1)]:
        assert np.array_equal(as_int(got.data1), want[0])
        assert np.array_equal(as_int(got.data2), want[1])
    status_ok(gffm)


def test_karatsuba_value_conversions(gffm):
    """KaratsubaMatrix(T, A, N1, N2, M) digit split (KaratsubaMatrix.jl:372-397) and KMatToMat."""
    N1, N2 = 13 ** 4, 13 ** 3
    rng = np.random.default_rng(9)
    V = rng.integers(0, N1 * N2 * 3, size=(50, 70))
    A = gffm.CuModMatrix(V, 2 ** 52, mod=False, elem_type=torch.float64)
    K = gffm.KaratsubaMatrix_from(A, N1, N2, N1 * N2)
    Vm = V % (N1 * N2)
    assert np.array_equal(as_int(K.data1), Vm % N1)
    assert np.array_equal(as_int(K.data2), Vm // N1)
    assert np.array_equal(K.Array(), Vm)
    assert np.array_equal(as_int(gffm.KMatToMat(K)), Vm)
    assert K[3, 4] == Vm[2, 3]
    status_ok(gffm)


def test_karatsuba_errors(gffm):
    A = kmat(gffm, [[1]], [[2]], 2 ** 26, 5)
    B = kmat(gffm, [[1]], [[2]], 2 ** 26, 5)
    C = gffm.KaratsubaZeros(torch.float64, 1, 1, 2 ** 26, 5, 2 ** 26 * 5, True)
    gffm.initialize_plan_(C)
    with pytest.raises(gffm.GFFMError) as ei:
        gffm.KMatMul_(C, A, B)
    assert ei.value.status == 3
    D = kmat(gffm, [[1]], [[2]], 7, 7)
    E = gffm.KaratsubaZeros(torch.float64, 1, 1, 7, 7, 49, True)
    gffm.initialize_plan_(E)
    with pytest.raises(ValueError):
        gffm.KMatMul_(E, A, D)                       # modulus tags differ
    F = kmat(gffm, [[1]], [[2]], 7, 7, plan=False)
    with pytest.raises(ValueError):
        gffm.KMatMul_(E, F, D)                       # no plan
    with pytest.raises(gffm.GFFMError) as ei:         # output aliases an operand
        gffm.KMatMul_(D, D, D)
    assert ei.value.status == 1
    G = gffm.KaratsubaMatrix(gffm.CuModMatrix([[1]], 7, elem_type=torch.float32),
                             gffm.CuModMatrix([[1]], 7, elem_type=torch.float32), 7, 7, 49)
    gffm.initialize_plan_(G)
    with pytest.raises(NotImplementedError):
        gffm.KMatMul_(E, G, G)
    status_ok(gffm)
