"""GPU parity tests: modular GEMM (limb tensor-core and plain paths), GEMV and
the elementwise kernels, against the oracle and the reference's known-answer
vectors.  Bar: bit-exact equality on every output element."""
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


def kat(op):
    with open(os.path.join(HERE, "golden", "reference_kat.json")) as f:
        return [c for c in json.load(f)["cases"] if c["op"] == op]


def status_ok(gffm):
    assert gffm.load_library().gffm_device_status(None) == 0


def as_int(M):
    return np.rint(M.Array()).astype(np.int64)


@pytest.mark.parametrize("case", kat("matmul") + kat("matmul_override"), ids=lambda c: c["src"])
@pytest.mark.parametrize("method", ["limb", "plain"])
def test_kat_matmul(gffm, case, method):
    Ns = case.get("N_storage", case["N"])
    A = gffm.CuModMatrix(case["A"], Ns, elem_type=torch.float64)
    B = gffm.CuModMatrix(case["B"], Ns, elem_type=torch.float64)
    C = gffm.mat_mul_gpu_type(A, B, case["N"] if "N_storage" in case else -1, method=method)
    assert as_int(C).tolist() == case["expected"]
    if "N_storage" not in case:
        C2 = A * B
        assert as_int(C2).tolist() == case["expected"]
    status_ok(gffm)


@pytest.mark.parametrize("elem", ["f32", "f64"])
def test_kat_elementwise(gffm, elem):
    dt = torch.float32 if elem == "f32" else torch.float64
    ops = {"add": gffm.add_, "sub": gffm.sub_, "elementwise_mul": gffm.elementwise_multiply_}
    for op, fn in ops.items():
        for c in kat(op):
            A = gffm.CuModMatrix(c["A"], 10 ** 6, mod=False, elem_type=dt)
            B = gffm.CuModMatrix(c["B"], 10 ** 6, mod=False, elem_type=dt)
            C = gffm.zeros(dt, *A.size, c["N"])
            fn(C, A, B, mod_N=c["N"]) if op != "elementwise_mul" else fn(C, A, B, c["N"])
            assert as_int(C).tolist() == c["expected"], (op, c["src"])
    sc = {"scalar_add": gffm.scalar_add_, "scalar_sub": gffm.scalar_sub_, "scalar_mul": gffm.scalar_mul_}
    for op, fn in sc.items():
        for c in kat(op):
            A = gffm.CuModMatrix(c["A"], 10 ** 6, mod=False, elem_type=dt)
            C = gffm.zeros(dt, *A.size, c["N"])
            fn(C, A, c["s"], c["N"])
            assert as_int(C).tolist() == c["expected"], (op, c["src"])
    for c in kat("negate"):
        A = gffm.CuModMatrix(c["A"], c["N"], elem_type=dt)
        C = gffm.zeros(dt, *A.size, c["N"])
        gffm.negate_(C, A)
        assert as_int(C).tolist() == c["expected"]
        assert as_int(-A).tolist() == c["expected"]
    for c in kat("mod"):
        A = gffm.CuModMatrix(c["A"], 10 ** 6, mod=False, elem_type=dt)
        gffm.mod_elements_(A, c["N"])
        assert as_int(A).tolist() == c["expected"]
    for c in kat("fill"):
        F = gffm.zeros(dt, *c["shape"], c["N"])
        gffm.fill_(F, c["s"])
        assert as_int(F).tolist() == c["expected"]
    status_ok(gffm)


def test_operators_match_reference_formulas(gffm):
    A_data = np.array([[1, 2, 3], [4, 5, 6], [7, 8, 9]])
    B_data = np.array([[9, 8, 7], [6, 5, 4], [3, 2, 1]])
    A = gffm.CuModMatrix(A_data, 11)
    B = gffm.CuModMatrix(B_data, 11)
    assert (as_int(A + B) == (A_data + B_data) % 11).all()
    assert (as_int(A - B) == (A_data - B_data) % 11).all()
    assert (as_int(A * B) == (A_data @ B_data) % 11).all()
    assert (as_int(3 + A) == (3 + A_data) % 11).all()
    assert (as_int(A - 3) == (A_data - 3) % 11).all()
    assert (as_int(3 * A) == (3 * A_data) % 11).all()
    assert (as_int(A * -1) == (-A_data) % 11).all()
    G_data = np.array([[1, 2, 3], [0, 1, 4], [5, 6, 0]])
    G = gffm.CuModMatrix(G_data, 11)
    assert (as_int(G ** 2) == (G_data @ G_data) % 11).all()
    assert (as_int(G ** 0) == np.eye(3, dtype=np.int64)).all()
    status_ok(gffm)


# moduli at each digit-count boundary of the limb path, plus the benchmark primes
LIMB_MODULI = [2, 7, 127, 128, 16255, 16256, 65521, 2080639, 2080640, P25, P26, 2 ** 26 - 1]
SHAPES = [(1, 1, 1), (5, 7, 3), (129, 65, 100), (130, 200, 1025), (64, 64, 4160), (300, 70, 1344)]


def patterns(rng, N, m, n, k):
    yield "uniform", rng.integers(0, N, size=(m, k)), rng.integers(0, N, size=(k, n))
    # largest centred magnitudes: every digit near +-64, partial sums at the exactness bound
    hi = (N - 1) // 2 if N > 2 else 1
    lo = (N + 1) // 2 if N > 2 else 1
    yield "all_hi", np.full((m, k), hi), np.full((k, n), hi)
    yield "hi_lo", np.full((m, k), hi), np.full((k, n), lo)
    yield "mixed", np.where(rng.random((m, k)) < 0.5, hi, lo), np.where(rng.random((k, n)) < 0.5, lo, hi)


@pytest.mark.parametrize("N", LIMB_MODULI)
@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: "x".join(map(str, s)))
def test_limb_gemm_matches_oracle(gffm, N, shape):
    rng = np.random.default_rng(N * 7 + shape[2])
    m, n, k = shape
    for name, A, B in patterns(rng, N, m, n, k):
        Ag = gffm.CuModMatrix(A, N, elem_type=torch.float64)
        Bg = gffm.CuModMatrix(B, N, elem_type=torch.float64)
        C = gffm.mat_mul_gpu_type(Ag, Bg, method="limb")
        want = oracle.matmul(A, B, N)
        got = as_int(C)
        assert np.array_equal(got, want), "%s: %d mismatches" % (name, int((got != want).sum()))
    status_ok(gffm)


@pytest.mark.parametrize("N", [11, 2 ** 11, 11 ** 3, 4093])
def test_limb_gemm_f32_storage(gffm, N):
    rng = np.random.default_rng(N)
    A = rng.integers(0, N, size=(100, 100))
    B = rng.integers(0, N, size=(100, 100))
    A[4, 4] = N - 5
    B[94, 94] = N - 23 if N > 23 else 0
    Ag = gffm.CuModMatrix(A, N, elem_type=torch.float32)
    Bg = gffm.CuModMatrix(B, N, elem_type=torch.float32)
    C = gffm.zeros(torch.float32, 100, 100, N)
    gffm.mul_(C, Ag, Bg, method="limb")
    assert np.array_equal(as_int(C), oracle.matmul(A, B, N))
    status_ok(gffm)


@pytest.mark.parametrize("N,elem", [(2 ** 11, "f32"), (11 ** 3, "f32"), (65521, "f64"), (P25, "f64"), (P26, "f64")])
def test_plain_gemm_matches_oracle(gffm, N, elem):
    # stripe_mul_test.jl:2-50 pattern: random entries with injected large residues
    dt = torch.float32 if elem == "f32" else torch.float64
    rng = np.random.default_rng(N)
    for (m, n, k) in [(100, 100, 100), (77, 130, 257)]:
        A = rng.integers(0, N, size=(m, k))
        B = rng.integers(0, N, size=(k, n))
        A[4, 4] = N - 5
        B[min(94, k - 1), min(94, n - 1)] = N - 23
        Ag = gffm.CuModMatrix(A, N, elem_type=dt)
        Bg = gffm.CuModMatrix(B, N, elem_type=dt)
        C = gffm.zeros(dt, m, n, N)
        gffm.stripe_mul_(C, Ag, Bg)
        assert np.array_equal(as_int(C), oracle.matmul(A, B, N))
    status_ok(gffm)


@pytest.mark.parametrize("N,elem", [(11 ** 3, "f32"), (7 ** 4, "f32"), (65521, "f64"), (P26, "f64")])
def test_plain_matvec_matches_oracle(gffm, N, elem):
    dt = torch.float32 if elem == "f32" else torch.float64
    rng = np.random.default_rng(N + 1)
    m, k = 3003, 1000
    A = rng.integers(0, N, size=(m, k))
    x = rng.integers(0, N, size=(k,))
    A[4, 4] = N - 5
    z = gffm.zeros(dt, m, N)
    gffm.mul_(z, gffm.CuModMatrix(A, N, elem_type=dt), gffm.CuModVector(x, N, elem_type=dt))
    want = oracle.matmul(A, x.reshape(-1, 1), N).reshape(-1)
    assert np.array_equal(np.rint(z.Array()).astype(np.int64), want)
    status_ok(gffm)


def test_limb_and_plain_agree_medium(gffm):
    rng = np.random.default_rng(99)
    m = n = k = 640
    A = rng.integers(0, P26, size=(m, k))
    B = rng.integers(0, P26, size=(k, n))
    Ag = gffm.CuModMatrix(A, P26, elem_type=torch.float64)
    Bg = gffm.CuModMatrix(B, P26, elem_type=torch.float64)
    C1 = gffm.mat_mul_gpu_type(Ag, Bg, method="limb")
    C2 = gffm.mat_mul_gpu_type(Ag, Bg, method="plain")
    assert np.array_equal(as_int(C1), as_int(C2))
    assert np.array_equal(as_int(C1), oracle.matmul(A, B, P26))
    status_ok(gffm)


def test_limb_gemm_8192_cube_properties(gffm):
    """8192^3 mod p26 (the benchmark size): Freivalds' check C x = A (B x) on two
    random vectors, plus exact oracle values for sampled rows and columns."""
    n = 8192
    g = torch.Generator(device="cuda")
    g.manual_seed(1234)
    A = gffm.rand(torch.float64, n, n, P26, generator=g)
    B = gffm.rand(torch.float64, n, n, P26, generator=g)
    C = gffm.mat_mul_gpu_type(A, B, method="limb")
    torch.cuda.synchronize()
    Ah, Bh, Ch = as_int(A), as_int(B), as_int(C)
    rng = np.random.default_rng(5)
    for _ in range(2):
        x = rng.integers(0, P26, size=(n, 1))
        lhs = oracle.matmul(Ch, x, P26)
        rhs = oracle.matmul(Ah, oracle.matmul(Bh, x, P26), P26)
        assert np.array_equal(lhs, rhs)
    rows = rng.integers(0, n, size=4)
    cols = rng.integers(0, n, size=4)
    assert np.array_equal(Ch[rows, :], oracle.matmul(Ah[rows, :], Bh, P26))
    assert np.array_equal(Ch[:, cols], oracle.matmul(Ah, Bh[:, cols], P26))
    status_ok(gffm)


def test_limb_gemm_caller_workspace_and_ld(gffm):
    """Caller-provided workspace and leading dimensions larger than the padding."""
    import ctypes
    rng = np.random.default_rng(3)
    m, n, k, N = 100, 90, 333, 65521
    A = rng.integers(0, N, size=(m, k))
    B = rng.integers(0, N, size=(k, n))
    lda, ldb, ldc = m + 40, k + 8, m + 3
    Ad = torch.zeros((k, lda), dtype=torch.float64, device="cuda")
    Bd = torch.zeros((n, ldb), dtype=torch.float64, device="cuda")
    Cd = torch.full((n, ldc), -1.0, dtype=torch.float64, device="cuda")
    Ad[:, :m] = torch.from_numpy(A.T.astype(np.float64)).cuda()
    Bd[:, :k] = torch.from_numpy(B.T.astype(np.float64)).cuda()
    L = gffm.load_library()
    ws = ctypes.c_size_t(0)
    assert L.gffm_matmul_limb_workspace_size(m, n, k, N, ctypes.byref(ws)) == 0
    buf = torch.empty(ws.value, dtype=torch.uint8, device="cuda")
    st = L.gffm_matmul_limb_f64(m, n, k, Ad.data_ptr(), lda, Bd.data_ptr(), ldb, Cd.data_ptr(), ldc, N,
                                buf.data_ptr(), ws.value, None)
    assert st == 0
    torch.cuda.synchronize()
    got = Cd.cpu().numpy().T
    assert np.array_equal(np.rint(got[:m, :]).astype(np.int64), oracle.matmul(A, B, N))
    assert (got[m:, :] == -1.0).all()           # rows past m untouched
    small = torch.empty(16, dtype=torch.uint8, device="cuda")
    assert L.gffm_matmul_limb_f64(m, n, k, Ad.data_ptr(), lda, Bd.data_ptr(), ldb, Cd.data_ptr(), ldc, N,
                                  small.data_ptr(), 16, None) == 5
    status_ok(gffm)


def test_empty_and_degenerate(gffm):
    N = P26
    A = gffm.zeros(torch.float64, 5, 0, N)
    B = gffm.zeros(torch.float64, 0, 7, N)
    C = gffm.zeros(torch.float64, 5, 7, N)
    gffm.fill_(C, 3)
    gffm.mul_(C, A, B, method="limb")
    assert (as_int(C) == 0).all()
    Z = gffm.zeros(torch.float64, 0, 4, N)
    gffm.mul_(gffm.zeros(torch.float64, 0, 3, N), Z, gffm.zeros(torch.float64, 4, 3, N), method="limb")
    status_ok(gffm)


# ---- digit width (the autotuner's choice): 8-bit digits at every boundary ----
BITS8_MODULI = [2, 7, 255, 256, 65279, 65280, 65521, 2080640, 8388593, 16711423, 16711424, P26]


@pytest.mark.parametrize("N", BITS8_MODULI)
@pytest.mark.parametrize("shape", [(5, 7, 3), (129, 65, 100), (130, 200, 1025), (64, 64, 4160)],
                         ids=lambda s: "x".join(map(str, s)))
def test_limb_gemm_8bit_digits(gffm, N, shape):
    rng = np.random.default_rng(N * 3 + shape[2])
    m, n, k = shape
    tu = gffm.LimbTuning(8, 0, 0, 0)
    for name, A, B in patterns(rng, N, m, n, k):
        Ag = gffm.CuModMatrix(A, N, elem_type=torch.float64)
        Bg = gffm.CuModMatrix(B, N, elem_type=torch.float64)
        got = as_int(gffm.mat_mul_gpu_type(Ag, Bg, method="limb", tuning=tu))
        want = oracle.matmul(A, B, N)
        assert np.array_equal(got, want), "%s: %d mismatches" % (name, int((got != want).sum()))
    status_ok(gffm)


def test_tune_table_routes_products(gffm):
    """A tune table entry switches the digit width (visible in the workspace size) and the
    grid; the products stay exact; clearing restores the defaults."""
    import ctypes
    from gffm import autotune
    N, m, n, k = 8388593, 300, 200, 1000
    L = gffm.load_library()
    table = {"gemm": [{"N_lo": 2080640, "N_hi": 16711423, "work_lo": 0, "work_hi": 1e30, "digit_bits": 8,
                       "max_ctas": 7}], "batched": {}}
    try:
        assert autotune.apply({"gemm": []}) == 0          # no table: 7-bit digits
        ws7 = ctypes.c_size_t(0)
        assert L.gffm_matmul_limb_workspace_size(m, n, k, N, ctypes.byref(ws7)) == 0
        assert autotune.apply(table) == 1
        ws8 = ctypes.c_size_t(0)
        assert L.gffm_matmul_limb_workspace_size(m, n, k, N, ctypes.byref(ws8)) == 0
        assert ws8.value * 4 == ws7.value * 3          # 3 digits instead of 4
        rng = np.random.default_rng(5)
        A, B = rng.integers(0, N, size=(m, k)), rng.integers(0, N, size=(k, n))
        C = gffm.mat_mul_gpu_type(gffm.CuModMatrix(A, N, elem_type=torch.float64),
                                  gffm.CuModMatrix(B, N, elem_type=torch.float64))
        assert np.array_equal(as_int(C), oracle.matmul(A, B, N))
    finally:
        autotune.apply()                                  # back to the shipped table
    status_ok(gffm)


def test_limb_tuning_errors(gffm):
    A = gffm.CuModMatrix([[1, 2], [3, 4]], 7, elem_type=torch.float64)
    with pytest.raises(gffm.GFFMError) as ei:
        gffm.mat_mul_gpu_type(A, A, method="limb", tuning=gffm.LimbTuning(9, 0, 0, 0))
    assert ei.value.status == 1
    with pytest.raises(gffm.GFFMError) as ei:
        gffm.mat_mul_gpu_type(A, A, method="limb", tuning=gffm.LimbTuning(7, -1, 0, 0))
    assert ei.value.status == 1


@pytest.mark.parametrize("N", [7, 16255, 65521, 8388593, P26])
@pytest.mark.parametrize("bits", [7, 8])
@pytest.mark.parametrize("shape", [(130, 200, 128), (129, 65, 1025), (300, 70, 5000)], ids=lambda s: "x".join(map(str, s)))
def test_limb_gemm_32_column_tiles(gffm, N, bits, shape):
    """The 32-column tile with two accumulator sets (a tuner candidate) is exact too."""
    rng = np.random.default_rng(N + bits + shape[2])
    m, n, k = shape
    tu = gffm.LimbTuning(bits, 0, 32, 0)
    for name, A, B in patterns(rng, N, m, n, k):
        got = as_int(gffm.mat_mul_gpu_type(gffm.CuModMatrix(A, N, elem_type=torch.float64),
                                           gffm.CuModMatrix(B, N, elem_type=torch.float64), method="limb", tuning=tu))
        want = oracle.matmul(A, B, N)
        assert np.array_equal(got, want), "%s: %d mismatches" % (name, int((got != want).sum()))
    status_ok(gffm)


# ---- the two product forms: schoolbook (16 digit products) and one-level Karatsuba (12) ----
KARA_MODULI = [2080640, 8388593, P25, P26, 2 ** 26 - 1]
KARA_SHAPES = [(1, 1, 1), (130, 200, 1024), (129, 257, 1025), (64, 130, 2048), (64, 130, 2112), (200, 64, 4096),
               (70, 300, 4161), (256, 256, 8256)]


def kara_extreme(N, rng, shape):
    """Residues whose Karatsuba digits sit at their extremes: a0, a2 in {-64, 63}, a1 in
    {-32, 31, 32} and a3 at the largest magnitude the modulus allows
    (c = a0 + 2^7 a1 + 2^13 (a2 + 2^7 a3)), kept within the centred range."""
    half = (N - 1) // 2
    top = max(1, min(32, (half // 8192 + 63) // 128))
    size = int(np.prod(shape))
    got = np.zeros(0, dtype=np.int64)
    for _ in range(100):
        if got.size >= size:
            break
        a0 = rng.choice(np.array([-64, 63]), size=2 * size)
        a2 = rng.choice(np.array([-64, 63]), size=2 * size)
        a1 = rng.choice(np.array([-32, 31, 32]), size=2 * size)
        a3 = rng.choice(np.array([-top, top - 1, top]), size=2 * size)
        lo = a0 + 128 * a1
        c = lo + 8192 * (a2 + 128 * a3)
        ok = (lo >= -4096) & (lo <= 4095) & (np.abs(c) <= half)
        got = np.concatenate([got, c[ok] % N])
    assert got.size >= size
    return got[:size].reshape(shape)


def kara_worst(N):
    """One residue whose Karatsuba digits sit at the exactness bounds: halves lo = hi = 4032
    give a0 = a2 = -64 with a1 = a3 = 32 (P0 and P2: |a0 b1| + |a1 b0| = 4096 per k) and the
    sum S = 8064 = 128 * 63 (Pm's last shift: |s1 t1| = 3969 per k);
    smaller halves where N is too small for them."""
    for h in (4032, 2048, 1024, 0):
        c = 4032 + 8192 * h
        if abs(c) <= (N - 1) // 2:
            return c % N
    return 1


def kara_sigma_worst(N):
    """A residue whose Karatsuba sum S = lo + hi = 8128 has digits s0 = -64, s1 = 64: the middle
    product's cross shift |s0 t1| + |s1 t0| reaches its bound 8192 per k."""
    c = 4064 + 8192 * 4064          # lo = hi = 4064, S = 8128 = -64 + 128 * 64
    return c % N if abs(c) <= (N - 1) // 2 else kara_worst(N)


@pytest.mark.parametrize("N", KARA_MODULI)
@pytest.mark.parametrize("shape", KARA_SHAPES, ids=lambda s: "x".join(map(str, s)))
@pytest.mark.parametrize("form", [1, 2], ids=["schoolbook", "karatsuba"])
def test_limb_gemm_forms_match_oracle(gffm, N, shape, form):
    rng = np.random.default_rng(N % 1000 + shape[2] + form)
    m, n, k = shape
    tu = gffm.LimbTuning(0, 0, 0, form)
    cases = list(patterns(rng, N, m, n, k))
    cases.append(("kara_extreme", kara_extreme(N, rng, (m, k)), kara_extreme(N, rng, (k, n))))
    w = kara_worst(N)
    cases.append(("kara_worst", np.full((m, k), w), np.full((k, n), w)))
    cases.append(("kara_worst_neg", np.full((m, k), w), np.full((k, n), (N - w) % N)))
    v = kara_sigma_worst(N)
    cases.append(("kara_sigma_worst", np.full((m, k), v), np.full((k, n), v)))
    cases.append(("kara_sigma_worst_neg", np.full((m, k), v), np.full((k, n), (N - v) % N)))
    for name, A, B in cases:
        got = as_int(gffm.mat_mul_gpu_type(gffm.CuModMatrix(A, N, elem_type=torch.float64),
                                           gffm.CuModMatrix(B, N, elem_type=torch.float64), method="limb", tuning=tu))
        want = oracle.matmul(A, B, N)
        assert np.array_equal(got, want), "%s: %d mismatches" % (name, int((got != want).sum()))
    status_ok(gffm)


@pytest.mark.parametrize("N", [8388593, P26])
def test_karatsuba_form_f32_storage_and_workspace(gffm, N):
    """The Karatsuba form through the Float32 entry point (N < 2^24 only) and with a caller
    workspace of exactly the queried size; a tune table entry selects the form (the
    Float32 entry point takes no tuning argument)."""
    import ctypes
    from gffm import autotune
    rng = np.random.default_rng(N)
    m, n, k = 190, 250, 3000
    A, B = rng.integers(0, N, size=(m, k)), rng.integers(0, N, size=(k, n))
    L = gffm.load_library()
    table = {"gemm": [{"N_lo": 2080640, "N_hi": 2 ** 26 - 1, "work_lo": 0, "work_hi": 1e30, "digit_bits": 7,
                       "form": 2}], "batched": {}}
    try:
        assert autotune.apply(table) == 1
        ws = ctypes.c_size_t(0)
        assert L.gffm_matmul_limb_workspace_size(m, n, k, N, ctypes.byref(ws)) == 0
        # six planes of 128-row padded A and B digits
        assert ws.value == 6 * 2 * (256 + 256) * 3008
        buf = torch.empty(ws.value, dtype=torch.uint8, device="cuda")
        for dt, sfx in ((torch.float64, "f64"), (torch.float32, "f32")):
            if dt == torch.float32 and N >= 2 ** 24:
                continue
            Ag = gffm.CuModMatrix(A, N, elem_type=dt)
            Bg = gffm.CuModMatrix(B, N, elem_type=dt)
            C = gffm.zeros(dt, m, n, N)
            st = getattr(L, "gffm_matmul_limb_" + sfx)(m, n, k, Ag.data.data_ptr(), Ag.ld, Bg.data.data_ptr(), Bg.ld,
                                                      C.data.data_ptr(), C.ld, N, buf.data_ptr(), ws.value, None)
            assert st == 0
            assert np.array_equal(as_int(C), oracle.matmul(A, B, N))
    finally:
        autotune.apply()                                  # back to the shipped table
    status_ok(gffm)


def test_karatsuba_form_errors(gffm):
    A = gffm.CuModMatrix([[1, 2], [3, 4]], 65521, elem_type=torch.float64)
    with pytest.raises(gffm.GFFMError) as ei:            # the form needs four 7-bit digits
        gffm.mat_mul_gpu_type(A, A, method="limb", tuning=gffm.LimbTuning(0, 0, 0, 2))
    assert ei.value.status == 10
    with pytest.raises(gffm.GFFMError) as ei:
        gffm.mat_mul_gpu_type(A, A, method="limb", tuning=gffm.LimbTuning(0, 0, 0, 3))
    assert ei.value.status == 1
    status_ok(gffm)
