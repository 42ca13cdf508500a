"""GPU parity tests: the limb GEMM on host buffers (gffm_matmul_host_f64), whose
copies in and out run block by block beside the block products.  Bar:
bit-exact equality with the oracle on every output element, for one block and
for ragged block grids (the last row / column block shorter), padded leading
dimensions, pageable buffers, an empty inner dimension and every digit count."""
import ctypes

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
P26 = 67108859


def status_ok(gffm):
    assert gffm.load_library().gffm_device_status(None) == 0


@pytest.mark.parametrize("m,n,k,N", [
    (1, 1, 1, 7),
    (5, 7, 3, 65521),
    (300, 200, 100, P26),
    (130, 70, 300, 127),            # one digit
    (257, 129, 65, 16255),          # two digits
    (200, 300, 90, 2080639),        # three digits
    (2100, 300, 70, P26),           # two row blocks of A (1152 + 948)
    (300, 2200, 64, P26),           # two column blocks of B (1152 + 1048)
    (2200, 4200, 40, 65521),        # 2 x 3 blocks, ragged in both
    (4500, 300, 20, 65521),         # row blocks of 1536, 1536, 1428
])
def test_host_gemm_matches_oracle(gffm, m, n, k, N):
    rng = np.random.default_rng(m * 7 + n * 3 + k)
    A = rng.integers(0, N, size=(m, k))
    B = rng.integers(0, N, size=(k, n))
    got = gffm.matmul_host(A, B, N)
    np.testing.assert_array_equal(got, oracle.matmul(A, B, N))
    status_ok(gffm)


def test_host_gemm_pageable_and_unreduced(gffm):
    rng = np.random.default_rng(5)
    N = 1000003
    A = rng.integers(-3 * N, 3 * N, size=(150, 90))     # any integers: reduced mod N first
    B = rng.integers(-3 * N, 3 * N, size=(90, 110))
    got = gffm.matmul_host(A, B, N, pinned=False)
    np.testing.assert_array_equal(got, oracle.matmul(np.mod(A, N), np.mod(B, N), N))


def test_host_gemm_padded_leading_dims_and_workspace(gffm):
    """The CuModMatrix host layout: (rows + 32) x (cols + 32) column-major buffers, C's
    padding untouched; a caller-provided workspace of the queried size."""
    lib = gffm.load_library()
    rng = np.random.default_rng(9)
    m, n, k, N = 333, 2150, 77, P26
    A = rng.integers(0, N, size=(m, k))
    B = rng.integers(0, N, size=(k, n))
    hA = torch.zeros((k + 32, m + 32), dtype=torch.float64).pin_memory()
    hB = torch.zeros((n + 32, k + 32), dtype=torch.float64).pin_memory()
    hC = torch.full((n + 32, m + 32), -5.0, dtype=torch.float64).pin_memory()
    hA[:k, :m] = torch.from_numpy(A.T.astype(np.float64))
    hB[:n, :k] = torch.from_numpy(B.T.astype(np.float64))
    ws = ctypes.c_size_t(0)
    assert lib.gffm_matmul_host_workspace_size(m, n, k, N, ctypes.byref(ws)) == 0
    buf = torch.empty(ws.value, dtype=torch.uint8, device="cuda")
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = lib.gffm_matmul_host_f64(m, n, k, ctypes.c_void_p(hA.data_ptr()), m + 32, ctypes.c_void_p(hB.data_ptr()),
                                  k + 32, ctypes.c_void_p(hC.data_ptr()), m + 32, N, ctypes.c_void_p(buf.data_ptr()),
                                  ws.value, s)
    assert st == 0
    torch.cuda.current_stream().synchronize()
    C = hC.numpy().T
    np.testing.assert_array_equal(C[:m, :n].astype(np.int64), oracle.matmul(A, B, N))
    assert (C[m:, :] == -5.0).all() and (C[:, n:] == -5.0).all()
    status_ok(gffm)


def test_host_gemm_empty_inner_dimension(gffm):
    got = gffm.matmul_host(np.zeros((40, 0), dtype=np.int64), np.zeros((0, 30), dtype=np.int64), 97)
    assert got.shape == (40, 30) and not got.any()


def test_host_gemm_errors(gffm):
    with pytest.raises(gffm.GFFMError):
        gffm.matmul_host(np.ones((4, 4)), np.ones((4, 4)), 1 << 26)      # modulus out of range
    with pytest.raises(gffm.CuModArraySizeMismatchException):
        gffm.matmul_host(np.ones((4, 3)), np.ones((4, 4)), 97)
