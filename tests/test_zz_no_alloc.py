"""GPU test of gffm_matmul_limb_static_f64, the limb GEMM that allocates nothing.

That entry point exists for callers that cannot allocate device memory when
they multiply -- a process whose HBM is already held by another allocator's
pool, or a pipeline that must not take the device-wide synchronization of
cudaMalloc/cudaFree -- so it keeps its digit-plane scratch in a fixed 32 MiB
array owned by the library.  Here it is called through the C ABI and its
output is compared, bit for bit, with gffm_matmul_limb_f64 (which takes a
workspace) on two calls in a row: the second call reuses the array the first
one left behind.  The file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

P26 = 67108859


def _operands(rng, m, n, k, N):
    A = torch.zeros((k, m + 32), dtype=torch.float64, device="cuda")
    B = torch.zeros((n, k + 32), dtype=torch.float64, device="cuda")
    A[:, :m] = torch.from_numpy(rng.integers(0, N, size=(k, m)).astype(np.float64)).cuda()
    B[:, :k] = torch.from_numpy(rng.integers(0, N, size=(n, k)).astype(np.float64)).cuda()
    return A, B


def _with_workspace(L, A, B, m, n, k, N):
    C = torch.zeros((n, m + 32), dtype=torch.float64, device="cuda")
    ws = ctypes.c_size_t(0)
    assert L.gffm_matmul_limb_workspace_size(m, n, k, N, ctypes.byref(ws)) == 0
    buf = torch.empty(max(ws.value, 1), dtype=torch.uint8, device="cuda")
    st = L.gffm_matmul_limb_f64(m, n, k, A.data_ptr(), m + 32, B.data_ptr(), k + 32, C.data_ptr(), m + 32, N,
                                buf.data_ptr(), ws.value, None)
    assert st == 0, L.gffm_last_error_string()
    return C


def _without_allocation(L, A, B, m, n, k, N):
    C = torch.full((n, m + 32), -7.0, dtype=torch.float64, device="cuda")
    st = L.gffm_matmul_limb_static_f64(m, n, k, A.data_ptr(), m + 32, B.data_ptr(), k + 32, C.data_ptr(), m + 32,
                                       N, None)
    assert st == 0, L.gffm_last_error_string()
    return C


def test_no_alloc_matches_workspace_entry_point_twice(gffm):
    L = gffm.load_library()
    rng = np.random.default_rng(4242)
    # two calls in a row with different shapes and moduli (3 and 4 digits):
    # the second one runs over the scratch contents the first one left behind
    for (m, n, k, N) in [(1000, 900, 1100, P26), (333, 517, 1024, 2080639)]:
        A, B = _operands(rng, m, n, k, N)
        want = _with_workspace(L, A, B, m, n, k, N)
        got = _without_allocation(L, A, B, m, n, k, N)
        torch.cuda.synchronize()
        assert torch.equal(got[:, :m], want[:, :m])
        assert (got[:, m:] == -7.0).all()     # nothing outside the m x n result is written
    assert L.gffm_device_status(None) == 0


def test_no_alloc_rejects_products_beyond_its_scratch(gffm):
    L = gffm.load_library()
    cap = ctypes.c_size_t(0)
    assert L.gffm_matmul_limb_static_max_bytes(ctypes.byref(cap)) == 0
    assert cap.value == 32 << 20
    # its scratch need is its own query's, whatever the tuned workspace path would take
    need = ctypes.c_size_t(0)
    assert L.gffm_matmul_limb_static_scratch_size(1000, 900, 1100, P26, ctypes.byref(need)) == 0
    assert need.value == 4 * (1024 + 960) * 1152 * 2          # 4 digit planes, 128 / 64 / 64 padding
    m = n = k = 2048             # 4 digits: 4 * (2048 + 2048) * 2048 * 2 bytes = 64 MiB > 32 MiB
    assert L.gffm_matmul_limb_static_scratch_size(m, n, k, P26, ctypes.byref(need)) == 0
    assert need.value > cap.value
    A = torch.zeros((k, m + 32), dtype=torch.float64, device="cuda")
    B = torch.zeros((n, k + 32), dtype=torch.float64, device="cuda")
    C = torch.zeros((n, m + 32), dtype=torch.float64, device="cuda")
    st = L.gffm_matmul_limb_static_f64(m, n, k, A.data_ptr(), m + 32, B.data_ptr(), k + 32, C.data_ptr(), m + 32,
                                       P26, None)
    assert st == 5
    assert b"fixed" in L.gffm_last_error_string()
