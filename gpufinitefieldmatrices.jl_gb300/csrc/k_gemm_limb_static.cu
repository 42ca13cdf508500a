// k_gemm_limb_static.cu -- the limb tensor-core GEMM with its digit-plane
// scratch in a fixed, library-owned device array instead of a workspace.
//
// Some callers cannot allocate device memory at call time: a process whose
// HBM is already reserved by another allocator (a framework memory pool that
// holds nearly all of the device) gets an out-of-memory error from any extra
// cudaMalloc/cudaMallocAsync, and a pipeline that must not stall cannot accept
// the implicit device synchronization of cudaMalloc/cudaFree.  For them
// gffm_matmul_limb_static_f64 takes inputs and outputs only and uses the
// array below as scratch; it never allocates or frees device memory.
//
// Limits and sharing: the array is kLimbStaticScratchBytes (32 MiB) on every
// GPU that loads the library, held until the process exits; a product whose
// digit planes need more is rejected.  All calls share the one array, so calls
// that overlap on the GPU (e.g. on two streams at once) race on it; calls on
// one stream are ordered and safe.  Each call rewrites every byte of scratch it
// reads (the split kernels write the digit planes, padding included), so the
// contents left by a previous call never need clearing.
#include "gffm_common.cuh"
#include "limb_host.h"

#include <cudaTypedefs.h>
#include <mutex>

namespace {

constexpr size_t kLimbStaticScratchBytes = size_t(32) << 20;

static __device__ __align__(256) uint8_t g_limb_static_scratch[kLimbStaticScratchBytes];

// Device address of the array, looked up with the device current (in host code
// the array's name is only a host-side stand-in) once per device and context:
// the address belongs to the context that loaded the module, so after
// cudaDeviceReset (a new primary context) it is looked up again.  Contexts are
// told apart by the driver's process-unique context ID.
constexpr int kMaxDev = 64;
struct ScratchAddr {
    unsigned long long ctx_id = 0;
    void *addr = nullptr;
};
ScratchAddr g_scratch_addr[kMaxDev];
std::mutex g_scratch_mu;

PFN_cuCtxGetCurrent_v4000 g_ctx_current = nullptr;
PFN_cuCtxGetId_v12000 g_ctx_id = nullptr;
std::once_flag g_ctx_once;

// the process-unique ID of the current context, or 0 when none is current (or it was destroyed)
unsigned long long current_context_id() {
    std::call_once(g_ctx_once, [] {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 4000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_ctx_current = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(fn);
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_ctx_id = reinterpret_cast<PFN_cuCtxGetId_v12000>(fn);
    });
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (!g_ctx_current || !g_ctx_id || g_ctx_current(&ctx) != CUDA_SUCCESS || !ctx ||
        g_ctx_id(ctx, &id) != CUDA_SUCCESS)
        return 0;
    return id;
}

int scratch_address(void **out) {
    int dev = 0;
    GFFM_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDev) return gffm::set_error(GFFM_ERR_UNSUPPORTED, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    ScratchAddr &a = g_scratch_addr[dev];
    const unsigned long long id = current_context_id();
    if (a.addr && id != 0 && id == a.ctx_id) {
        *out = a.addr;
        return GFFM_OK;
    }
    // first call on this device, or a new context: look the address up (this also makes
    // the device's primary context current), then remember which context it belongs to
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_limb_static_scratch);
    if (e != cudaSuccess) return gffm::cuda_error(e, "cudaGetSymbolAddress(limb static scratch)");
    a.addr = p;
    a.ctx_id = current_context_id();
    *out = p;
    return GFFM_OK;
}

}  // namespace

extern "C" {

int gffm_matmul_limb_static_max_bytes(size_t *bytes) {
    if (!bytes) return gffm::set_error(GFFM_ERR_ARG, "bytes is NULL");
    *bytes = kLimbStaticScratchBytes;
    return GFFM_OK;
}

int gffm_matmul_limb_static_scratch_size(int64_t m, int64_t n, int64_t k, int64_t N, size_t *bytes) {
    if (!bytes) return gffm::set_error(GFFM_ERR_ARG, "bytes is NULL");
    int st = limb::check_args(m, n, k, m > 1 ? m : 1, k > 1 ? k : 1, m > 1 ? m : 1, N);
    if (st) return st;
    // the static path always uses the untuned layout: 7-bit schoolbook digits, 128 x 64 tiles
    const limb::Layout g = limb::layout(m, n, k, N);
    *bytes = (m == 0 || n == 0 || k == 0) ? 0 : g.a_bytes + g.b_bytes;
    return GFFM_OK;
}

int gffm_matmul_limb_static_f64(int64_t m, int64_t n, int64_t k, const double *A, int64_t lda, const double *B,
                                int64_t ldb, double *C, int64_t ldc, int64_t N, gffm_stream_t stream) {
    using namespace gffm;
    int st = limb::check_args(m, n, k, lda, ldb, ldc, N);
    if (st) return st;
    if (m == 0 || n == 0) return GFFM_OK;
    if (!C || (k > 0 && (!A || !B))) return set_error(GFFM_ERR_ARG, "null data pointer");
    st = check_device();
    if (st) return st;
    cudaStream_t s = as_stream(stream);
    if (k == 0) {
        GFFM_CUDA(cudaMemset2DAsync(C, (size_t)ldc * sizeof(double), 0, (size_t)m * sizeof(double), (size_t)n, s));
        return GFFM_OK;
    }
    limb::Layout g = limb::layout(m, n, k, N);
    const size_t need = g.a_bytes + g.b_bytes;
    if (need > kLimbStaticScratchBytes)
        return set_error(GFFM_ERR_WORKSPACE,
                         "gffm_matmul_limb_static_f64: %lld x %lld x %lld mod %lld needs %zu bytes of digit planes, "
                         "more than the fixed %zu-byte scratch; use gffm_matmul_limb_f64",
                         (long long)m, (long long)n, (long long)k, (long long)N, need, kLimbStaticScratchBytes);
    void *scratch = nullptr;
    st = scratch_address(&scratch);
    if (st) return st;
    __half *Ad = static_cast<__half *>(scratch);
    __half *Bd = reinterpret_cast<__half *>(static_cast<uint8_t *>(scratch) + g.a_bytes);
    st = limb::split_a<double>(A, lda, m, k, Ad, g, N, s);
    if (st) return st;
    st = limb::split_b<double>(B, ldb, k, n, Bd, g, N, s);
    if (st) return st;
    return limb::gemm_digits(g, Ad, Bd, m, n, k, N, C, ldc, 0 /* EPI_STORE_F64 */, 0, s);
}

}  // extern "C"
