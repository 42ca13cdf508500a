// k_gemm_limb.cu -- host side of the limb tensor-core GEMM (gemm_limb.cuh):
// argument checks, workspace layout, TMA descriptors and launches.
#include "gemm_limb.cuh"
#include "limb_host.h"

#include <cudaTypedefs.h>
#include <mutex>

namespace limb {

static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
static std::once_flag g_encode_once;

static int get_encoder() {
    std::call_once(g_encode_once, [] {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    });
    if (!g_encode) return gffm::set_error(GFFM_ERR_CUDA, "cuTensorMapEncodeTiled is unavailable");
    return GFFM_OK;
}

// 2-D fp16 tensor map over `rows` rows of `kpad` elements, box = 64 x box_rows, 128-byte swizzle
static int make_map(CUtensorMap *map, const void *base, int64_t kpad, int64_t rows, int box_rows) {
    cuuint64_t dims[2] = {(cuuint64_t)kpad, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)(kpad * 2)};
    cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<void *>(base), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return gffm::set_error(GFFM_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return GFFM_OK;
}

int limbs_for(int64_t N) {
    // largest centred residue floor(N/2) must fit L balanced base-128 digits:
    // max positive value 63 * (128^L - 1) / 127
    if (N <= 127) return 1;
    if (N <= 16255) return 2;
    if (N <= 2080639) return 3;
    return 4;
}

Layout layout(int64_t m, int64_t n, int64_t k, int64_t N) {
    Layout g;
    g.L = limbs_for(N);
    g.Mpad = gffm::round_up(m > 0 ? m : 1, BM);
    g.Npad = gffm::round_up(n > 0 ? n : 1, BN);
    g.Kpad = gffm::round_up(k > 0 ? k : 1, BK);
    g.a_bytes = (size_t)g.L * g.Mpad * g.Kpad * 2;
    g.b_bytes = (size_t)g.L * g.Npad * g.Kpad * 2;
    return g;
}

int check_args(int64_t m, int64_t n, int64_t k, int64_t lda, int64_t ldb, int64_t ldc, int64_t N) {
    using gffm::set_error;
    if (m < 0 || n < 0 || k < 0) return set_error(GFFM_ERR_ARG, "negative matrix size");
    if (lda < (m > 1 ? m : 1) || ldb < (k > 1 ? k : 1) || ldc < (m > 1 ? m : 1))
        return set_error(GFFM_ERR_ARG, "leading dimension smaller than the number of rows");
    if (N < 2 || N >= (int64_t(1) << 26))
        return set_error(GFFM_ERR_MODULUS, "the limb tensor-core path needs 2 <= N < 2^26 (got %lld)", (long long)N);
    if (m > (int64_t(1) << 24) || n > (int64_t(1) << 24) || k > (int64_t(1) << 24))
        return set_error(GFFM_ERR_ARG, "matrix dimension above 2^24");
    return GFFM_OK;
}

template <typename T>
int split_a(const T *A, int64_t lda, int64_t m, int64_t k, __half *D, const Layout &g, int64_t N, cudaStream_t s) {
    ModN M{N, ~uint64_t(0) / (uint64_t)N};
    dim3 grid((unsigned)(g.Kpad / 32), (unsigned)(g.Mpad / 32));
    switch (g.L) {
        case 1: k_split_a<T, 1><<<grid, 256, 0, s>>>(A, lda, (int)m, (int)k, D, (int)g.Mpad, (int)g.Kpad, M); break;
        case 2: k_split_a<T, 2><<<grid, 256, 0, s>>>(A, lda, (int)m, (int)k, D, (int)g.Mpad, (int)g.Kpad, M); break;
        case 3: k_split_a<T, 3><<<grid, 256, 0, s>>>(A, lda, (int)m, (int)k, D, (int)g.Mpad, (int)g.Kpad, M); break;
        default: k_split_a<T, 4><<<grid, 256, 0, s>>>(A, lda, (int)m, (int)k, D, (int)g.Mpad, (int)g.Kpad, M); break;
    }
    GFFM_LAUNCH_CHECK("k_split_a");
    return GFFM_OK;
}

template <typename T>
int split_b(const T *B, int64_t ldb, int64_t k, int64_t n, __half *D, const Layout &g, int64_t N, cudaStream_t s) {
    ModN M{N, ~uint64_t(0) / (uint64_t)N};
    int64_t total = (g.Kpad / 2) * g.Npad;
    unsigned blocks = (unsigned)((total + 255) / 256);
    switch (g.L) {
        case 1: k_split_b<T, 1><<<blocks, 256, 0, s>>>(B, ldb, (int)k, (int)n, D, (int)g.Npad, (int)g.Kpad, M); break;
        case 2: k_split_b<T, 2><<<blocks, 256, 0, s>>>(B, ldb, (int)k, (int)n, D, (int)g.Npad, (int)g.Kpad, M); break;
        case 3: k_split_b<T, 3><<<blocks, 256, 0, s>>>(B, ldb, (int)k, (int)n, D, (int)g.Npad, (int)g.Kpad, M); break;
        default: k_split_b<T, 4><<<blocks, 256, 0, s>>>(B, ldb, (int)k, (int)n, D, (int)g.Npad, (int)g.Kpad, M); break;
    }
    GFFM_LAUNCH_CHECK("k_split_b");
    return GFFM_OK;
}

template <int L, int EPI>
static int launch_gemm_L(const CUtensorMap &ta, const CUtensorMap &tb, const Params &p, int grid, cudaStream_t s) {
    auto kern = k_gemm_limb<L, EPI>;
    GFFM_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, Cfg<L>::SMEM_BYTES));
    gffm::profile_hook().before(s);
    kern<<<grid, NUM_THREADS, Cfg<L>::SMEM_BYTES, s>>>(ta, tb, p);
    gffm::profile_hook().after(s);
    GFFM_LAUNCH_CHECK("k_gemm_limb");
    return GFFM_OK;
}

template <int EPI>
static int launch_gemm(int L, const CUtensorMap &ta, const CUtensorMap &tb, const Params &p, int grid, cudaStream_t s) {
    switch (L) {
        case 1: return launch_gemm_L<1, EPI>(ta, tb, p, grid, s);
        case 2: return launch_gemm_L<2, EPI>(ta, tb, p, grid, s);
        case 3: return launch_gemm_L<3, EPI>(ta, tb, p, grid, s);
        default: return launch_gemm_L<4, EPI>(ta, tb, p, grid, s);
    }
}

int gemm_digits(const Layout &g, const __half *Ad, const __half *Bd, int64_t m, int64_t n, int64_t k, int64_t N,
                void *C, int64_t ldc, int epi, int max_ctas, cudaStream_t s) {
    int st = get_encoder();
    if (st) return st;
    CUtensorMap ta, tb;
    st = make_map(&ta, Ad, g.Kpad, (int64_t)g.L * g.Mpad, BM);
    if (st) return st;
    st = make_map(&tb, Bd, g.Kpad, (int64_t)g.L * g.Npad, BN);
    if (st) return st;
    Params p;
    p.m = (int)m;
    p.n = (int)n;
    p.kblocks = (int)(k > 0 ? gffm::round_up(k, BK) / BK : 0);
    p.Mpad = (int)g.Mpad;
    p.Npad = (int)g.Npad;
    p.mtiles = (int)((m + BM - 1) / BM);
    p.ntiles = (int)((n + BN - 1) / BN);
    p.chunk_kb = 64 / g.L;
    p.N = N;
    p.minv = ~uint64_t(0) / (uint64_t)N;
    p.bias = N * (((int64_t(1) << 60) + N - 1) / N);
    int64_t w = 1 % N;
    for (int sft = 0; sft < MAX_SHIFTS; sft++) {
        p.W[sft] = (int32_t)w;
        w = (w * 128) % N;
    }
    p.C = C;
    p.ldc = ldc;
    p.err = gffm::device_error_flag();
    if (!p.err) return gffm::check_device();
    int ntiles = p.mtiles * p.ntiles;
    if (ntiles == 0) return GFFM_OK;
    int grid = gffm::sm_count();
    if (max_ctas > 0 && grid > max_ctas) grid = max_ctas;
    if (grid > ntiles) grid = ntiles;
    switch (epi) {
        case EPI_STORE_F64: return launch_gemm<EPI_STORE_F64>(g.L, ta, tb, p, grid, s);
        case EPI_STORE_F32: return launch_gemm<EPI_STORE_F32>(g.L, ta, tb, p, grid, s);
        case EPI_STORE_I32: return launch_gemm<EPI_STORE_I32>(g.L, ta, tb, p, grid, s);
        default: return launch_gemm<EPI_SUB_I32>(g.L, ta, tb, p, grid, s);
    }
}

template int split_a<double>(const double *, int64_t, int64_t, int64_t, __half *, const Layout &, int64_t, cudaStream_t);
template int split_a<float>(const float *, int64_t, int64_t, int64_t, __half *, const Layout &, int64_t, cudaStream_t);
template int split_a<int32_t>(const int32_t *, int64_t, int64_t, int64_t, __half *, const Layout &, int64_t, cudaStream_t);
template int split_b<double>(const double *, int64_t, int64_t, int64_t, __half *, const Layout &, int64_t, cudaStream_t);
template int split_b<float>(const float *, int64_t, int64_t, int64_t, __half *, const Layout &, int64_t, cudaStream_t);
template int split_b<int32_t>(const int32_t *, int64_t, int64_t, int64_t, __half *, const Layout &, int64_t, cudaStream_t);

}  // namespace limb

namespace {

template <typename T>
int matmul_limb(int64_t m, int64_t n, int64_t k, const T *A, int64_t lda, const T *B, int64_t ldb, T *C, int64_t ldc,
                int64_t N, void *ws, size_t ws_bytes, gffm_stream_t stream) {
    using namespace gffm;
    int st = limb::check_args(m, n, k, lda, ldb, ldc, N);
    if (st) return st;
    if (m == 0 || n == 0) return GFFM_OK;
    if (!C || (k > 0 && (!A || !B))) return set_error(GFFM_ERR_ARG, "null data pointer");
    st = check_device();
    if (st) return st;
    cudaStream_t s = as_stream(stream);
    if (k == 0) {
        // empty inner dimension: C = 0
        GFFM_CUDA(cudaMemset2DAsync(C, (size_t)ldc * sizeof(T), 0, (size_t)m * sizeof(T), (size_t)n, s));
        return GFFM_OK;
    }
    limb::Layout g = limb::layout(m, n, k, N);
    Scratch scr;
    st = scr.acquire(ws, ws_bytes, g.a_bytes + g.b_bytes, s);
    if (st) return st;
    __half *Ad = static_cast<__half *>(scr.ptr);
    __half *Bd = reinterpret_cast<__half *>(static_cast<uint8_t *>(scr.ptr) + g.a_bytes);
    st = limb::split_a<T>(A, lda, m, k, Ad, g, N, s);
    if (st) return st;
    st = limb::split_b<T>(B, ldb, k, n, Bd, g, N, s);
    if (st) return st;
    return limb::gemm_digits(g, Ad, Bd, m, n, k, N, C, ldc,
                             sizeof(T) == 8 ? limb::EPI_STORE_F64 : limb::EPI_STORE_F32, 0, s);
}

}  // namespace

extern "C" {

int gffm_matmul_limb_workspace_size(int64_t m, int64_t n, int64_t k, int64_t N, size_t *bytes) {
    if (!bytes) return gffm::set_error(GFFM_ERR_ARG, "bytes is NULL");
    int st = limb::check_args(m, n, k, m > 1 ? m : 1, k > 1 ? k : 1, m > 1 ? m : 1, N);
    if (st) return st;
    limb::Layout g = limb::layout(m, n, k, N);
    *bytes = (m == 0 || n == 0 || k == 0) ? 0 : g.a_bytes + g.b_bytes;
    return GFFM_OK;
}

int gffm_matmul_limb_f64(int64_t m, int64_t n, int64_t k, const double *A, int64_t lda, const double *B, int64_t ldb,
                         double *C, int64_t ldc, int64_t N, void *ws, size_t ws_bytes, gffm_stream_t s) {
    return matmul_limb<double>(m, n, k, A, lda, B, ldb, C, ldc, N, ws, ws_bytes, s);
}

int gffm_matmul_limb_f32(int64_t m, int64_t n, int64_t k, const float *A, int64_t lda, const float *B, int64_t ldb,
                         float *C, int64_t ldc, int64_t N, void *ws, size_t ws_bytes, gffm_stream_t s) {
    return matmul_limb<float>(m, n, k, A, lda, B, ldb, C, ldc, N, ws, ws_bytes, s);
}

}  // extern "C"
