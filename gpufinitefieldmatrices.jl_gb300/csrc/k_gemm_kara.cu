// k_gemm_kara.cu -- host side of the 12-product Karatsuba limb GEMM
// (gemm_kara.cuh): workspace layout, digit splits, TMA descriptors, weights
// and launches.
#include "gemm_kara.cuh"
#include "kara_host.h"
#include "limb_host.h"

namespace kara {

bool applies(int64_t N) { return N > 2080639 && N < (int64_t(1) << 26); }

Layout layout(int64_t m, int64_t n, int64_t k) {
    Layout g;
    g.Mpad = gffm::round_up(m > 0 ? m : 1, BM);
    g.Npad = gffm::round_up(n > 0 ? n : 1, BN);
    g.Kpad = gffm::round_up(k > 0 ? k : 1, BK);
    g.a_bytes = (size_t)PLANES * g.Mpad * g.Kpad * 2;
    g.b_bytes = (size_t)PLANES * g.Npad * g.Kpad * 2;
    return g;
}

template <typename T>
int split_a(const T *A, int64_t lda, int64_t m, int64_t k, __half *D, const Layout &g, int64_t N, cudaStream_t s,
            const T *A2) {
    limb::ModN M{N, ~uint64_t(0) / (uint64_t)N};
    dim3 grid((unsigned)(g.Kpad / 32), (unsigned)(g.Mpad / 32));
    if (A2)
        k_split_a6<T, limb::SPLIT_SUM><<<grid, 256, 0, s>>>(A, A2, lda, (int)m, (int)k, D, (int)g.Mpad, (int)g.Kpad, M);
    else
        k_split_a6<T, limb::SPLIT_CENTRED><<<grid, 256, 0, s>>>(A, A, lda, (int)m, (int)k, D, (int)g.Mpad, (int)g.Kpad, M);
    GFFM_LAUNCH_CHECK("k_split_a6");
    return GFFM_OK;
}

template <typename T>
int split_b(const T *B, int64_t ldb, int64_t k, int64_t n, __half *D, const Layout &g, int64_t N, cudaStream_t s,
            const T *B2) {
    limb::ModN M{N, ~uint64_t(0) / (uint64_t)N};
    const int64_t total = (g.Kpad / 2) * g.Npad;
    const unsigned blocks = (unsigned)((total + 255) / 256);
    if (B2)
        k_split_b6<T, limb::SPLIT_SUM><<<blocks, 256, 0, s>>>(B, B2, ldb, (int)k, (int)n, D, (int)g.Npad, (int)g.Kpad, M);
    else
        k_split_b6<T, limb::SPLIT_CENTRED><<<blocks, 256, 0, s>>>(B, B, ldb, (int)k, (int)n, D, (int)g.Npad, (int)g.Kpad, M);
    GFFM_LAUNCH_CHECK("k_split_b6");
    return GFFM_OK;
}

template <int EPI>
static int launch(const CUtensorMap &ta, const CUtensorMap &tb, const Params &p, int grid, cudaStream_t s) {
    GFFM_CUDA((gffm::ensure_dynamic_smem<k_gemm_kara<EPI>>(SMEM_BYTES)));
    gffm::profile_hook().before(s);
    k_gemm_kara<EPI><<<grid, THREADS, SMEM_BYTES, s>>>(ta, tb, p);
    gffm::profile_hook().after(s);
    GFFM_LAUNCH_CHECK("k_gemm_kara");
    return GFFM_OK;
}

int gemm_digits(const Layout &g, const __half *Ad, const __half *Bd, int64_t m, int64_t n, int64_t k, int64_t N,
                void *C, int64_t ldc, int epi, int max_ctas, cudaStream_t s, const double *X, const double *Y) {
    if (!applies(N)) return gffm::set_error(GFFM_ERR_MODULUS, "the Karatsuba form needs 2080639 < N < 2^26");
    if (epi == limb::EPI_KSUB_F64 && (!X || !Y))
        return gffm::set_error(GFFM_ERR_ARG, "subtracting epilogue without X, Y");
    if (epi != limb::EPI_STORE_F64 && epi != limb::EPI_STORE_F32 && epi != limb::EPI_STORE_I32 &&
        epi != limb::EPI_KSUB_F64)
        return gffm::set_error(GFFM_ERR_UNSUPPORTED, "epilogue %d is not available in the Karatsuba form", epi);
    CUtensorMap ta, tb;
    int st = limb::encode_digit_map(&ta, Ad, g.Kpad, (int64_t)PLANES * g.Mpad, BM);
    if (st) return st;
    st = limb::encode_digit_map(&tb, Bd, g.Kpad, (int64_t)PLANES * g.Npad, BN);
    if (st) return st;
    Params p;
    p.m = (int)m;
    p.n = (int)n;
    p.kblocks = (int)(k > 0 ? gffm::round_up(k, BK) / BK : 0);
    p.Mpad = (int)g.Mpad;
    p.Npad = (int)g.Npad;
    p.mtiles = (int)((m + BM - 1) / BM);
    p.ntiles = (int)((n + BN - 1) / BN);
    // exact chunks: |C_s| <= 4096 per k for P0 and P2, <= 8192 for Pm (fp32 sums within 2^24)
    p.chunk_kb[0] = 4096 / BK;
    p.chunk_kb[1] = 4096 / BK;
    p.chunk_kb[2] = 2048 / BK;
    p.N = N;
    p.minv = ~uint64_t(0) / (uint64_t)N;
    p.bias = N * (((int64_t(1) << 60) + N - 1) / N);
    // A*B = sum_s X^s [(1 - Y) C0_s + (Y^2 - Y) C2_s + Y Cm_s], X = 2^7, Y = 2^13
    const int64_t Y1 = (int64_t(1) << 13) % N;
    const int64_t Y2 = (int64_t)(((__int128)Y1 * Y1) % N);
    const int64_t coef[3] = {(1 - Y1 + N) % N, (Y2 - Y1 + N) % N, Y1};
    int64_t xs = 1 % N;
    for (int sft = 0; sft < 3; sft++) {
        for (int prod = 0; prod < 3; prod++) p.W[prod][sft] = (int32_t)(((__int128)xs * coef[prod]) % N);
        xs = (xs * 128) % N;
    }
    p.C = C;
    p.ldc = ldc;
    p.X = X;
    p.Y = Y;
    p.err = gffm::device_error_flag();
    if (!p.err) return gffm::check_device();
    const int ntiles = p.mtiles * p.ntiles;
    if (ntiles == 0 || p.kblocks == 0) return GFFM_OK;
    int grid = gffm::sm_count();
    if (max_ctas > 0 && grid > max_ctas) grid = max_ctas;
    if (grid > ntiles) grid = ntiles;
    switch (epi) {
        case limb::EPI_STORE_F64: return launch<limb::EPI_STORE_F64>(ta, tb, p, grid, s);
        case limb::EPI_STORE_F32: return launch<limb::EPI_STORE_F32>(ta, tb, p, grid, s);
        case limb::EPI_STORE_I32: return launch<limb::EPI_STORE_I32>(ta, tb, p, grid, s);
        default: return launch<limb::EPI_KSUB_F64>(ta, tb, p, grid, s);
    }
}

template int split_a<double>(const double *, int64_t, int64_t, int64_t, __half *, const Layout &, int64_t,
                             cudaStream_t, const double *);
template int split_a<float>(const float *, int64_t, int64_t, int64_t, __half *, const Layout &, int64_t, cudaStream_t,
                            const float *);
template int split_a<int32_t>(const int32_t *, int64_t, int64_t, int64_t, __half *, const Layout &, int64_t,
                              cudaStream_t, const int32_t *);
template int split_b<double>(const double *, int64_t, int64_t, int64_t, __half *, const Layout &, int64_t,
                             cudaStream_t, const double *);
template int split_b<float>(const float *, int64_t, int64_t, int64_t, __half *, const Layout &, int64_t, cudaStream_t,
                            const float *);
template int split_b<int32_t>(const int32_t *, int64_t, int64_t, int64_t, __half *, const Layout &, int64_t,
                              cudaStream_t, const int32_t *);

}  // namespace kara
