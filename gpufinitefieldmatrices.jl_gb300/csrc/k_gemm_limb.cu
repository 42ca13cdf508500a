// k_gemm_limb.cu -- host side of the limb tensor-core GEMM (gemm_limb.cuh):
// argument checks, workspace layout, TMA descriptors and launches.
#include "gemm_limb.cuh"
#include "kara_host.h"
#include "limb_host.h"
#include "limb_launch.cuh"

#include <cudaTypedefs.h>
#include <algorithm>
#include <mutex>
#include <vector>

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

int encode_digit_map(void *map, const void *base, int64_t kpad, int64_t rows, int box_rows) {
    int st = get_encoder();
    if (st) return st;
    return make_map(static_cast<CUtensorMap *>(map), base, kpad, rows, box_rows);
}

int encode_digit_map_k32(void *map, const void *base, int64_t rows, int box_rows) {
    int st = get_encoder();
    if (st) return st;
    cuuint64_t dims[2] = {32, (cuuint64_t)rows};
    cuuint64_t strides[1] = {64};
    cuuint32_t box[2] = {32, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = g_encode(static_cast<CUtensorMap *>(map), CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<void *>(base),
                          dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
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

int limbs_for_bits(int64_t N, int bits) {
    if (bits != 8) return limbs_for(N);
    // largest centred residue floor(N/2) within 127 * (256^L - 1) / 255
    if (N <= 255) return 1;
    if (N <= 65279) return 2;
    if (N <= 16711423) return 3;
    return 4;
}

int chunk_kblocks(const Layout &g) {
    // |d_i d_j| <= 2^(2 bits - 2) and at most L products per shift and k: the fp32 sums stay
    // exact (<= 2^24) over 2^(26 - 2 bits) / L values of k
    return g.bits == 8 ? std::max(1, 16 / g.L) : 64 / g.L;
}

void fast_consts(int64_t N, int L, int bits, bool paired, uint32_t *ninv, int32_t *Wm, int64_t *fbias) {
    uint32_t inv = 1;                         // N^-1 mod 2^32 by Newton's iteration
    for (int it = 0; it < 5; it++) inv *= 2u - (uint32_t)N * inv;
    *ninv = 0u - inv;
    int64_t w = 1 % N;
    for (int s = 0; s < MAX_SHIFTS; s++) {
        Wm[s] = (int32_t)(((__int128)w << 32) % N);
        w = (w << bits) % N;
    }
    const int nshift = 2 * L - 1;
    if (paired && bits == 7) {
        // pairs (0, 1), (2, 3), ... read as C_s + 2^7 C_{s+1} + FAST_PAIR_OFFSET with weight
        // Wm[s], the last shift alone as C + FAST_MAGIC_BITS.  The sum of the L terms is
        // within +-2^30.6 N, so the bias N 2^31 keeps x in (0, 2^32 N).
        int64_t b = N * (int64_t(1) << 31);
        for (int s = 0; s + 1 < nshift; s += 2) b -= (int64_t)FAST_PAIR_OFFSET * Wm[s];
        *fbias = b - (int64_t)FAST_MAGIC_BITS * Wm[nshift - 1];
    } else {
        // one shift at a time: each read as C + FAST_MAGIC_BITS; the sum is within
        // +-7 2^22 N, so the bias N 2^25 keeps x in (0, 2^26 N)
        int64_t wsum = 0;
        for (int s = 0; s < nshift; s++) wsum += Wm[s];
        *fbias = N * (int64_t(1) << 25) - (int64_t)FAST_MAGIC_BITS * wsum;
    }
}

Layout layout_bits(int64_t m, int64_t n, int64_t k, int64_t N, int bits) {
    Layout g = layout_L(m, n, k, limbs_for_bits(N, bits));
    g.bits = bits == 8 ? 8 : 7;
    return g;
}

int raw_limbs_for(int64_t N) {
    // largest non-centred residue N - 1 must fit L balanced base-128 digits
    if (N <= 64) return 1;
    if (N <= 8128) return 2;
    if (N <= 1040320) return 3;
    return 4;
}

Layout layout_L(int64_t m, int64_t n, int64_t k, int L) {
    Layout g;
    g.L = L;
    g.Mpad = gffm::round_up(m > 0 ? m : 1, BM);
    g.Npad = gffm::round_up(n > 0 ? n : 1, BN);
    g.Kpad = gffm::round_up(k > 0 ? k : 1, BK);
    g.a_bytes = (size_t)g.L * g.Mpad * g.Kpad * 2;
    g.b_bytes = (size_t)g.L * g.Npad * g.Kpad * 2;
    return g;
}

Layout layout(int64_t m, int64_t n, int64_t k, int64_t N) { return layout_L(m, n, k, limbs_for(N)); }

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

template <typename T, int MODE>
static void launch_split_a(const T *A, const T *A2, int64_t lda, int64_t m, int64_t k, __half *D, const Layout &g,
                           ModN M, cudaStream_t s) {
    dim3 grid((unsigned)(g.Kpad / 32), (unsigned)(g.Mpad / 32));
    const int mm = (int)m, kk = (int)k, Mp = (int)g.Mpad, Kp = (int)g.Kpad;
    switch (g.L) {
        case 1: k_split_a<T, 1, MODE><<<grid, 256, 0, s>>>(A, A2, lda, mm, kk, D, Mp, Kp, M, g.bits); break;
        case 2: k_split_a<T, 2, MODE><<<grid, 256, 0, s>>>(A, A2, lda, mm, kk, D, Mp, Kp, M, g.bits); break;
        case 3: k_split_a<T, 3, MODE><<<grid, 256, 0, s>>>(A, A2, lda, mm, kk, D, Mp, Kp, M, g.bits); break;
        default: k_split_a<T, 4, MODE><<<grid, 256, 0, s>>>(A, A2, lda, mm, kk, D, Mp, Kp, M, g.bits); break;
    }
}

template <typename T, int MODE>
static void launch_split_b(const T *B, const T *B2, int64_t ldb, int64_t k, int64_t n, __half *D, const Layout &g,
                           ModN M, cudaStream_t s) {
    int64_t total = (g.Kpad / 2) * g.Npad;
    unsigned blocks = (unsigned)((total + 255) / 256);
    const int kk = (int)k, nn = (int)n, Np = (int)g.Npad, Kp = (int)g.Kpad;
    switch (g.L) {
        case 1: k_split_b<T, 1, MODE><<<blocks, 256, 0, s>>>(B, B2, ldb, kk, nn, D, Np, Kp, M, g.bits); break;
        case 2: k_split_b<T, 2, MODE><<<blocks, 256, 0, s>>>(B, B2, ldb, kk, nn, D, Np, Kp, M, g.bits); break;
        case 3: k_split_b<T, 3, MODE><<<blocks, 256, 0, s>>>(B, B2, ldb, kk, nn, D, Np, Kp, M, g.bits); break;
        default: k_split_b<T, 4, MODE><<<blocks, 256, 0, s>>>(B, B2, ldb, kk, nn, D, Np, Kp, M, g.bits); break;
    }
}

// the raw and summed splits serve the Karatsuba products, which take Float64 digits only
static int check_mode(int mode, bool is_double, const void *second, int bits) {
    if (mode == SPLIT_CENTRED) return GFFM_OK;
    if (bits != 7) return gffm::set_error(GFFM_ERR_UNSUPPORTED, "raw and summed digit splits use 7-bit digits");
    if (!is_double || (mode != SPLIT_RAW && mode != SPLIT_SUM))
        return gffm::set_error(GFFM_ERR_UNSUPPORTED, "digit split mode %d is not available for this element type", mode);
    if (mode == SPLIT_SUM && !second) return gffm::set_error(GFFM_ERR_ARG, "summed digit split without a second operand");
    return GFFM_OK;
}

template <typename T>
int split_a(const T *A, int64_t lda, int64_t m, int64_t k, __half *D, const Layout &g, int64_t N, cudaStream_t s,
            int mode, const T *A2) {
    int st = check_mode(mode, sizeof(T) == 8, A2, g.bits);
    if (st) return st;
    ModN M{N, ~uint64_t(0) / (uint64_t)N};
    if constexpr (sizeof(T) == 8) {
        if (mode == SPLIT_RAW)
            launch_split_a<T, SPLIT_RAW>(A, A2, lda, m, k, D, g, M, s);
        else if (mode == SPLIT_SUM)
            launch_split_a<T, SPLIT_SUM>(A, A2, lda, m, k, D, g, M, s);
        else
            launch_split_a<T, SPLIT_CENTRED>(A, A2, lda, m, k, D, g, M, s);
    } else {
        launch_split_a<T, SPLIT_CENTRED>(A, A2, lda, m, k, D, g, M, s);
    }
    GFFM_LAUNCH_CHECK("k_split_a");
    return GFFM_OK;
}

template <typename T>
int split_b(const T *B, int64_t ldb, int64_t k, int64_t n, __half *D, const Layout &g, int64_t N, cudaStream_t s,
            int mode, const T *B2) {
    int st = check_mode(mode, sizeof(T) == 8, B2, g.bits);
    if (st) return st;
    ModN M{N, ~uint64_t(0) / (uint64_t)N};
    if constexpr (sizeof(T) == 8) {
        if (mode == SPLIT_RAW)
            launch_split_b<T, SPLIT_RAW>(B, B2, ldb, k, n, D, g, M, s);
        else if (mode == SPLIT_SUM)
            launch_split_b<T, SPLIT_SUM>(B, B2, ldb, k, n, D, g, M, s);
        else
            launch_split_b<T, SPLIT_CENTRED>(B, B2, ldb, k, n, D, g, M, s);
    } else {
        launch_split_b<T, SPLIT_CENTRED>(B, B2, ldb, k, n, D, g, M, s);
    }
    GFFM_LAUNCH_CHECK("k_split_b");
    return GFFM_OK;
}

template <int EPI>
static int launch_gemm(int L, const CUtensorMap &ta, const CUtensorMap &tb, const Params &p, int grid, cudaStream_t s) {
    switch (L) {
        case 1: return launch_gemm_L<1, EPI, 64>(ta, tb, p, grid, s);
        case 2: return launch_gemm_L<2, EPI, 64>(ta, tb, p, grid, s);
        case 3: return launch_gemm_L<3, EPI, 64>(ta, tb, p, grid, s);
        default: return launch_gemm_L<4, EPI, 64>(ta, tb, p, grid, s);
    }
}


int gemm_digits(const Layout &g, const __half *Ad, const __half *Bd, int64_t m, int64_t n, int64_t k, int64_t N,
                void *C, int64_t ldc, int epi, int max_ctas, cudaStream_t s, const double *X, const double *Y,
                int *tile_counter) {
    if (epi == EPI_KSUB_F64 && (!X || !Y)) return gffm::set_error(GFFM_ERR_ARG, "subtracting epilogue without X, Y");
    if (N < 2 || N >= (epi == EPI_EXACT_I64 ? (int64_t(1) << 52) : (int64_t(1) << 26)))
        return gffm::set_error(GFFM_ERR_MODULUS, "modulus %lld out of range for epilogue %d", (long long)N, epi);
    if (epi == EPI_EXACT_I64 && g.bits != 7)
        return gffm::set_error(GFFM_ERR_UNSUPPORTED, "the exact epilogue takes 7-bit digits");
    int st = get_encoder();
    if (st) return st;
    CUtensorMap ta, tb;
    st = make_map(&ta, Ad, g.Kpad, (int64_t)g.L * g.Mpad, BM);
    if (st) return st;
    // 64-column tiles (one accumulator set) unless the tuning asks for 32-column tiles with
    // two accumulator sets; measured on GB300 the 64-column tile wins at every K tried (the
    // narrower tile doubles the A-operand traffic per output), so 32 is a tuner candidate only
    const int bnv = g.bn == 32 ? 32 : 64;
    st = make_map(&tb, Bd, g.Kpad, (int64_t)g.L * g.Npad, bnv);
    if (st) return st;
    Params p;
    p.m = (int)m;
    p.n = (int)n;
    p.kblocks = (int)(k > 0 ? gffm::round_up(k, BK) / BK : 0);
    p.Mpad = (int)g.Mpad;
    p.Npad = (int)g.Npad;
    p.mtiles = (int)((m + BM - 1) / BM);
    p.ntiles = (int)((n + bnv - 1) / bnv);
    p.chunk_kb = chunk_kblocks(g);
    p.N = N;
    p.minv = ~uint64_t(0) / (uint64_t)N;
    p.bias = N * (((int64_t(1) << 60) + N - 1) / N);
    int64_t w = 1 % N;
    for (int sft = 0; sft < MAX_SHIFTS; sft++) {
        p.W[sft] = (int32_t)w;      // unused by EPI_EXACT_I64, whose N may exceed 32 bits
        w = (int64_t)(((__int128)w * (g.bits == 8 ? 256 : 128)) % N);
    }
    // the read-modify-write fast path: odd N, one exact chunk, shift sums within 2^22, 7-bit
    // digits (its drain reads the shifts in pairs)
    if (epi == EPI_SUB_I32 && (N & 1) && g.bits == 7 && p.kblocks <= p.chunk_kb &&
        (int64_t)p.kblocks * BK * g.L * (int64_t(1) << (2 * g.bits - 2)) <= (int64_t(1) << 22)) {
        fast_consts(N, g.L, g.bits, true, &p.ninv, p.Wm, &p.fbias);
        epi = EPI_SUB_I32M;
    }
    p.C = C;
    p.ldc = ldc;
    p.X = X;
    p.Y = Y;
    p.err = gffm::device_error_flag();
    p.tile_counter = tile_counter;
    if (!p.err) return gffm::check_device();
    int ntiles = p.mtiles * p.ntiles;
    if (ntiles == 0) return GFFM_OK;
    int grid = gffm::sm_count();
    if (max_ctas > 0 && grid > max_ctas) grid = max_ctas;
    if (grid > ntiles) grid = ntiles;
    if (bnv == 32) return launch_gemm_short(epi, g.L, ta, tb, p, grid, s);
    switch (epi) {
        case EPI_STORE_F64: return launch_gemm<EPI_STORE_F64>(g.L, ta, tb, p, grid, s);
        case EPI_STORE_F32: return launch_gemm<EPI_STORE_F32>(g.L, ta, tb, p, grid, s);
        case EPI_STORE_I32: return launch_gemm<EPI_STORE_I32>(g.L, ta, tb, p, grid, s);
        case EPI_EXACT_I64: return launch_gemm<EPI_EXACT_I64>(g.L, ta, tb, p, grid, s);
        case EPI_KSUB_F64: return launch_gemm<EPI_KSUB_F64>(g.L, ta, tb, p, grid, s);
        case EPI_SUB_I32M: return launch_gemm<EPI_SUB_I32M>(g.L, ta, tb, p, grid, s);
        default: return launch_gemm<EPI_SUB_I32>(g.L, ta, tb, p, grid, s);
    }
}

template int split_a<double>(const double *, int64_t, int64_t, int64_t, __half *, const Layout &, int64_t, cudaStream_t,
                            int, const double *);
template int split_a<float>(const float *, int64_t, int64_t, int64_t, __half *, const Layout &, int64_t, cudaStream_t,
                            int, const float *);
template int split_a<int32_t>(const int32_t *, int64_t, int64_t, int64_t, __half *, const Layout &, int64_t, cudaStream_t,
                            int, const int32_t *);
template int split_b<double>(const double *, int64_t, int64_t, int64_t, __half *, const Layout &, int64_t, cudaStream_t,
                            int, const double *);
template int split_b<float>(const float *, int64_t, int64_t, int64_t, __half *, const Layout &, int64_t, cudaStream_t,
                            int, const float *);
template int split_b<int32_t>(const int32_t *, int64_t, int64_t, int64_t, __half *, const Layout &, int64_t, cudaStream_t,
                            int, const int32_t *);

}  // namespace limb

namespace limb {

// The process-wide tune table (the one piece of global mutable state: written by
// gffm_tune_table_set, read by every limb product).
static std::vector<gffm_tune_entry> g_tune;
static std::mutex g_tune_mu;

void tuned_for(int64_t m, int64_t n, int64_t k, int64_t N, int *bits, int *max_ctas, int *tile_n, int *form) {
    *bits = 7;
    *max_ctas = 0;
    *tile_n = 64;
    *form = FORM_DEFAULT;
    const double work = (double)m * (double)n * (double)k;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    for (const gffm_tune_entry &e : g_tune) {
        if (N < e.N_lo || N > e.N_hi || work < e.work_lo || work > e.work_hi) continue;
        *bits = e.tuning.digit_bits == 8 ? 8 : 7;
        *max_ctas = e.tuning.max_ctas > 0 ? e.tuning.max_ctas : 0;
        *tile_n = e.tuning.tile_n == 32 ? 32 : 64;
        *form = e.tuning.form;
        return;
    }
}

int resolve_form(int form, int bits, int tile_n, int64_t N, int64_t k) {
    if (form == FORM_SCHOOLBOOK || form == FORM_KARATSUBA) return form;
    // the default: Karatsuba for four 7-bit digits once the products are long enough to
    // amortise its three per-product accumulator drains, unless the schoolbook's 8-bit
    // digits or 32-column tiles were asked for
    return (bits == 7 && tile_n != 32 && kara::applies(N) && k >= KARA_MIN_K) ? FORM_KARATSUBA : FORM_SCHOOLBOOK;
}

}  // namespace limb

namespace {

int check_tuning(const gffm_limb_tuning *t) {
    if (!t) return GFFM_OK;
    if (t->form < 0 || t->form > 2) return gffm::set_error(GFFM_ERR_ARG, "form must be 0, 1 or 2");
    if (t->digit_bits != 0 && t->digit_bits != 7 && t->digit_bits != 8)
        return gffm::set_error(GFFM_ERR_ARG, "digit_bits must be 0, 7 or 8");
    if (t->max_ctas < 0) return gffm::set_error(GFFM_ERR_ARG, "max_ctas must be >= 0");
    if (t->tile_n != 0 && t->tile_n != 32 && t->tile_n != 64)
        return gffm::set_error(GFFM_ERR_ARG, "tile_n must be 0, 32 or 64");
    return GFFM_OK;
}

// the digit width, grid, tile width and product form of a product: an explicit tuning, else
// the tune table; an explicit Karatsuba form must fit the modulus
int pick(const gffm_limb_tuning *t, int64_t m, int64_t n, int64_t k, int64_t N, int *bits, int *ctas, int *tile_n,
         int *form) {
    limb::tuned_for(m, n, k, N, bits, ctas, tile_n, form);
    if (t) {
        if (t->digit_bits) *bits = t->digit_bits;
        *ctas = t->max_ctas;
        if (t->tile_n) *tile_n = t->tile_n;
        if (t->form) *form = t->form;
        if (t->form == limb::FORM_KARATSUBA && !kara::applies(N))
            return gffm::set_error(GFFM_ERR_UNSUPPORTED, "the Karatsuba form needs 2080639 < N < 2^26 (got %lld)",
                                   (long long)N);
    }
    if (*form == limb::FORM_KARATSUBA && !kara::applies(N)) *form = limb::FORM_SCHOOLBOOK;   // a table range
    *form = limb::resolve_form(*form, *bits, *tile_n, N, k);
    return GFFM_OK;
}

// scratch bytes of a product in the chosen form
size_t scratch_bytes(int64_t m, int64_t n, int64_t k, int64_t N, int bits, int form) {
    if (form == limb::FORM_KARATSUBA) {
        kara::Layout g = kara::layout(m, n, k);
        return g.a_bytes + g.b_bytes;
    }
    limb::Layout g = limb::layout_bits(m, n, k, N, bits);
    return g.a_bytes + g.b_bytes;
}

template <typename T>
int matmul_limb(int64_t m, int64_t n, int64_t k, const T *A, int64_t lda, const T *B, int64_t ldb, T *C, int64_t ldc,
                int64_t N, void *ws, size_t ws_bytes, gffm_stream_t stream, const gffm_limb_tuning *tune = nullptr) {
    using namespace gffm;
    int st = check_tuning(tune);
    if (st) return st;
    st = limb::check_args(m, n, k, lda, ldb, ldc, N);
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
    int bits, ctas, tile_n, form;
    st = pick(tune, m, n, k, N, &bits, &ctas, &tile_n, &form);
    if (st) return st;
    const int epi = sizeof(T) == 8 ? limb::EPI_STORE_F64 : limb::EPI_STORE_F32;
    Scratch scr;
    if (form == limb::FORM_KARATSUBA) {
        kara::Layout kg = kara::layout(m, n, k);
        st = scr.acquire(ws, ws_bytes, kg.a_bytes + kg.b_bytes, s);
        if (st) return st;
        __half *Ad = static_cast<__half *>(scr.ptr);
        __half *Bd = reinterpret_cast<__half *>(static_cast<uint8_t *>(scr.ptr) + kg.a_bytes);
        st = kara::split_a<T>(A, lda, m, k, Ad, kg, N, s);
        if (st) return st;
        st = kara::split_b<T>(B, ldb, k, n, Bd, kg, N, s);
        if (st) return st;
        return kara::gemm_digits(kg, Ad, Bd, m, n, k, N, C, ldc, epi, ctas, s);
    }
    limb::Layout g = limb::layout_bits(m, n, k, N, bits);
    g.bn = tile_n;
    st = scr.acquire(ws, ws_bytes, g.a_bytes + g.b_bytes, s);
    if (st) return st;
    __half *Ad = static_cast<__half *>(scr.ptr);
    __half *Bd = reinterpret_cast<__half *>(static_cast<uint8_t *>(scr.ptr) + g.a_bytes);
    st = limb::split_a<T>(A, lda, m, k, Ad, g, N, s);
    if (st) return st;
    st = limb::split_b<T>(B, ldb, k, n, Bd, g, N, s);
    if (st) return st;
    return limb::gemm_digits(g, Ad, Bd, m, n, k, N, C, ldc, epi, ctas, s);
}

}  // namespace

extern "C" {

int gffm_matmul_limb_tuned_workspace_size(int64_t m, int64_t n, int64_t k, int64_t N, const gffm_limb_tuning *tuning,
                                          size_t *bytes) {
    if (!bytes) return gffm::set_error(GFFM_ERR_ARG, "bytes is NULL");
    int st = check_tuning(tuning);
    if (st) return st;
    st = limb::check_args(m, n, k, m > 1 ? m : 1, k > 1 ? k : 1, m > 1 ? m : 1, N);
    if (st) return st;
    int bits, ctas, tile_n, form;
    st = pick(tuning, m, n, k, N, &bits, &ctas, &tile_n, &form);
    if (st) return st;
    *bytes = (m == 0 || n == 0 || k == 0) ? 0 : scratch_bytes(m, n, k, N, bits, form);
    return GFFM_OK;
}

int gffm_matmul_limb_workspace_size(int64_t m, int64_t n, int64_t k, int64_t N, size_t *bytes) {
    return gffm_matmul_limb_tuned_workspace_size(m, n, k, N, nullptr, bytes);
}

int gffm_matmul_limb_tuned_f64(int64_t m, int64_t n, int64_t k, const double *A, int64_t lda, const double *B,
                               int64_t ldb, double *C, int64_t ldc, int64_t N, const gffm_limb_tuning *tuning, void *ws,
                               size_t ws_bytes, gffm_stream_t s) {
    if (!tuning) return gffm::set_error(GFFM_ERR_ARG, "tuning is NULL");
    return matmul_limb<double>(m, n, k, A, lda, B, ldb, C, ldc, N, ws, ws_bytes, s, tuning);
}

int gffm_tune_table_set(const gffm_tune_entry *entries, int64_t count) {
    if (count < 0 || (count > 0 && !entries)) return gffm::set_error(GFFM_ERR_ARG, "bad tune table");
    for (int64_t i = 0; i < count; i++) {
        int st = check_tuning(&entries[i].tuning);
        if (st) return st;
    }
    std::lock_guard<std::mutex> lk(limb::g_tune_mu);
    limb::g_tune.assign(entries, entries + count);
    return GFFM_OK;
}

int gffm_tune_table_size(int64_t *count) {
    if (!count) return gffm::set_error(GFFM_ERR_ARG, "count is NULL");
    std::lock_guard<std::mutex> lk(limb::g_tune_mu);
    *count = (int64_t)limb::g_tune.size();
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
