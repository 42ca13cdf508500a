// k_karatsuba.cu -- KaratsubaArray arithmetic (src/KaratsubaMatrix/KaratsubaMatrix.jl,
// src/KaratsubaMatrix/KaratsubaKernels.jl).
//
// An element is two digits (d1, d2), d1 in [0, N1), d2 in [0, N2), of the value
// x = d1 + N1*d2 in Z/(N1*N2) (KaratsubaMatrix.jl:304,318-336).
//
// Product (KMatMul!, KaratsubaMatrix.jl:133-204).  With x = a1 + N1 a2, y = b1 + N1 b2 and
//     S1 = sum a1 b1 (exact integer),  S2 = sum (a1 + a2)(b1 + b2),  S3 = sum a2 b2
// the three component products of the reference (nKMuls = 3, :211) give
//     sum x y = S1 + N1 (S2 - S1 - S3) + N1^2 S3,
// so with S1' = S1 mod N1*N2:
//     c1 = S1' mod N1,
//     c2 = (floor(S1' / N1) + S2 - S1 + (N1 - 1) S3) mod N2.
// S2 and S3 are only needed mod N2 and run on the limb GEMM mod N2; S1' runs on
// the same GEMM with non-centred digits and the exact epilogue modulo N1*N2.
// karatsuba_matmul_kernel_2! (KaratsubaKernels.jl:141-158) evaluates the same
// expression with S1 mod N1^2 and without the N1*S3 term; both coincide with
// this exact product when N2 divides N1 (every modulus pair the reference
// builds: MatToKMat uses N1 = N2, its tests use 13^4, 13^3 and 100, 100).
//
// Polynomial form (the two-component reading of the same three products):
// (A0 + A1 x)(B0 + B1 x) mod p = C0 + C1 x + C2 x^2 with
//     C0 = A0 B0,  C2 = A1 B1,  C1 = (A0 + A1)(B0 + B1) - C0 - C2,
// the last product fused with its subtraction in the GEMM epilogue.
//
// Elementwise digit ops (karatsuba_add_kernel!, karatsuba_sub_kernel!,
// karatsuba_negate_kernel!, karatsuba_scalar_multiply_kernel!,
// KaratsubaKernels.jl:2-125) work on the value x exactly: one HBM pass, the
// digits recovered with a Barrett quotient by N1.
#include "gffm_common.cuh"
#include "kara_host.h"
#include "limb_host.h"

namespace {

using gffm::set_error;

struct KMod {
    uint64_t n1, n2, m;        // N1, N2, N1*N2
    uint64_t minv1, minv2, minvm;
    uint64_t n1m1_mod_n2;      // (N1 - 1) mod N2
};

__device__ __forceinline__ uint64_t red(uint64_t x, uint64_t n, uint64_t minv) {
    // x < 2^63
    return gffm_dev::barrett64(x, n, minv);
}

// quotient and remainder of x < 2^63 by n
__device__ __forceinline__ uint64_t divrem(uint64_t x, uint64_t n, uint64_t minv, uint64_t &r) {
    uint64_t q = __umul64hi(x, minv);
    r = x - q * n;
    if (r >= n) {
        r -= n;
        q++;
    }
    return q;
}

__device__ __forceinline__ uint64_t to_u(double v, uint64_t n, uint64_t minv) {
    // digits are integer-valued; negative or oversized digits are reduced mod n
    const int64_t x = (int64_t)v;
    if (x >= 0) return (uint64_t)x < n ? (uint64_t)x : red((uint64_t)x, n, minv);
    const uint64_t r = red((uint64_t)(-x), n, minv);
    return r ? n - r : 0;
}

// ---------------------------------------------------------------------------
// digit-form combine: (S1' int64, S2 in C2, S3 in C1) -> (c1, c2)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_kara_combine(double *__restrict__ C1, double *__restrict__ C2, int64_t ldc,
                                                      const int64_t *__restrict__ S1, int64_t lds, int m, int n,
                                                      int row_blocks, KMod K) {
    const int64_t j = blockIdx.x / row_blocks;
    const int64_t i = (int64_t)(blockIdx.x - j * row_blocks) * blockDim.x + threadIdx.x;
    if (i >= m || j >= n) return;
    const int64_t off = i + j * ldc;
    const uint64_t s1 = (uint64_t)S1[i + j * lds];
    const uint64_t s2 = (uint64_t)C2[off];
    const uint64_t s3 = (uint64_t)C1[off];
    uint64_t c1;
    const uint64_t q = divrem(s1, K.n1, K.minv1, c1);          // q < N2
    const uint64_t s1m = red(s1, K.n2, K.minv2);
    const uint64_t t = red(K.n1m1_mod_n2 * s3, K.n2, K.minv2);  // < 2^52
    const uint64_t c2 = red(q + s2 + (K.n2 - s1m) + t, K.n2, K.minv2);
    C1[off] = (double)c1;
    C2[off] = (double)c2;
}

// ---------------------------------------------------------------------------
// elementwise digit ops on x = d1 + N1 d2
// ---------------------------------------------------------------------------
enum KOp { K_ADD, K_SUB, K_NEG, K_SMUL, K_FROM, K_TO };

template <int OP>
__global__ void __launch_bounds__(256) k_kara_elementwise(double *__restrict__ C1, double *__restrict__ C2,
                                                          const double *__restrict__ A1, const double *__restrict__ A2,
                                                          const double *__restrict__ B1, const double *__restrict__ B2,
                                                          uint64_t s, int64_t len, KMod K) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (; i < len; i += stride) {
        if (OP == K_FROM) {
            // MatToKMat: value A1[i] (a non-negative integer) -> digits of its class mod N1*N2
            const uint64_t v = to_u(A1[i], K.m, K.minvm);
            uint64_t d1;
            const uint64_t d2 = divrem(v, K.n1, K.minv1, d1);
            C1[i] = (double)d1;
            C2[i] = (double)d2;
            continue;
        }
        const uint64_t x = to_u(A1[i], K.n1, K.minv1) + K.n1 * to_u(A2[i], K.n2, K.minv2);   // < N1 N2
        if (OP == K_TO) {
            C1[i] = (double)x;   // N1 N2 <= 2^52: exact
            continue;
        }
        uint64_t r;
        if (OP == K_ADD || OP == K_SUB) {
            const uint64_t y = to_u(B1[i], K.n1, K.minv1) + K.n1 * to_u(B2[i], K.n2, K.minv2);
            if (OP == K_ADD) {
                r = x + y;
                if (r >= K.m) r -= K.m;
            } else {
                r = x >= y ? x - y : x + (K.m - y);
            }
        } else if (OP == K_NEG) {
            r = x ? K.m - x : 0;
        } else {
            r = (uint64_t)(((unsigned __int128)x * s) % K.m);
        }
        uint64_t d1;
        const uint64_t d2 = divrem(r, K.n1, K.minv1, d1);
        C1[i] = (double)d1;
        C2[i] = (double)d2;
    }
}

int check_moduli(int64_t N1, int64_t N2, bool matmul) {
    if (N1 < 2 || N2 < 2) return set_error(GFFM_ERR_MODULUS, "Karatsuba moduli must be >= 2 (got %lld, %lld)",
                                           (long long)N1, (long long)N2);
    if (matmul) {
        if (N1 >= (int64_t(1) << 26) || N2 >= (int64_t(1) << 26))
            return set_error(GFFM_ERR_MODULUS, "the Karatsuba product needs N1, N2 < 2^26 (got %lld, %lld)",
                             (long long)N1, (long long)N2);
    } else if ((__int128)N1 * N2 > ((__int128)1 << 52)) {
        return set_error(GFFM_ERR_MODULUS, "N1*N2 must be at most 2^52 (got %lld * %lld)", (long long)N1,
                         (long long)N2);
    }
    return GFFM_OK;
}

KMod make_kmod(int64_t N1, int64_t N2) {
    KMod K;
    K.n1 = (uint64_t)N1;
    K.n2 = (uint64_t)N2;
    K.m = (uint64_t)N1 * (uint64_t)N2;
    K.minv1 = ~uint64_t(0) / K.n1;
    K.minv2 = ~uint64_t(0) / K.n2;
    K.minvm = ~uint64_t(0) / K.m;
    K.n1m1_mod_n2 = (K.n1 - 1) % K.n2;
    return K;
}

template <int OP>
int elementwise(double *C1, double *C2, const double *A1, const double *A2, const double *B1, const double *B2,
                int64_t s, int64_t len, int64_t N1, int64_t N2, gffm_stream_t stream) {
    int st = check_moduli(N1, N2, false);
    if (st) return st;
    if (len < 0) return set_error(GFFM_ERR_ARG, "negative length");
    if (len == 0) return GFFM_OK;
    const bool needs_b = OP == K_ADD || OP == K_SUB;
    const bool needs_a2 = OP != K_FROM;
    const bool needs_c2 = OP != K_TO;
    if (!C1 || !A1 || (needs_a2 && !A2) || (needs_b && (!B1 || !B2)) || (needs_c2 && !C2))
        return set_error(GFFM_ERR_ARG, "null data pointer");
    st = gffm::check_device();
    if (st) return st;
    KMod K = make_kmod(N1, N2);
    int64_t sm = s % (int64_t)K.m;
    if (sm < 0) sm += (int64_t)K.m;
    int64_t blocks = (len + 255) / 256;
    const int64_t cap = (int64_t)gffm::sm_count() * 16;
    if (blocks > cap) blocks = cap;
    k_kara_elementwise<OP><<<(unsigned)blocks, 256, 0, gffm::as_stream(stream)>>>(C1, C2, A1, A2, B1, B2, (uint64_t)sm,
                                                                                 len, K);
    GFFM_LAUNCH_CHECK("k_kara_elementwise");
    return GFFM_OK;
}

bool overlaps(const void *a, const void *b) { return a && b && a == b; }

int check_mm(int64_t m, int64_t n, int64_t k, int64_t lda, int64_t ldb, int64_t ldc) {
    if (m < 0 || n < 0 || k < 0) return set_error(GFFM_ERR_ARG, "negative matrix size");
    if (lda < (m > 1 ? m : 1) || ldb < (k > 1 ? k : 1) || ldc < (m > 1 ? m : 1))
        return set_error(GFFM_ERR_ARG, "leading dimension smaller than the number of rows");
    if (m > (int64_t(1) << 24) || n > (int64_t(1) << 24) || k > (int64_t(1) << 24))
        return set_error(GFFM_ERR_ARG, "matrix dimension above 2^24");
    return GFFM_OK;
}

// The products mod a single modulus below 2^26 take the limb GEMM's Karatsuba digit form
// (kara_host.h) where it applies, as gffm_matmul_limb_f64 does by default.
bool kara_form(int64_t N, int64_t k) {
    return limb::resolve_form(limb::FORM_DEFAULT, 7, 64, N, k) == limb::FORM_KARATSUBA;
}

struct KaraLayout {
    limb::Layout exact, modn2;
    kara::Layout kmodn2;
    bool kform = false;   // the mod-N2 products in the Karatsuba digit form
    size_t da, db, s1;    // digit buffers for A and B, the int64 S1' matrix
    size_t total() const { return da + db + s1; }
};

KaraLayout kara_layout(int64_t m, int64_t n, int64_t k, int64_t N1, int64_t N2) {
    KaraLayout kl;
    kl.exact = limb::layout_L(m, n, k, limb::raw_limbs_for(N1));
    kl.modn2 = limb::layout(m, n, k, N2);
    kl.kmodn2 = kara::layout(m, n, k);
    kl.kform = N2 < (int64_t(1) << 26) && kara_form(N2, k);
    const size_t a2 = kl.kform ? kl.kmodn2.a_bytes : kl.modn2.a_bytes;
    const size_t b2 = kl.kform ? kl.kmodn2.b_bytes : kl.modn2.b_bytes;
    kl.da = gffm::round_up((int64_t)(kl.exact.a_bytes > a2 ? kl.exact.a_bytes : a2), 256);
    kl.db = gffm::round_up((int64_t)(kl.exact.b_bytes > b2 ? kl.exact.b_bytes : b2), 256);
    kl.s1 = (size_t)(m > 0 ? m : 1) * (size_t)(n > 0 ? n : 1) * 8;
    return kl;
}

// C (ldc) = A B mod N (Float64), A = the residues of X, or of (X + X2) mod N with X2; the
// digit planes in dA / dB; the Karatsuba digit form when `kform`
int product(bool kform, const limb::Layout &g, const kara::Layout &kg, const double *X, const double *X2,
            int64_t lda, const double *Y, const double *Y2, int64_t ldb, int64_t m, int64_t n, int64_t k, int64_t N,
            __half *dA, __half *dB, double *C, int64_t ldc, int epi, cudaStream_t s, const double *S0 = nullptr,
            const double *S2 = nullptr) {
    int st;
    if (kform) {
        st = kara::split_a<double>(X, lda, m, k, dA, kg, N, s, X2);
        if (!st) st = kara::split_b<double>(Y, ldb, k, n, dB, kg, N, s, Y2);
        if (!st) st = kara::gemm_digits(kg, dA, dB, m, n, k, N, C, ldc, epi, 0, s, S0, S2);
        return st;
    }
    const int mode = X2 ? limb::SPLIT_SUM : limb::SPLIT_CENTRED;
    st = limb::split_a<double>(X, lda, m, k, dA, g, N, s, mode, X2);
    if (!st) st = limb::split_b<double>(Y, ldb, k, n, dB, g, N, s, mode, Y2);
    if (!st) st = limb::gemm_digits(g, dA, dB, m, n, k, N, C, ldc, epi, 0, s, S0, S2);
    return st;
}

int kara_matmul(int64_t m, int64_t n, int64_t k, const double *A1, const double *A2, int64_t lda, const double *B1,
                const double *B2, int64_t ldb, double *C1, double *C2, int64_t ldc, int64_t N1, int64_t N2, void *ws,
                size_t ws_bytes, gffm_stream_t stream) {
    using namespace gffm;
    int st = check_moduli(N1, N2, true);
    if (st) return st;
    st = check_mm(m, n, k, lda, ldb, ldc);
    if (st) return st;
    if (m == 0 || n == 0) return GFFM_OK;
    if (!C1 || !C2 || (k > 0 && (!A1 || !A2 || !B1 || !B2))) return set_error(GFFM_ERR_ARG, "null data pointer");
    if (overlaps(C1, A1) || overlaps(C1, A2) || overlaps(C1, B1) || overlaps(C1, B2) || overlaps(C2, A1) ||
        overlaps(C2, A2) || overlaps(C2, B1) || overlaps(C2, B2) || overlaps(C1, C2))
        return set_error(GFFM_ERR_ARG, "the Karatsuba product cannot overwrite its operands");
    st = check_device();
    if (st) return st;
    cudaStream_t s = as_stream(stream);
    if (k == 0) {
        GFFM_CUDA(cudaMemset2DAsync(C1, (size_t)ldc * 8, 0, (size_t)m * 8, (size_t)n, s));
        GFFM_CUDA(cudaMemset2DAsync(C2, (size_t)ldc * 8, 0, (size_t)m * 8, (size_t)n, s));
        return GFFM_OK;
    }
    KaraLayout kl = kara_layout(m, n, k, N1, N2);
    Scratch scr;
    st = scr.acquire(ws, ws_bytes, kl.total(), s);
    if (st) return st;
    uint8_t *base = static_cast<uint8_t *>(scr.ptr);
    __half *dA = reinterpret_cast<__half *>(base);
    __half *dB = reinterpret_cast<__half *>(base + kl.da);
    int64_t *S1 = reinterpret_cast<int64_t *>(base + kl.da + kl.db);
    const int64_t M12 = N1 * N2;

    // S1' = A1 B1 mod N1 N2 from non-centred digits
    st = limb::split_a<double>(A1, lda, m, k, dA, kl.exact, N1, s, limb::SPLIT_RAW);
    if (!st) st = limb::split_b<double>(B1, ldb, k, n, dB, kl.exact, N1, s, limb::SPLIT_RAW);
    if (!st) st = limb::gemm_digits(kl.exact, dA, dB, m, n, k, M12, S1, m, limb::EPI_EXACT_I64, 0, s);
    // S2 = (A1 + A2)(B1 + B2) mod N2 -> C2
    if (!st)
        st = product(kl.kform, kl.modn2, kl.kmodn2, A1, A2, lda, B1, B2, ldb, m, n, k, N2, dA, dB, C2, ldc,
                     limb::EPI_STORE_F64, s);
    // S3 = A2 B2 mod N2 -> C1
    if (!st)
        st = product(kl.kform, kl.modn2, kl.kmodn2, A2, nullptr, lda, B2, nullptr, ldb, m, n, k, N2, dA, dB, C1, ldc,
                     limb::EPI_STORE_F64, s);
    if (st) return st;
    const int row_blocks = (int)((m + 255) / 256);
    k_kara_combine<<<(unsigned)(row_blocks * n), 256, 0, s>>>(C1, C2, ldc, S1, m, (int)m, (int)n, row_blocks,
                                                              make_kmod(N1, N2));
    GFFM_LAUNCH_CHECK("k_kara_combine");
    return GFFM_OK;
}

int poly_matmul(int64_t m, int64_t n, int64_t k, const double *A0, const double *A1, int64_t lda, const double *B0,
                const double *B1, int64_t ldb, double *C0, double *C1, double *C2, int64_t ldc, int64_t p, void *ws,
                size_t ws_bytes, gffm_stream_t stream) {
    using namespace gffm;
    int st = limb::check_args(m, n, k, lda, ldb, ldc, p);
    if (st) return st;
    if (m == 0 || n == 0) return GFFM_OK;
    if (!C0 || !C1 || !C2 || (k > 0 && (!A0 || !A1 || !B0 || !B1))) return set_error(GFFM_ERR_ARG, "null data pointer");
    const void *outs[3] = {C0, C1, C2};
    const void *ins[4] = {A0, A1, B0, B1};
    for (int a = 0; a < 3; a++) {
        for (int b = 0; b < 4; b++)
            if (overlaps(outs[a], ins[b])) return set_error(GFFM_ERR_ARG, "the Karatsuba product cannot overwrite its operands");
        for (int b = a + 1; b < 3; b++)
            if (overlaps(outs[a], outs[b])) return set_error(GFFM_ERR_ARG, "output components must be distinct");
    }
    st = check_device();
    if (st) return st;
    cudaStream_t s = as_stream(stream);
    if (k == 0) {
        for (double *C : {C0, C1, C2}) GFFM_CUDA(cudaMemset2DAsync(C, (size_t)ldc * 8, 0, (size_t)m * 8, (size_t)n, s));
        return GFFM_OK;
    }
    const limb::Layout g = limb::layout(m, n, k, p);
    const kara::Layout kg = kara::layout(m, n, k);
    const bool kform = kara_form(p, k);
    const size_t da = gffm::round_up((int64_t)(kform ? kg.a_bytes : g.a_bytes), 256);
    Scratch scr;
    st = scr.acquire(ws, ws_bytes, da + (kform ? kg.b_bytes : g.b_bytes), s);
    if (st) return st;
    __half *dA = static_cast<__half *>(scr.ptr);
    __half *dB = reinterpret_cast<__half *>(static_cast<uint8_t *>(scr.ptr) + da);
    st = product(kform, g, kg, A0, nullptr, lda, B0, nullptr, ldb, m, n, k, p, dA, dB, C0, ldc, limb::EPI_STORE_F64, s);
    if (!st)
        st = product(kform, g, kg, A1, nullptr, lda, B1, nullptr, ldb, m, n, k, p, dA, dB, C2, ldc, limb::EPI_STORE_F64,
                     s);
    if (!st)
        st = product(kform, g, kg, A0, A1, lda, B0, B1, ldb, m, n, k, p, dA, dB, C1, ldc, limb::EPI_KSUB_F64, s, C0,
                     C2);
    return st;
}

}  // namespace

extern "C" {

int gffm_karatsuba_workspace_size(int64_t m, int64_t n, int64_t k, int64_t N1, int64_t N2, size_t *bytes) {
    if (!bytes) return set_error(GFFM_ERR_ARG, "bytes is NULL");
    int st = check_moduli(N1, N2, true);
    if (st) return st;
    st = check_mm(m, n, k, m > 1 ? m : 1, k > 1 ? k : 1, m > 1 ? m : 1);
    if (st) return st;
    *bytes = (m == 0 || n == 0 || k == 0) ? 0 : kara_layout(m, n, k, N1, N2).total();
    return GFFM_OK;
}

int gffm_karatsuba_matmul_f64(int64_t m, int64_t n, int64_t k, const double *A1, const double *A2, int64_t lda,
                              const double *B1, const double *B2, int64_t ldb, double *C1, double *C2, int64_t ldc,
                              int64_t N1, int64_t N2, void *ws, size_t ws_bytes, gffm_stream_t stream) {
    return kara_matmul(m, n, k, A1, A2, lda, B1, B2, ldb, C1, C2, ldc, N1, N2, ws, ws_bytes, stream);
}

int gffm_karatsuba_poly_workspace_size(int64_t m, int64_t n, int64_t k, int64_t p, size_t *bytes) {
    if (!bytes) return set_error(GFFM_ERR_ARG, "bytes is NULL");
    int st = limb::check_args(m, n, k, m > 1 ? m : 1, k > 1 ? k : 1, m > 1 ? m : 1, p);
    if (st) return st;
    const limb::Layout g = limb::layout(m, n, k, p);
    const kara::Layout kg = kara::layout(m, n, k);
    const bool kform = kara_form(p, k);
    *bytes = (m == 0 || n == 0 || k == 0) ? 0
                                           : gffm::round_up((int64_t)(kform ? kg.a_bytes : g.a_bytes), 256) +
                                                 (kform ? kg.b_bytes : g.b_bytes);
    return GFFM_OK;
}

int gffm_karatsuba_poly_matmul_f64(int64_t m, int64_t n, int64_t k, const double *A0, const double *A1, int64_t lda,
                                   const double *B0, const double *B1, int64_t ldb, double *C0, double *C1, double *C2,
                                   int64_t ldc, int64_t p, void *ws, size_t ws_bytes, gffm_stream_t stream) {
    return poly_matmul(m, n, k, A0, A1, lda, B0, B1, ldb, C0, C1, C2, ldc, p, ws, ws_bytes, stream);
}

int gffm_karatsuba_add_f64(double *C1, double *C2, const double *A1, const double *A2, const double *B1,
                           const double *B2, int64_t len, int64_t N1, int64_t N2, gffm_stream_t stream) {
    return elementwise<K_ADD>(C1, C2, A1, A2, B1, B2, 0, len, N1, N2, stream);
}

int gffm_karatsuba_sub_f64(double *C1, double *C2, const double *A1, const double *A2, const double *B1,
                           const double *B2, int64_t len, int64_t N1, int64_t N2, gffm_stream_t stream) {
    return elementwise<K_SUB>(C1, C2, A1, A2, B1, B2, 0, len, N1, N2, stream);
}

int gffm_karatsuba_negate_f64(double *C1, double *C2, const double *A1, const double *A2, int64_t len, int64_t N1,
                              int64_t N2, gffm_stream_t stream) {
    return elementwise<K_NEG>(C1, C2, A1, A2, nullptr, nullptr, 0, len, N1, N2, stream);
}

int gffm_karatsuba_scalar_mul_f64(double *C1, double *C2, const double *A1, const double *A2, int64_t s, int64_t len,
                                  int64_t N1, int64_t N2, gffm_stream_t stream) {
    return elementwise<K_SMUL>(C1, C2, A1, A2, nullptr, nullptr, s, len, N1, N2, stream);
}

int gffm_karatsuba_from_values_f64(double *D1, double *D2, const double *A, int64_t len, int64_t N1, int64_t N2,
                                   gffm_stream_t stream) {
    return elementwise<K_FROM>(D1, D2, A, nullptr, nullptr, nullptr, 0, len, N1, N2, stream);
}

int gffm_karatsuba_to_values_f64(double *A, const double *D1, const double *D2, int64_t len, int64_t N1, int64_t N2,
                                 gffm_stream_t stream) {
    return elementwise<K_TO>(A, nullptr, D1, D2, nullptr, nullptr, 0, len, N1, N2, stream);
}

}  // extern "C"
