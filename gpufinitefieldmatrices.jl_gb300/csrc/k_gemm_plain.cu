// k_gemm_plain.cu -- the "plain" modular GEMM/GEMV: the reference's own method
// (src/CuModMatrix/kernel_mul/stripe_mul.jl:82-244).  Residues are held in the
// floating-point element type, products are summed exactly with FMAs in
// K-stripes of find_max_stripe_ops(type, N) columns (so every partial sum stays
// below 2^53 for Float64 / 2^24 for Float32) and reduced mod N after each
// stripe.  The reference does each stripe as a cuBLAS GEMM over the whole
// padded C followed by a full-matrix mod! pass; here the stripes are reduced in
// registers of one SIMT kernel, so C is written once.
#include "gffm_common.cuh"

namespace {

template <typename T>
struct FMod;

template <>
struct FMod<double> {
    // x: an integer-valued double with |x| < 2^53; returns x mod n in [0, n) exactly
    // (floor's quotient is off by at most one either way; the corrections fix it).
    __device__ static __forceinline__ double red(double x, double n, double inv) {
        double q = floor(x * inv);
        double r = fma(-q, n, x);
        if (r < 0.0) r += n;
        if (r >= n) r -= n;
        return r;
    }
    // x: an integer-valued double with |x| < 2^52 + 2^26 (one product plus a value in
    // (-n, n)); returns a value congruent to x mod n in (-n, n), exactly: x * inv is
    // within 2^-25 of x / n, so q = rint(x / n) leaves |x - q n| <= n/2 + 1, an integer
    // the fma computes without rounding.  With the product's fma that is four FP64
    // instructions per multiply-add instead of the two corrections of red().
    __device__ static __forceinline__ double red_signed(double x, double n, double inv) {
        return fma(-rint(x * inv), n, x);
    }
    __device__ static __forceinline__ double fma_(double a, double b, double c) { return fma(a, b, c); }
};

template <>
struct FMod<float> {
    __device__ static __forceinline__ float red(float x, float n, float inv) {
        float q = floorf(x * inv);
        float r = fmaf(-q, n, x);
        if (r < 0.0f) r += n;
        if (r >= n) r -= n;
        return r;
    }
    __device__ static __forceinline__ float red_signed(float x, float n, float inv) {
        return fmaf(-rintf(x * inv), n, x);
    }
    __device__ static __forceinline__ float fma_(float a, float b, float c) { return fmaf(a, b, c); }
};

// loads reduce an input element into [0, N) (inputs may exceed N under a
// modulus override, mat_mul_gpu_type(A, B, mod_N))
template <typename T>
__device__ __forceinline__ T load_red(const T *p, T n, T inv) {
    T v = *p;
    if (v >= (T)0 && v < n) return v;
    return FMod<T>::red(v, n, inv);  // exact for any integer |v| < 2^53 (2^24)
}

constexpr int PBM = 64, PBN = 64, PBK = 16;

template <typename T>
__global__ void __launch_bounds__(256) k_matmul_plain(int64_t m, int64_t n, int64_t k, const T *__restrict__ A,
                                                      int64_t lda, const T *__restrict__ B, int64_t ldb,
                                                      T *__restrict__ C, int64_t ldc, T Nt, T inv, int64_t stripe) {
    __shared__ T As[PBK][PBM + 1];
    __shared__ T Bs[PBK][PBN + 1];
    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
    const int64_t r0 = (int64_t)blockIdx.y * PBM, c0 = (int64_t)blockIdx.x * PBN;
    T acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = (T)0;
    int64_t cnt = 0;
    for (int64_t k0 = 0; k0 < k; k0 += PBK) {
#pragma unroll
        for (int q = 0; q < 4; q++) {
            int e = tid + 256 * q;
            int r = e % PBM, kk = e / PBM;
            int64_t gr = r0 + r, gk = k0 + kk;
            As[kk][r] = (gr < m && gk < k) ? load_red(A + gr + gk * lda, Nt, inv) : (T)0;
            int kb = e % PBK, cb = e / PBK;
            int64_t gc = c0 + cb, gk2 = k0 + kb;
            Bs[kb][cb] = (gc < n && gk2 < k) ? load_red(B + gk2 + gc * ldb, Nt, inv) : (T)0;
        }
        __syncthreads();
        int kmax = (int)((k - k0) < PBK ? (k - k0) : PBK);
        for (int kk = 0; kk < kmax; kk++) {
            T a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; i++) a[i] = As[kk][tx + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; j++) b[j] = Bs[kk][ty + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) acc[i][j] = FMod<T>::fma_(a[i], b[j], acc[i][j]);
            if (++cnt == stripe) {
                if (stripe == 1) {
                    // one product per stripe (N near the type's limit): the accumulators stay
                    // in (-N, N), so acc + a b stays below (N-1)^2 + N, exact
#pragma unroll
                    for (int i = 0; i < 4; i++)
#pragma unroll
                        for (int j = 0; j < 4; j++) acc[i][j] = FMod<T>::red_signed(acc[i][j], Nt, inv);
                } else {
#pragma unroll
                    for (int i = 0; i < 4; i++)
#pragma unroll
                        for (int j = 0; j < 4; j++) acc[i][j] = FMod<T>::red(acc[i][j], Nt, inv);
                }
                cnt = 0;
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int j = 0; j < 4; j++) {
        int64_t gc = c0 + ty + 16 * j;
        if (gc >= n) continue;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            int64_t gr = r0 + tx + 16 * i;
            if (gr < m) C[gr + gc * ldc] = FMod<T>::red(acc[i][j], Nt, inv);   // also for acc in (-N, 0)
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(256) k_matvec_plain(int64_t m, int64_t k, const T *__restrict__ A, int64_t lda,
                                                      const T *__restrict__ x, T *__restrict__ z, T Nt, T inv,
                                                      int64_t stripe) {
    __shared__ T xs[1024];
    int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    T acc = (T)0;
    int64_t cnt = 0;
    for (int64_t k0 = 0; k0 < k; k0 += 1024) {
        int kmax = (int)((k - k0) < 1024 ? (k - k0) : 1024);
        for (int i = threadIdx.x; i < kmax; i += blockDim.x) xs[i] = load_red(x + k0 + i, Nt, inv);
        __syncthreads();
        if (row < m) {
            for (int i = 0; i < kmax; i++) {
                acc = FMod<T>::fma_(load_red(A + row + (k0 + i) * lda, Nt, inv), xs[i], acc);
                if (++cnt == stripe) {
                    acc = FMod<T>::red(acc, Nt, inv);
                    cnt = 0;
                }
            }
        }
        __syncthreads();
    }
    if (row < m) z[row] = FMod<T>::red(acc, Nt, inv);
}

template <typename T>
int resolve_stripe(int64_t N, int64_t stripe, int64_t *out) {
    const int bits = sizeof(T) == 8 ? 53 : 24;
    if (N > (int64_t(1) << 52))
        return gffm::set_error(GFFM_ERR_MODULUS, "Modulus %lld is bigger than 2^52 = 4503599627370496, the largest supported modulus",
                               (long long)N);
    if (N < 1) return gffm::set_error(GFFM_ERR_MODULUS, "modulus %lld < 1", (long long)N);
    int64_t M = stripe;
    if (M <= 0) {
        int st = gffm_find_max_stripe_ops(bits, N, &M);
        if (st) return st;
    }
    if (M < 1)
        return gffm::set_error(GFFM_ERR_STRIPE, "cannot perform a single multiplication for modulus %lld with datatype %s",
                               (long long)N, sizeof(T) == 8 ? "Float64" : "Float32");
    *out = M;
    return GFFM_OK;
}

template <typename T>
int matmul_plain(int64_t m, int64_t n, int64_t k, const T *A, int64_t lda, const T *B, int64_t ldb, T *C,
                 int64_t ldc, int64_t N, int64_t stripe, gffm_stream_t stream) {
    using namespace gffm;
    if (m < 0 || n < 0 || k < 0) return set_error(GFFM_ERR_ARG, "negative matrix size");
    if (lda < (m > 1 ? m : 1) || ldb < (k > 1 ? k : 1) || ldc < (m > 1 ? m : 1))
        return set_error(GFFM_ERR_ARG, "leading dimension smaller than the number of rows");
    int64_t M = 0;
    int st = resolve_stripe<T>(N, stripe, &M);
    if (st) return st;
    if (m == 0 || n == 0) return GFFM_OK;
    if (!C || (k > 0 && (!A || !B))) return set_error(GFFM_ERR_ARG, "null data pointer");
    st = check_device();
    if (st) return st;
    dim3 grid((unsigned)((n + PBN - 1) / PBN), (unsigned)((m + PBM - 1) / PBM));
    if (grid.y > 65535u) return set_error(GFFM_ERR_ARG, "too many rows for the plain kernel");
    T Nt = (T)N;
    T inv = (T)1 / Nt;
    k_matmul_plain<T><<<grid, 256, 0, as_stream(stream)>>>(m, n, k, A, lda, B, ldb, C, ldc, Nt, inv, M);
    GFFM_LAUNCH_CHECK("k_matmul_plain");
    return GFFM_OK;
}

template <typename T>
int matvec_plain(int64_t m, int64_t k, const T *A, int64_t lda, const T *x, T *z, int64_t N, int64_t stripe,
                 gffm_stream_t stream) {
    using namespace gffm;
    if (m < 0 || k < 0) return set_error(GFFM_ERR_ARG, "negative size");
    if (lda < (m > 1 ? m : 1)) return set_error(GFFM_ERR_ARG, "leading dimension smaller than the number of rows");
    int64_t M = 0;
    int st = resolve_stripe<T>(N, stripe, &M);
    if (st) return st;
    if (m == 0) return GFFM_OK;
    if (!z || (k > 0 && (!A || !x))) return set_error(GFFM_ERR_ARG, "null data pointer");
    st = check_device();
    if (st) return st;
    T Nt = (T)N;
    T inv = (T)1 / Nt;
    k_matvec_plain<T><<<(unsigned)((m + 255) / 256), 256, 0, as_stream(stream)>>>(m, k, A, lda, x, z, Nt, inv, M);
    GFFM_LAUNCH_CHECK("k_matvec_plain");
    return GFFM_OK;
}

}  // namespace

extern "C" {
int gffm_matmul_plain_f64(int64_t m, int64_t n, int64_t k, const double *A, int64_t lda, const double *B,
                          int64_t ldb, double *C, int64_t ldc, int64_t N, int64_t stripe, gffm_stream_t s) {
    return matmul_plain<double>(m, n, k, A, lda, B, ldb, C, ldc, N, stripe, s);
}
int gffm_matmul_plain_f32(int64_t m, int64_t n, int64_t k, const float *A, int64_t lda, const float *B,
                          int64_t ldb, float *C, int64_t ldc, int64_t N, int64_t stripe, gffm_stream_t s) {
    return matmul_plain<float>(m, n, k, A, lda, B, ldb, C, ldc, N, stripe, s);
}
int gffm_matvec_plain_f64(int64_t m, int64_t k, const double *A, int64_t lda, const double *x, double *z,
                          int64_t N, int64_t stripe, gffm_stream_t s) {
    return matvec_plain<double>(m, k, A, lda, x, z, N, stripe, s);
}
int gffm_matvec_plain_f32(int64_t m, int64_t k, const float *A, int64_t lda, const float *x, float *z, int64_t N,
                          int64_t stripe, gffm_stream_t s) {
    return matvec_plain<float>(m, k, A, lda, x, z, N, stripe, s);
}
}
