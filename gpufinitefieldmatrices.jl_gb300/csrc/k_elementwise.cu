// k_elementwise.cu -- the reference's grid-stride elementwise kernels
// (src/CuModMatrix/kernel_ops/{add,sub,mul,div,mod}_ops.jl) over the whole padded
// data array, HBM-bound.  Values are converted to 64-bit integers, combined
// exactly and reduced with Julia mod semantics (result in [0, N)), so results
// equal the reference's whenever its floating-point arithmetic is exact.
#include "gffm_common.cuh"
#include "modarith.cuh"

namespace {

enum Op { OP_ADD, OP_SUB, OP_MULE, OP_SADD, OP_SSUB, OP_RSSUB, OP_SMUL, OP_MOD, OP_TDIV };

struct ModN {
    int64_t n;
    uint64_t minv;  // floor((2^64 - 1) / n)
};

__device__ __forceinline__ int64_t mod_i64(int64_t x, const ModN &M) {
    if (x >= 0) return (int64_t)gffm_dev::barrett64((uint64_t)x, (uint64_t)M.n, M.minv);
    uint64_t r = gffm_dev::barrett64((uint64_t)(-x), (uint64_t)M.n, M.minv);
    return r ? M.n - (int64_t)r : 0;
}

__device__ __forceinline__ int64_t mulmod_i64(int64_t a, int64_t b, const ModN &M) {
    // a, b in [0, n)
    if (M.n <= (int64_t(1) << 31)) return (int64_t)gffm_dev::barrett64((uint64_t)(a * b), (uint64_t)M.n, M.minv);
    unsigned __int128 p = (unsigned __int128)a * (unsigned __int128)b;
    return (int64_t)(p % (unsigned __int128)M.n);
}

template <typename T>
__device__ __forceinline__ int64_t to_i64(T v) {
    return (int64_t)v;  // values are integers
}

template <typename T, int OP>
__global__ void __launch_bounds__(256) k_elementwise(T *__restrict__ C, const T *__restrict__ A,
                                                     const T *__restrict__ B, int64_t s, int64_t len, ModN M) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (; i < len; i += stride) {
        if (OP == OP_TDIV) {   // div(A, N): truncating integer division, no reduction
            C[i] = (T)(to_i64(A[i]) / M.n);
            continue;
        }
        int64_t a = mod_i64(to_i64(A[i]), M);
        int64_t r;
        if (OP == OP_ADD) {
            r = a + mod_i64(to_i64(B[i]), M);
            if (r >= M.n) r -= M.n;
        } else if (OP == OP_SUB) {
            r = a - mod_i64(to_i64(B[i]), M);
            if (r < 0) r += M.n;
        } else if (OP == OP_MULE) {
            r = mulmod_i64(a, mod_i64(to_i64(B[i]), M), M);
        } else if (OP == OP_SADD) {
            r = a + s;
            if (r >= M.n) r -= M.n;
        } else if (OP == OP_SSUB) {
            r = a - s;
            if (r < 0) r += M.n;
        } else if (OP == OP_RSSUB) {
            r = s - a;
            if (r < 0) r += M.n;
        } else if (OP == OP_SMUL) {
            r = mulmod_i64(a, s, M);
        } else {
            r = a;
        }
        C[i] = (T)r;
    }
}

template <typename T, int OP>
int launch(T *C, const T *A, const T *B, double s, int64_t len, int64_t N, gffm_stream_t stream) {
    using namespace gffm;
    if (len < 0) return set_error(GFFM_ERR_ARG, "negative length");
    if (N < 1 || N > (int64_t(1) << 52))
        return set_error(GFFM_ERR_MODULUS, "Modulus %lld is outside [1, 2^52]", (long long)N);
    if (len == 0) return GFFM_OK;
    if (!C || !A || ((OP == OP_ADD || OP == OP_SUB || OP == OP_MULE) && !B))
        return set_error(GFFM_ERR_ARG, "null data pointer");
    int st = check_device();
    if (st) return st;
    ModN M{N, ~uint64_t(0) / (uint64_t)N};
    // the scalar is reduced once on the host (Julia mod semantics)
    int64_t si = (int64_t)s;
    int64_t sr = si % N;
    if (sr < 0) sr += N;
    int64_t blocks = (len + 255) / 256;
    int64_t cap = (int64_t)sm_count() * 16;
    if (blocks > cap) blocks = cap;
    k_elementwise<T, OP><<<(unsigned)blocks, 256, 0, as_stream(stream)>>>(C, A, B, sr, len, M);
    GFFM_LAUNCH_CHECK("elementwise kernel");
    return GFFM_OK;
}

}  // namespace

#define GFFM_EW_BINARY(name, OP)                                                                       \
    int gffm_##name##_f64(double *C, const double *A, const double *B, int64_t len, int64_t N,       \
                          gffm_stream_t s) {                                                         \
        return launch<double, OP>(C, A, B, 0.0, len, N, s);                                          \
    }                                                                                                \
    int gffm_##name##_f32(float *C, const float *A, const float *B, int64_t len, int64_t N,          \
                          gffm_stream_t s) {                                                         \
        return launch<float, OP>(C, A, B, 0.0, len, N, s);                                           \
    }
#define GFFM_EW_SCALAR(name, OP)                                                                       \
    int gffm_##name##_f64(double *C, const double *A, double sc, int64_t len, int64_t N,              \
                          gffm_stream_t s) {                                                         \
        return launch<double, OP>(C, A, nullptr, sc, len, N, s);                                     \
    }                                                                                                \
    int gffm_##name##_f32(float *C, const float *A, float sc, int64_t len, int64_t N, gffm_stream_t s) { \
        return launch<float, OP>(C, A, nullptr, (double)sc, len, N, s);                              \
    }

extern "C" {
GFFM_EW_BINARY(add, OP_ADD)
GFFM_EW_BINARY(sub, OP_SUB)
GFFM_EW_BINARY(mul_elementwise, OP_MULE)
GFFM_EW_SCALAR(scalar_add, OP_SADD)
GFFM_EW_SCALAR(scalar_sub, OP_SSUB)
GFFM_EW_SCALAR(rscalar_sub, OP_RSSUB)
GFFM_EW_SCALAR(scalar_mul, OP_SMUL)

int gffm_mod_f64(double *C, const double *A, int64_t len, int64_t N, gffm_stream_t s) {
    return launch<double, OP_MOD>(C, A, nullptr, 0.0, len, N, s);
}
int gffm_mod_f32(float *C, const float *A, int64_t len, int64_t N, gffm_stream_t s) {
    return launch<float, OP_MOD>(C, A, nullptr, 0.0, len, N, s);
}

int gffm_mod_inv(int64_t p, int64_t P, int64_t *out) {
    if (!out) return gffm::set_error(GFFM_ERR_ARG, "out is NULL");
    if (P < 1 || P > (int64_t(1) << 52)) return gffm::set_error(GFFM_ERR_MODULUS, "Modulus %lld is outside [1, 2^52]", (long long)P);
    *out = elim::ref_mod_inv(p, P);
    return GFFM_OK;
}

// div!(C, A, s, mod_N): C = A * mod_inv(s, N) mod N
int gffm_div_scalar_f64(double *C, const double *A, int64_t s, int64_t len, int64_t N, gffm_stream_t st) {
    if (N < 1 || N > (int64_t(1) << 52)) return gffm::set_error(GFFM_ERR_MODULUS, "Modulus %lld is outside [1, 2^52]", (long long)N);
    return launch<double, OP_SMUL>(C, A, nullptr, (double)elim::ref_mod_inv(s, N), len, N, st);
}
int gffm_div_scalar_f32(float *C, const float *A, int64_t s, int64_t len, int64_t N, gffm_stream_t st) {
    if (N < 1 || N > (int64_t(1) << 52)) return gffm::set_error(GFFM_ERR_MODULUS, "Modulus %lld is outside [1, 2^52]", (long long)N);
    return launch<float, OP_SMUL>(C, A, nullptr, (double)elim::ref_mod_inv(s, N), len, N, st);
}

// div.(A, N) elementwise (divide_elements!): truncating integer division
int gffm_trunc_div_f64(double *C, const double *A, int64_t len, int64_t N, gffm_stream_t s) {
    return launch<double, OP_TDIV>(C, A, nullptr, 0.0, len, N, s);
}
int gffm_trunc_div_f32(float *C, const float *A, int64_t len, int64_t N, gffm_stream_t s) {
    return launch<float, OP_TDIV>(C, A, nullptr, 0.0, len, N, s);
}
}
