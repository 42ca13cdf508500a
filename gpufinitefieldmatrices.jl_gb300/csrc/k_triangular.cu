// k_triangular.cu -- triangular inverses and the 32-row substitutions
// (src/CuModMatrix/triangular/substitution_inplace.jl and
// triangular_inverse_no_copy.jl).
//
// Substitution (forward_sub_kernel_32 / backward_sub_kernel_32): the inverse of
// the 32 x 32 triangular window of A at (row_shift, col_shift), column c of the
// result by one thread, row by row:
//   lower: X[r][c] = inv(a[r][r]) * ([r == c] - sum_{k < r} a[r][k] X[k][c])
//   upper: X[r][c] = inv(a[r][r]) * ([r == c] - sum_{k > r} a[r][k] X[k][c])
// with a[r][k] = A[row_shift + r][col_shift + k], the diagonal read at
// (row_shift + r, row_shift + r) as the reference does, entries outside A read
// as zero (the reference reads its zero padding there) and inv the reference's
// mod_inv (0 for a zero diagonal).  Arithmetic is exact: 64-bit sums of products
// below 2^52, reduced mod N.
//
// Inverse (upper/lower_triangular_inverse_no_copy): the reference's recursion on
// the leading k x k triangle, k = min(m, n): halves split at a multiple of 32
// (m = floor(size / 64 + 1/2) blocks of 32 first), the 32-blocks on the diagonal
// by substitution (all of them in one launch), then, bottom-up,
//   upper: X12 = -(X11 A12 mod N) X22 mod N,   lower: X21 = -(X22 A21 mod N) X11 mod N
// with the limb tensor-core GEMM.  For an invertible diagonal that is the
// inverse; with zero diagonal entries it is the reference's block result.  The
// output is n x m (the reference's transposed shape), zero outside the leading
// k x k.
#include "gffm_common.cuh"
#include "limb_host.h"
#include "modarith.cuh"

#include <algorithm>
#include <vector>

namespace {

using gffm::set_error;

struct ModQ {
    uint64_t n, minv;
};

template <typename T>
__device__ __forceinline__ uint32_t residue(T v, const ModQ &M) {
    const int64_t x = (int64_t)v;
    if (x >= 0) return (uint32_t)gffm_dev::barrett64((uint64_t)x, M.n, M.minv);
    const uint64_t r = gffm_dev::barrett64((uint64_t)(-x), M.n, M.minv);
    return r ? (uint32_t)(M.n - r) : 0u;
}

// One 32 x 32 window per CTA (32 threads, thread = result column).  Window b of
// the launch sits at (rs + 32 b, cs + 32 b) with its diagonal at rows rd + 32 b;
// its result goes to X at (32 b, 32 b), rows < min(32, vr - 32 b), columns
// < min(32, vc - 32 b).
template <typename T, bool UPPER>
__global__ void __launch_bounds__(32) k_tri_sub32(const T *__restrict__ A, int64_t lda, int64_t m, int64_t n,
                                                  int64_t rs, int64_t cs, int64_t rd, T *__restrict__ X, int64_t ldx,
                                                  int64_t vr, int64_t vc, ModQ M) {
    __shared__ uint32_t a[32][33];   // a[r][k] of the window
    __shared__ uint32_t dinv[32];
    __shared__ uint32_t xs[32][33];  // xs[r][c]
    const int c = threadIdx.x;
    const int64_t off = 32 * (int64_t)blockIdx.x;
    for (int r = 0; r < 32; r++) {
        const int64_t i = rs + off + r, j = cs + off + c;
        a[r][c] = (i < m && j < n) ? residue(A[i + j * lda], M) : 0u;
    }
    {
        const int64_t i = rd + off + c, j = rd + off + c;
        const uint32_t d = (i < m && j < n) ? residue(A[i + j * lda], M) : 0u;
        dinv[c] = (uint32_t)elim::ref_mod_inv((int64_t)d, (int64_t)M.n);
    }
    __syncwarp();
    for (int q = 0; q < 32; q++) {
        const int r = UPPER ? 31 - q : q;
        uint64_t acc = 0;
        if (UPPER) {
            for (int k = r + 1; k < 32; k++) acc += (uint64_t)a[r][k] * xs[k][c];
        } else {
            for (int k = 0; k < r; k++) acc += (uint64_t)a[r][k] * xs[k][c];
        }
        const uint32_t sum = (uint32_t)gffm_dev::barrett64(acc, M.n, M.minv);
        uint32_t rhs = (r == c) ? 1u : 0u;
        rhs = rhs >= sum ? rhs - sum : (uint32_t)(rhs + M.n - sum);
        xs[r][c] = (uint32_t)gffm_dev::barrett64((uint64_t)dinv[r] * rhs, M.n, M.minv);
        __syncwarp();
    }
    const int64_t nr = vr - off < 32 ? vr - off : 32, nc = vc - off < 32 ? vc - off : 32;
    if (c < nc)
        for (int r = 0; r < nr; r++) X[(off + r) + (off + c) * ldx] = (T)xs[r][c];
}

// X block <- (N - X block) mod N
template <typename T>
__global__ void __launch_bounds__(256) k_negate_block(T *X, int64_t ldx, int64_t rows, int64_t cols, int64_t N) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= rows * cols) return;
    const int64_t i = e % rows, j = e / rows;
    const int64_t v = (int64_t)X[i + j * ldx];
    X[i + j * ldx] = (T)(v ? N - v : 0);
}

template <typename T>
int limb_matmul(int64_t m, int64_t n, int64_t k, const T *A, int64_t lda, const T *B, int64_t ldb, T *C, int64_t ldc,
                int64_t N, void *ws, size_t wsb, cudaStream_t s);
template <>
int limb_matmul<double>(int64_t m, int64_t n, int64_t k, const double *A, int64_t lda, const double *B, int64_t ldb,
                        double *C, int64_t ldc, int64_t N, void *ws, size_t wsb, cudaStream_t s) {
    return gffm_matmul_limb_f64(m, n, k, A, lda, B, ldb, C, ldc, N, ws, wsb, s);
}
template <>
int limb_matmul<float>(int64_t m, int64_t n, int64_t k, const float *A, int64_t lda, const float *B, int64_t ldb,
                       float *C, int64_t ldc, int64_t N, void *ws, size_t wsb, cudaStream_t s) {
    return gffm_matmul_limb_f32(m, n, k, A, lda, B, ldb, C, ldc, N, ws, wsb, s);
}

// The recursion's combine steps, bottom-up, as (lo, mid, hi) triples
void combines(int64_t lo, int64_t hi, std::vector<int64_t> &out) {
    const int64_t s = hi - lo;
    if (s <= 32) return;
    int64_t q = (int64_t)((double)s / 64.0 + 0.5);
    if (q < 1) q = 1;
    const int64_t mid = lo + 32 * q;
    combines(lo, mid, out);
    combines(mid, hi, out);
    out.push_back(lo);
    out.push_back(mid);
    out.push_back(hi);
}

// workspace: the temporary product of the largest combine plus the limb GEMM's own
size_t tri_workspace(int64_t k, int64_t N) {
    std::vector<int64_t> cmb;
    combines(0, k, cmb);
    size_t need = 0;
    for (size_t i = 0; i < cmb.size(); i += 3) {
        const int64_t s1 = cmb[i + 1] - cmb[i], s2 = cmb[i + 2] - cmb[i + 1];
        size_t w1 = 0, w2 = 0;
        gffm_matmul_limb_workspace_size(s1, s2, s1, N, &w1);   // upper: X11 (s1 x s1) A12 (s1 x s2)
        gffm_matmul_limb_workspace_size(s1, s2, s2, N, &w2);   //        tmp (s1 x s2) X22 (s2 x s2)
        size_t w3 = 0, w4 = 0;
        gffm_matmul_limb_workspace_size(s2, s1, s2, N, &w3);   // lower: X22 A21, then tmp X11
        gffm_matmul_limb_workspace_size(s2, s1, s1, N, &w4);
        const size_t g = std::max(std::max(w1, w2), std::max(w3, w4));
        const size_t t = (size_t)gffm::round_up(s1 * s2 * 8, 256);
        need = std::max(need, t + g);
    }
    return need;
}

int check_tri(int64_t m, int64_t n, int64_t lda, int64_t ldx, int64_t N) {
    if (m < 0 || n < 0) return set_error(GFFM_ERR_ARG, "negative matrix size");
    if (lda < std::max<int64_t>(m, 1) || ldx < std::max<int64_t>(n, 1))
        return set_error(GFFM_ERR_ARG, "leading dimension smaller than the number of rows");
    if (N < 2 || N >= (int64_t(1) << 26))
        return set_error(GFFM_ERR_MODULUS, "triangular inverses need 2 <= N < 2^26 (got %lld)", (long long)N);
    return GFFM_OK;
}

template <typename T>
int tri_sub32(bool upper, int64_t m, int64_t n, const T *A, int64_t lda, int64_t rs, int64_t cs, T *X, int64_t ldx,
              int64_t N, gffm_stream_t stream) {
    int st = check_tri(m, n, lda, ldx, N);
    if (st) return st;
    if (rs < 0 || cs < 0) return set_error(GFFM_ERR_ARG, "negative shift");
    if (m == 0 || n == 0) return GFFM_OK;
    if (!A || !X) return set_error(GFFM_ERR_ARG, "null data pointer");
    st = gffm::check_device();
    if (st) return st;
    const ModQ M{(uint64_t)N, ~uint64_t(0) / (uint64_t)N};
    cudaStream_t s = gffm::as_stream(stream);
    // the result is n x m; the window fills its leading min(32, n) x min(32, m)
    if (upper)
        k_tri_sub32<T, true><<<1, 32, 0, s>>>(A, lda, m, n, rs, cs, rs, X, ldx, n, m, M);
    else
        k_tri_sub32<T, false><<<1, 32, 0, s>>>(A, lda, m, n, rs, cs, rs, X, ldx, n, m, M);
    GFFM_LAUNCH_CHECK("k_tri_sub32");
    return GFFM_OK;
}

template <typename T>
int tri_inverse(bool upper, int64_t m, int64_t n, const T *A, int64_t lda, T *X, int64_t ldx, int64_t N, void *ws,
                size_t ws_bytes, gffm_stream_t stream) {
    int st = check_tri(m, n, lda, ldx, N);
    if (st) return st;
    if (m == 0 || n == 0) return GFFM_OK;
    if (!A || !X) return set_error(GFFM_ERR_ARG, "null data pointer");
    // the reference: lower and tall beyond one window has no (right) inverse
    if (!upper && m > n && n > 32)
        return set_error(GFFM_ERR_SIZE, "(Right) pseudoinverse not defined for tall lower triangular matrices");
    st = gffm::check_device();
    if (st) return st;
    cudaStream_t s = gffm::as_stream(stream);
    const ModQ M{(uint64_t)N, ~uint64_t(0) / (uint64_t)N};
    GFFM_CUDA(cudaMemset2DAsync(X, (size_t)ldx * sizeof(T), 0, (size_t)n * sizeof(T), (size_t)m, s));
    const int64_t k = std::min(m, n);
    // the diagonal 32-blocks of the leading k x k
    const unsigned nblk = (unsigned)((k + 31) / 32);
    if (upper)
        k_tri_sub32<T, true><<<nblk, 32, 0, s>>>(A, lda, m, n, 0, 0, 0, X, ldx, k, k, M);
    else
        k_tri_sub32<T, false><<<nblk, 32, 0, s>>>(A, lda, m, n, 0, 0, 0, X, ldx, k, k, M);
    GFFM_LAUNCH_CHECK("k_tri_sub32");
    std::vector<int64_t> cmb;
    combines(0, k, cmb);
    if (cmb.empty()) return GFFM_OK;
    const size_t need = tri_workspace(k, N);
    gffm::Scratch scr;
    st = scr.acquire(ws, ws_bytes, need, s);
    if (st) return st;
    for (size_t i = 0; i < cmb.size(); i += 3) {
        const int64_t lo = cmb[i], mid = cmb[i + 1], hi = cmb[i + 2];
        const int64_t s1 = mid - lo, s2 = hi - mid;
        const size_t t = (size_t)gffm::round_up(s1 * s2 * 8, 256);
        T *tmp = static_cast<T *>(scr.ptr);
        void *gws = static_cast<uint8_t *>(scr.ptr) + t;
        const size_t gwsb = need - t;
        T *X11 = X + lo + lo * ldx, *X22 = X + mid + mid * ldx;
        if (upper) {
            // X12 = -(X11 A12) X22: tmp (s1 x s2), then the product into X's block
            st = limb_matmul<T>(s1, s2, s1, X11, ldx, A + lo + mid * lda, lda, tmp, s1, N, gws, gwsb, s);
            if (st) return st;
            T *X12 = X + lo + mid * ldx;
            st = limb_matmul<T>(s1, s2, s2, tmp, s1, X22, ldx, X12, ldx, N, gws, gwsb, s);
            if (st) return st;
            k_negate_block<T><<<(unsigned)((s1 * s2 + 255) / 256), 256, 0, s>>>(X12, ldx, s1, s2, N);
        } else {
            // X21 = -(X22 A21) X11: tmp (s2 x s1), then the product into X's block
            st = limb_matmul<T>(s2, s1, s2, X22, ldx, A + mid + lo * lda, lda, tmp, s2, N, gws, gwsb, s);
            if (st) return st;
            T *X21 = X + mid + lo * ldx;
            st = limb_matmul<T>(s2, s1, s1, tmp, s2, X11, ldx, X21, ldx, N, gws, gwsb, s);
            if (st) return st;
            k_negate_block<T><<<(unsigned)((s1 * s2 + 255) / 256), 256, 0, s>>>(X21, ldx, s2, s1, N);
        }
        GFFM_LAUNCH_CHECK("k_negate_block");
    }
    return GFFM_OK;
}

}  // namespace

extern "C" {

int gffm_tri_sub32_f64(int upper, int64_t m, int64_t n, const double *A, int64_t lda, int64_t row_shift,
                       int64_t col_shift, double *X, int64_t ldx, int64_t N, gffm_stream_t stream) {
    return tri_sub32<double>(upper != 0, m, n, A, lda, row_shift, col_shift, X, ldx, N, stream);
}
int gffm_tri_sub32_f32(int upper, int64_t m, int64_t n, const float *A, int64_t lda, int64_t row_shift,
                       int64_t col_shift, float *X, int64_t ldx, int64_t N, gffm_stream_t stream) {
    return tri_sub32<float>(upper != 0, m, n, A, lda, row_shift, col_shift, X, ldx, N, stream);
}

int gffm_triangular_inverse_workspace_size(int upper, int64_t m, int64_t n, int64_t N, size_t *bytes) {
    (void)upper;
    if (!bytes) return set_error(GFFM_ERR_ARG, "bytes is NULL");
    int st = check_tri(m, n, std::max<int64_t>(m, 1), std::max<int64_t>(n, 1), N);
    if (st) return st;
    *bytes = (m == 0 || n == 0) ? 0 : tri_workspace(std::min(m, n), N);
    return GFFM_OK;
}
int gffm_triangular_inverse_f64(int upper, int64_t m, int64_t n, const double *A, int64_t lda, double *X, int64_t ldx,
                                int64_t N, void *ws, size_t ws_bytes, gffm_stream_t stream) {
    return tri_inverse<double>(upper != 0, m, n, A, lda, X, ldx, N, ws, ws_bytes, stream);
}
int gffm_triangular_inverse_f32(int upper, int64_t m, int64_t n, const float *A, int64_t lda, float *X, int64_t ldx,
                                int64_t N, void *ws, size_t ws_bytes, gffm_stream_t stream) {
    return tri_inverse<float>(upper != 0, m, n, A, lda, X, ldx, N, ws, ws_bytes, stream);
}

}  // extern "C"
