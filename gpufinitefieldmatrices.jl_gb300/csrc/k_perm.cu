// k_perm.cu -- swap-stack permutations of rows / columns
// (src/CuModMatrix/rref_lu_pluq/permutations.jl:11-125): apply_row_perm!,
// apply_row_inv_perm!, apply_col_perm!, apply_col_inv_perm!.  As in the
// reference, one thread owns one column (row swaps) or one row (column
// swaps) and walks the stack in order (or reversed for the inverse).  The
// stack is validated on the host and passed in the kernel parameters in
// chunks of up to kChunk pairs.
#include "gffm_common.cuh"

#include <algorithm>

namespace {

constexpr int kChunk = 2048;

struct SwapChunk {
    int32_t a[kChunk];
    int32_t b[kChunk];
    int count;
};

// rows: element (i, j) at A[i + j*lda]; a row swap exchanges A[a, j] and A[b, j]
template <typename T>
__global__ void k_row_swaps(T *A, int64_t lda, int64_t ncols, const __grid_constant__ SwapChunk c) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= ncols) return;
    T *col = A + j * lda;
    for (int s = 0; s < c.count; s++) {
        T x = col[c.a[s]];
        col[c.a[s]] = col[c.b[s]];
        col[c.b[s]] = x;
    }
}

template <typename T>
__global__ void k_col_swaps(T *A, int64_t lda, int64_t nrows, const __grid_constant__ SwapChunk c) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nrows) return;
    for (int s = 0; s < c.count; s++) {
        T x = A[i + (int64_t)c.a[s] * lda];
        A[i + (int64_t)c.a[s] * lda] = A[i + (int64_t)c.b[s] * lda];
        A[i + (int64_t)c.b[s] * lda] = x;
    }
}

template <typename T>
int apply(T *A, int64_t lda, int64_t extent, int64_t other, const int64_t *swaps, int64_t nswaps, int inverse,
          bool rows, gffm_stream_t stream) {
    using namespace gffm;
    if (extent < 0 || other < 0 || nswaps < 0) return set_error(GFFM_ERR_ARG, "negative size");
    if (nswaps == 0 || other == 0) return GFFM_OK;
    if (!A || !swaps) return set_error(GFFM_ERR_ARG, "null pointer");
    if (rows && lda < extent) return set_error(GFFM_ERR_ARG, "leading dimension smaller than the number of rows");
    if (!rows && lda < other) return set_error(GFFM_ERR_ARG, "leading dimension smaller than the number of rows");
    for (int64_t s = 0; s < 2 * nswaps; s++)
        if (swaps[s] < 1 || swaps[s] > extent)
            return set_error(GFFM_ERR_BOUNDS, "swap index %lld outside 1..%lld", (long long)swaps[s],
                             (long long)extent);
    int st = check_device();
    if (st) return st;
    cudaStream_t sm = as_stream(stream);
    SwapChunk c;
    int64_t done = 0;
    while (done < nswaps) {
        c.count = (int)std::min<int64_t>(kChunk, nswaps - done);
        for (int q = 0; q < c.count; q++) {
            const int64_t k = inverse ? nswaps - 1 - (done + q) : done + q;
            c.a[q] = (int32_t)(swaps[2 * k] - 1);
            c.b[q] = (int32_t)(swaps[2 * k + 1] - 1);
        }
        const unsigned blocks = (unsigned)((other + 127) / 128);
        if (rows)
            k_row_swaps<T><<<blocks, 128, 0, sm>>>(A, lda, other, c);
        else
            k_col_swaps<T><<<blocks, 128, 0, sm>>>(A, lda, other, c);
        GFFM_LAUNCH_CHECK("swap kernel");
        done += c.count;
    }
    return GFFM_OK;
}

}  // namespace

extern "C" {

int gffm_apply_row_swaps_f64(double *A, int64_t lda, int64_t nrows, int64_t ncols, const int64_t *swaps,
                             int64_t nswaps, int inverse, gffm_stream_t s) {
    return apply<double>(A, lda, nrows, ncols, swaps, nswaps, inverse, true, s);
}
int gffm_apply_row_swaps_f32(float *A, int64_t lda, int64_t nrows, int64_t ncols, const int64_t *swaps,
                             int64_t nswaps, int inverse, gffm_stream_t s) {
    return apply<float>(A, lda, nrows, ncols, swaps, nswaps, inverse, true, s);
}
int gffm_apply_col_swaps_f64(double *A, int64_t lda, int64_t nrows, int64_t ncols, const int64_t *swaps,
                             int64_t nswaps, int inverse, gffm_stream_t s) {
    return apply<double>(A, lda, ncols, nrows, swaps, nswaps, inverse, false, s);
}
int gffm_apply_col_swaps_f32(float *A, int64_t lda, int64_t nrows, int64_t ncols, const int64_t *swaps,
                             int64_t nswaps, int inverse, gffm_stream_t s) {
    return apply<float>(A, lda, ncols, nrows, swaps, nswaps, inverse, false, s);
}

}  // extern "C"
