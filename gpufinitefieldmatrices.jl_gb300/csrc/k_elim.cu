// k_elim.cu -- blocked right-looking PLUQ / LU / RREF over Z/N (N < 2^26) with
// the exact step semantics of the reference's pluq_gpu_kernel
// (src/CuModMatrix/rref_lu_pluq/pluq_kernels.jl:46-440).
//
// Working copy.  A is copied into W, a row-major int32 matrix of residues, so
// that row swaps are contiguous copies.  Multipliers are kept below each pivot
// in W (LAPACK style) and moved into L at the end.
//
// One panel = up to NB consecutive pivot columns starting at (R0, C0).  The
// panel kernel (elim_panel.cuh) is a cooperative grid: CTA b keeps rows
// [R0 + b*R, R0 + (b+1)*R) of the panel in shared memory and factors
// left-looking (column t is formed only when the pivot search reaches it, by
// one exact dot product per row against U[0:t][t] = L11^{-1} W_piv[0:t][t]).
// Per pivot step it
//   1. publishes its candidate -- the largest residue of the pivot column in
//      its rows (lowest row on ties) and that row -- as words tagged with the
//      step in a parity-double-buffered global slot; the owner of the current
//      row r publishes that row,
//   2. polls the G keys (the grid barrier, bounded waits) while its row
//      threads form the next column's partial sums,
//   3. picks the global winner, fetches its row (and the displaced row r where
//      that lands) while one warp inverts the pivot by the reference's extended
//      Euclid, moves the two rows and completes the next column.
// A single CTA factors 32-column panels once the rows fit it (k_panel1).
// Both panels write L11^{-1} of their pivots.
// Everything the reference does to columns outside the panel is deferred and
// applied after the panel in the same order-independent form:
//   - columns left of the panel: the panel's row swaps (earlier multipliers and
//     skipped columns), then the pivot-row scaling of the skipped columns,
//   - trailing columns: the row swaps, the triangular solve for the panel rows
//     U12 = L11^{-1} P A12 (x_t = inv_t * (a_t - sum_{s<t} L[r_t, c_s] x_s):
//     the reference's scaling and updates in closed form, with the panel's
//     L11^{-1}) and the update of the rows below, A22 -= L21 * U12 mod N, both
//     on the limb tensor-core GEMM.
// W keeps every multiplier column permuted for this arithmetic; the
// reference's narrower swap width for L (32*cld(m, 32) columns) is restored
// when L is extracted.
// A zero pivot column ends the panel when the panel already has pivots; at the
// start of a panel it triggers the reference's swap with the last column
// (PLUQ) or is skipped (LU / RREF).  Exact modular arithmetic makes every
// pivot search see the same values as the unblocked reference, so the pivot
// sequence, P, L, U, Q and the swap stacks are identical.
#include "gffm_common.cuh"
#include "elim_panel.cuh"
#include "limb_host.h"

#include <algorithm>
#include <cstring>
#include <unordered_map>
#include <vector>

namespace elim {

enum Mode { MODE_PLUQ = 0, MODE_LU = 1, MODE_RREF = 2 };
constexpr int RB = 64;  // pivots per block of the RREF back substitution

// A (column-major, any element type holding integers) -> W (row-major int32 residues)
template <typename T>
__global__ void __launch_bounds__(256) k_to_rowmajor(const T *__restrict__ A, int64_t lda, int m, int n,
                                                     int32_t *__restrict__ W, int64_t ldw, ModP M) {
    __shared__ int32_t tile[32][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int64_t r0 = (int64_t)blockIdx.y * 32, c0 = (int64_t)blockIdx.x * 32;
    for (int i = 0; i < 4; i++) {
        int64_t c = c0 + ty + 8 * i, r = r0 + tx;
        int32_t v = 0;
        if (r < m && c < n) {
            int64_t x = (int64_t)A[r + c * lda];
            if (x < 0 || x >= (int64_t)M.n) {
                if (x >= 0) {
                    x = (int64_t)gffm_dev::barrett64((uint64_t)x, M.n, M.minv);
                } else {
                    uint64_t q = gffm_dev::barrett64((uint64_t)(-x), M.n, M.minv);
                    x = q ? (int64_t)M.n - (int64_t)q : 0;
                }
            }
            v = (int32_t)x;
        }
        tile[ty + 8 * i][tx] = v;
    }
    __syncthreads();
    for (int i = 0; i < 4; i++) {
        int64_t r = r0 + ty + 8 * i, c = c0 + tx;
        if (r < m && c < n) W[r * ldw + c] = tile[tx][ty + 8 * i];
    }
}

// Skipped (swapped-in, never eliminated) columns: the panel's row swaps for
// columns at or beyond lo (those below lo were covered by permute_rows2), then the
// scaling of every new pivot row, as swap_rows_and_mod does over all columns.
__global__ void k_skipped(int32_t *W, int64_t ldw, const int32_t *qlist, int nq, int lo, int R0, int t,
                          const int32_t *prow, const int32_t *inv, ModP M) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nq) return;
    const int q = qlist[k];
    if (q >= lo) {
        for (int s = 0; s < t; s++) {
            const int r = R0 + s, p = prow[s];
            if (p != r) {
                int32_t x = W[(int64_t)r * ldw + q];
                W[(int64_t)r * ldw + q] = W[(int64_t)p * ldw + q];
                W[(int64_t)p * ldw + q] = x;
            }
        }
    }
    for (int s = 0; s < t; s++) {
        int32_t *e = W + (int64_t)(R0 + s) * ldw + q;
        *e = (int32_t)mulmod((uint32_t)*e, (uint32_t)inv[s], M);
    }
}

// swap_cols(d_A, col, Perm_col_idx) over all rows
__global__ void k_colswap(int32_t *W, int64_t ldw, int m, int c1, int c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m || c1 == c2) return;
    int32_t x = W[(int64_t)i * ldw + c1];
    W[(int64_t)i * ldw + c1] = W[(int64_t)i * ldw + c2];
    W[(int64_t)i * ldw + c2] = x;
}

// *flag = 1 if any W[r][c] != 0 for r >= r0, c >= c0 (flag zeroed by the caller)
__global__ void __launch_bounds__(256) k_any_nonzero(const int32_t *__restrict__ W, int64_t ldw, int r0, int m, int c0,
                                                     int n, int *flag) {
    const int64_t cols = n - c0;
    const int64_t total = (int64_t)(m - r0) * cols;
    int found = 0;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = idx / cols, c = idx - r * cols;
        found |= W[(int64_t)(r0 + r) * ldw + c0 + c] != 0;
    }
    if (__syncthreads_or(found) && threadIdx.x == 0) atomicExch(flag, 1);
}

// W[r][c0 + j] <- W[r][src[j]] for every row r and j < ncols: a column permutation of
// [c0, c0 + ncols), one row per block through shared memory
__global__ void __launch_bounds__(256) k_permute_cols(int32_t *__restrict__ W, int64_t ldw, int c0, int ncols,
                                                      const int32_t *__restrict__ src) {
    extern __shared__ int32_t rowbuf[];
    int32_t *w = W + (int64_t)blockIdx.x * ldw;
    for (int j = threadIdx.x; j < ncols; j += blockDim.x) rowbuf[j] = w[c0 + j];
    __syncthreads();
    for (int j = threadIdx.x; j < ncols; j += blockDim.x) w[c0 + j] = rowbuf[src[j] - c0];
}

// [A | I] (n x 2n, column-major, ld) from A (n x n, column-major, lda)
template <typename T>
__global__ void __launch_bounds__(256) k_build_augmented(const T *__restrict__ A, int64_t lda, int n, T *__restrict__ X,
                                                         int64_t ld) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t total = (int64_t)n * 2 * n;
    if (idx >= total) return;
    const int64_t c = idx / n, r = idx - c * n;
    X[r + c * ld] = c < n ? A[r + c * lda] : (T)(c - n == r ? 1 : 0);
}

// U (column-major) from W: multipliers below each pivot become 0.
template <typename T>
__global__ void __launch_bounds__(256) k_extract_u(const int32_t *__restrict__ W, int64_t ldw, int m, int n,
                                                   const int32_t *__restrict__ colpiv, T *__restrict__ U,
                                                   int64_t ldu) {
    __shared__ int32_t tile[32][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int64_t r0 = (int64_t)blockIdx.y * 32, c0 = (int64_t)blockIdx.x * 32;
    for (int i = 0; i < 4; i++) {
        int64_t r = r0 + ty + 8 * i, c = c0 + tx;
        tile[ty + 8 * i][tx] = (r < m && c < n) ? W[r * ldw + c] : 0;
    }
    __syncthreads();
    for (int i = 0; i < 4; i++) {
        int64_t c = c0 + ty + 8 * i, r = r0 + tx;
        if (r < m && c < n) {
            const int pr = colpiv[c];
            U[r + c * ldu] = (pr >= 0 && r > pr) ? (T)0 : (T)tile[tx][ty + 8 * i];
        }
    }
}

// L (column-major, m x lcols): column c holds the multipliers of the pivot
// whose W column is lsrc[c] (below pivot row lrow[c]) and the pivot value on
// that row; columns without a pivot are zero.
template <typename T>
__global__ void __launch_bounds__(256) k_extract_l(const int32_t *__restrict__ W, int64_t ldw, int m, int lcols,
                                                   const int32_t *__restrict__ lsrc, const int32_t *__restrict__ lrow,
                                                   const int32_t *__restrict__ lpv, T *__restrict__ L, int64_t ldl) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= m) return;
    for (int c = blockIdx.y; c < lcols; c += gridDim.y) {
        const int sc = lsrc[c];
        T v = (T)0;
        if (sc >= 0) {
            const int pr = lrow[c];
            if (r > pr)
                v = (T)W[r * ldw + sc];
            else if (r == pr)
                v = (T)lpv[c];
        }
        L[r + (int64_t)c * ldl] = v;
    }
}

// RREF: zero the multipliers below the pivots of W
__global__ void k_zero_below(int32_t *W, int64_t ldw, int m, int n, const int32_t *colpiv) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= m) return;
    for (int c = blockIdx.y; c < n; c += gridDim.y) {
        const int pr = colpiv[c];
        if (pr >= 0 && r > pr) W[r * ldw + c] = 0;
    }
}

// RREF backward phase, one block of pivots (rows p0..p0+nbp-1, pivot columns
// pcol[]): the block's reduced rows R_B = V^{-1} U_B, V[k][i] = U_B[k][pcol[i]]
// unit upper triangular (coef, gathered before this kernel), by back
// substitution per column j >= pcol[0]: R[k] = U[k] - sum_{i>k} V[k][i] R[i].
__global__ void __launch_bounds__(128) k_rref_block(int32_t *W, int64_t ldw, int p0, int nbp, const int32_t *pcol,
                                                    const int32_t *coefbuf, int n, ModP M) {
    __shared__ uint32_t coef[RB][RB + 1];
    for (int e = threadIdx.x; e < RB * RB; e += blockDim.x) {
        int k = e / RB, i = e % RB;
        coef[k][i] = (k < nbp && i < nbp && i > k) ? (M.n - (uint32_t)coefbuf[k * RB + i]) % M.n : 0;
    }
    __syncthreads();
    const int j = pcol[0] + blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    uint32_t y[RB];
#pragma unroll
    for (int kk = RB - 1; kk >= 0; kk--) {
        y[kk] = 0;
        if (kk < nbp) {
            uint64_t acc = (uint32_t)W[(int64_t)(p0 + kk) * ldw + j];
#pragma unroll
            for (int i = RB - 1; i > kk; i--) acc += (uint64_t)coef[kk][i] * y[i];
            y[kk] = (uint32_t)gffm_dev::barrett64(acc, M.n, M.minv);
        }
    }
#pragma unroll
    for (int kk = 0; kk < RB; kk++)
        if (kk < nbp) W[(int64_t)(p0 + kk) * ldw + j] = (int32_t)y[kk];
}

// out[k][i] = W[row0 + k][pcol[i]] for k < rows (row-major, ld RB; zero past nbp)
__global__ void k_gather_cols(const int32_t *W, int64_t ldw, int row0, int rows, int nbp, const int32_t *pcol,
                              int32_t *out) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= rows) return;
    for (int i = 0; i < RB; i++) out[k * RB + i] = i < nbp ? W[(row0 + k) * ldw + pcol[i]] : 0;
}

// ---------------------------------------------------------------------------
// Host driver
// ---------------------------------------------------------------------------
struct Work {
    int32_t *W;
    int64_t ldw;
    Rec *rec;
    unsigned long long *old_row;                 // the panel's displaced-row words (exchange area)
    int32_t *piv_row, *piv_val, *piv_inv;
    int *result;
    int32_t *colpiv, *lsrc, *lrow, *lpv, *pcol;  // [n], [lcols] x3, [min(m,n)]
    int32_t *gather;                             // m x NB
    int32_t *coef;                               // NB x NB
    int32_t *linv;                               // NB x NB, inverse of the panel's L11
    int32_t *qlist;                              // [n] skipped columns
    __half *dA, *dB;                             // digit planes
    __half *dA2;                                 // digit planes of the next panel's columns (lookahead)
    limb::Layout gl;
    int plain = 0;                               // trailing products on the plain Float64 method
    int64_t stripe = 1;                          // its stripe: find_max_stripe_ops(Float64, N)
};

static size_t al(size_t x) { return (x + 255) & ~size_t(255); }

static void layout_ws(int64_t m, int64_t n, int64_t lcols, size_t *total, size_t off[15], limb::Layout *gl) {
    const int64_t ldw = gffm::round_up(n > 0 ? n : 1, 32);
    // digit planes large enough for any trailing update / back substitution of
    // this problem: operands n x NB and NB x m (4 digits)
    *gl = limb::layout(std::max<int64_t>(n, 1), std::max<int64_t>(m, 1), NB, int64_t(1) << 25);
    size_t sizes[15] = {
        (size_t)std::max<int64_t>(m, 1) * ldw * 4,      // W
        exchange_bytes(MAX_PANEL_CTAS),                 // old_row words + rec
        (size_t)NB * NB * 4,                            // linv
        NB * 4, NB * 4, NB * 4,                         // piv_row/val/inv
        64,                                             // result
        (size_t)std::max<int64_t>(n, 1) * 4,            // colpiv
        (size_t)std::max<int64_t>(lcols, 1) * 4 * 3,    // lsrc/lrow/lpv
        (size_t)std::max<int64_t>(std::min(m, n), 1) * 4,  // pcol
        (size_t)std::max<int64_t>(m, 1) * NB * 4,       // gather
        gl->a_bytes, gl->b_bytes,
        (size_t)NB * NB * 4 + (size_t)std::max<int64_t>(n, 1) * 4,  // coef, qlist
        limb::layout(NB, std::max<int64_t>(m, 1), NB, int64_t(1) << 25).a_bytes};  // dA2
    size_t o = 0;
    for (int i = 0; i < 15; i++) {
        off[i] = o;
        o += al(sizes[i]);
    }
    *total = o;
}

static void bind_ws(void *base, int64_t m, int64_t n, int64_t lcols, Work *w) {
    size_t total, off[15];
    layout_ws(m, n, lcols, &total, off, &w->gl);
    uint8_t *b = static_cast<uint8_t *>(base);
    w->W = (int32_t *)(b + off[0]);
    w->ldw = gffm::round_up(n > 0 ? n : 1, 32);
    w->old_row = (unsigned long long *)(b + off[1]);
    w->rec = (Rec *)(b + off[1] + OLD_ROW_WORDS * 8);
    w->linv = (int32_t *)(b + off[2]);
    w->piv_row = (int32_t *)(b + off[3]);
    w->piv_val = (int32_t *)(b + off[4]);
    w->piv_inv = (int32_t *)(b + off[5]);
    w->result = (int *)(b + off[6]);
    w->colpiv = (int32_t *)(b + off[7]);
    w->lsrc = (int32_t *)(b + off[8]);
    w->lrow = w->lsrc + std::max<int64_t>(lcols, 1);
    w->lpv = w->lrow + std::max<int64_t>(lcols, 1);
    w->pcol = (int32_t *)(b + off[9]);
    w->gather = (int32_t *)(b + off[10]);
    w->dA = (__half *)(b + off[11]);
    w->dB = (__half *)(b + off[12]);
    w->coef = (int32_t *)(b + off[13]);
    w->qlist = w->coef + NB * NB;
    w->dA2 = (__half *)(b + off[14]);
}

size_t workspace_bytes(int64_t m, int64_t n, int64_t lcols) {
    size_t total, off[15];
    limb::Layout gl;
    layout_ws(m, n, lcols, &total, off, &gl);
    return total;
}

struct Result {
    std::vector<int64_t> row_swaps, col_swaps;  // flattened 1-based pairs
    std::vector<int> piv_r, piv_c, piv_v;       // pivots in order
    std::vector<int> swap_step;                 // pivot index of each recorded row swap
    std::vector<int> perm;                      // LU: final row order (0-based original index)
    int rank = 0;
};

// The trailing products on the reference's plain Float64 arithmetic
// (src/CuModMatrix/kernel_mul/stripe_mul.jl:175-244): exact FP64 products
// summed in stripes of find_max_stripe_ops(Float64, N) and reduced mod N after
// each stripe, 64 x 64 tiles of C per CTA, 4 x 4 per thread.  Operands as in
// rowmajor_gemm; Y must not overlap C.  The comparison leg of the limb GEMM.
__device__ __forceinline__ double plain_red(double x, double n, double inv) {
    const double q = floor(x * inv);
    double r = fma(-q, n, x);
    if (r < 0.0) r += n;
    if (r >= n) r -= n;
    return r;
}

template <bool SUB>
__global__ void __launch_bounds__(256) k_plain_rowmajor(int32_t *__restrict__ C, int64_t ldc,
                                                        const int32_t *__restrict__ X, int64_t ldx,
                                                        const int32_t *__restrict__ Y, int64_t ldy, int rows, int cols,
                                                        int k, double Nd, double inv, int64_t stripe) {
    __shared__ double Xs[16][65];
    __shared__ double Ys[16][65];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int r0 = blockIdx.y * 64, c0 = blockIdx.x * 64;
    double acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = 0.0;
    int64_t cnt = 0;
    for (int k0 = 0; k0 < k; k0 += 16) {
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int e = tid + 256 * q;
            const int r = e >> 4, kk = e & 15;
            Xs[kk][r] = (r0 + r < rows && k0 + kk < k) ? (double)X[(int64_t)(r0 + r) * ldx + k0 + kk] : 0.0;
            const int kk2 = e >> 6, c = e & 63;
            Ys[kk2][c] = (k0 + kk2 < k && c0 + c < cols) ? (double)Y[(int64_t)(k0 + kk2) * ldy + c0 + c] : 0.0;
        }
        __syncthreads();
        const int kmax = min(16, k - k0);
        for (int kk = 0; kk < kmax; kk++) {
            double xv[4], yv[4];
#pragma unroll
            for (int i = 0; i < 4; i++) xv[i] = Xs[kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; j++) yv[j] = Ys[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) acc[i][j] = fma(xv[i], yv[j], acc[i][j]);
            if (++cnt == stripe) {
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int j = 0; j < 4; j++) acc[i][j] = plain_red(acc[i][j], Nd, inv);
                cnt = 0;
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int r = r0 + ty + 16 * i;
        if (r >= rows) continue;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int c = c0 + tx + 16 * j;
            if (c >= cols) continue;
            const double v = plain_red(acc[i][j], Nd, inv);
            int32_t *cp = C + (int64_t)r * ldc + c;
            if (SUB) {
                double d = (double)*cp - v;
                *cp = (int32_t)(d < 0.0 ? d + Nd : d);
            } else {
                *cp = (int32_t)v;
            }
        }
    }
}

// Row-major products on the limb GEMM:
// C (rows x cols, row-major, ldc) (-)= X (rows x k, row-major, ldx) * Y (k x cols, row-major, ldy),
// epi = limb::EPI_SUB_I32 (C -= XY) or limb::EPI_STORE_I32 (C = XY; C may overlap Y, which is
// split into digit planes before the product runs).
static int rowmajor_gemm(Work &w, int64_t N, int32_t *C, int64_t ldc, const int32_t *X, int64_t ldx,
                         const int32_t *Y, int64_t ldy, int64_t rows, int64_t cols, int64_t k, int epi,
                         cudaStream_t s) {
    if (rows <= 0 || cols <= 0 || k <= 0) return GFFM_OK;
    if (w.plain) {
        // Y may overlap C (U12 = L11^-1 P A12 in place): copy it out first
        int32_t *Yc = reinterpret_cast<int32_t *>(w.dA);
        GFFM_CUDA(cudaMemcpy2DAsync(Yc, (size_t)cols * 4, Y, (size_t)ldy * 4, (size_t)cols * 4, (size_t)k,
                                    cudaMemcpyDeviceToDevice, s));
        dim3 grid((unsigned)((cols + 63) / 64), (unsigned)((rows + 63) / 64));
        const double Nd = (double)N;
        if (epi == limb::EPI_SUB_I32)
            k_plain_rowmajor<true><<<grid, 256, 0, s>>>(C, ldc, X, ldx, Yc, cols, (int)rows, (int)cols, (int)k, Nd,
                                                         1.0 / Nd, w.stripe);
        else
            k_plain_rowmajor<false><<<grid, 256, 0, s>>>(C, ldc, X, ldx, Yc, cols, (int)rows, (int)cols, (int)k, Nd,
                                                          1.0 / Nd, w.stripe);
        GFFM_LAUNCH_CHECK("k_plain_rowmajor");
        return GFFM_OK;
    }
    // column-major view: C^T (cols x rows) -= Y^T (cols x k) * X^T (k x rows)
    limb::Layout g = limb::layout(cols, rows, k, N);
    int st = limb::split_a<int32_t>(Y, ldy, cols, k, w.dA, g, N, s);
    if (st) return st;
    st = limb::split_b<int32_t>(X, ldx, k, rows, w.dB, g, N, s);
    if (st) return st;
    return limb::gemm_digits(g, w.dA, w.dB, cols, rows, k, N, C, ldc, epi, 0, s);
}

// Apply a composed row permutation to columns [0, c_left) and [c_lo, c_hi) of W.
static int permute_rows2(const Work &w, const PermArgs &perm, int c_left, int c_lo, int c_hi, cudaStream_t s) {
    if (perm.K == 0) return GFFM_OK;
    const int nb = (c_left + 31) / 32 + (c_hi > c_lo ? (c_hi - c_lo + 31) / 32 : 0);
    if (nb == 0) return GFFM_OK;
    k_rows_permute<<<nb, 256, (size_t)perm.K * 32 * 4, s>>>(w.W, w.ldw, c_left, c_lo, c_hi > c_lo ? c_hi : c_lo, perm);
    GFFM_LAUNCH_CHECK("k_rows_permute");
    return GFFM_OK;
}

// rows the cooperative panel holds in shared memory (one CTA per SM, PANEL_MAX_R rows each)
static int panel_capacity() { return std::min(gffm::sm_count(), MAX_PANEL_CTAS) * PANEL_MAX_R; }
// the width of a panel with `rows` rows from its first pivot row down
static int panel_width(int rows) { return rows <= P1_MAX_ROWS ? P1_NB : (rows <= panel_capacity() ? NB : TALL_NB); }

// a panel with more rows below it than the cooperative panel holds: TALL_NB columns, right-looking
static int tall_panel(Work &w, int m, int R0, int C0, int nbw, const ModP &M, int lcols_check, cudaStream_t s) {
    using namespace gffm;
    // the kernels' key, state and scaled pivot row live in the (otherwise idle) exchange area
    uint8_t *ex = reinterpret_cast<uint8_t *>(w.old_row);
    TallArgs a;
    a.W = w.W;
    a.ldw = w.ldw;
    a.m = m;
    a.R0 = R0;
    a.C0 = C0;
    a.nbw = nbw;
    a.M = M;
    a.l_cols = lcols_check;
    a.key = reinterpret_cast<unsigned long long *>(ex);
    a.state = reinterpret_cast<int *>(ex + 64);
    a.urow = reinterpret_cast<uint32_t *>(ex + 128);
    a.piv_row = w.piv_row;
    a.piv_val = w.piv_val;
    a.piv_inv = w.piv_inv;
    a.linv = w.linv;
    a.result = w.result;
    GFFM_CUDA(cudaMemsetAsync(ex, 0, 128, s));
    const int rows = m - R0;
    const int tmax = std::min(nbw, rows);
    const int sms = sm_count();
    const unsigned search_blocks = (unsigned)std::min<int64_t>((rows + 255) / 256, 4 * sms);
    const unsigned update_blocks = (unsigned)std::min<int64_t>((rows + 7) / 8, 8 * sms);
    for (int t = 0; t < tmax; t++) {
        k_tall_search<<<search_blocks, 256, 0, s>>>(a, t);
        k_tall_pivot<<<1, TALL_NB, 0, s>>>(a, t);
        k_tall_update<<<update_blocks, 256, 0, s>>>(a, t);
    }
    k_tall_finish<<<1, 32, 0, s>>>(a, tmax);
    GFFM_LAUNCH_CHECK("k_tall_*");
    return GFFM_OK;
}

static int run_panel(Work &w, int m, int n, int R0, int C0, int nbw, const ModP &M, int lcols_check,
                     cudaStream_t s, void *stage, int h_res[2], std::vector<int32_t> &h_prow, std::vector<int32_t> &h_pv,
                     int max_g = 0) {
    using namespace gffm;
    const int rows = m - R0;
    const int sms = sm_count();
    const bool tall = rows > panel_capacity();
    if (tall && nbw > TALL_NB) return set_error(GFFM_ERR_ARG, "elimination: a tall panel is at most %d columns", TALL_NB);
    // rows per CTA: at least 64, and at most 128 CTAs while the rows fit; at most
    // max_g CTAs when the panel shares the GPU with a trailing update
    int R = 64;
    if (max_g > 0) {
        while ((rows + R - 1) / R > max_g && R < PANEL_MAX_R) R += 32;
    } else {
        while ((rows + R - 1) / R > std::min(sms, 128) && R < PANEL_MAX_R) R += 32;
    }
    const int G = std::max(1, (rows + R - 1) / R);
    const bool one = rows <= P1_MAX_ROWS && nbw <= P1_NB;   // the whole panel in one CTA
    const size_t smem = one ? p1_smem_bytes(rows) : panel_smem_bytes(R);
    if (tall) {
        int st = tall_panel(w, m, R0, C0, nbw, M, lcols_check, s);
        if (st) return st;
    } else if (!one) {
        GFFM_CUDA(cudaMemsetAsync(w.old_row, 0, exchange_bytes(G), s));
    }
    PanelArgs a;
    a.W = w.W;
    a.ldw = w.ldw;
    a.m = m;
    a.n = n;
    a.R0 = R0;
    a.C0 = C0;
    a.nbw = nbw;
    a.R = R;
    a.M = M;
    a.l_cols = lcols_check;
    a.rec = w.rec;
    a.old_row = w.old_row;
    a.piv_row = w.piv_row;
    a.piv_val = w.piv_val;
    a.piv_inv = w.piv_inv;
    a.linv = w.linv;
    a.result = w.result;
    a.err = device_error_flag();
    if (tall) {
        // factored above
    } else if (one) {
        GFFM_CUDA(ensure_dynamic_smem<k_panel1>((int)smem));
        k_panel1<<<1, P1_THREADS, smem, s>>>(a);
        GFFM_LAUNCH_CHECK("k_panel1");
    } else {
        GFFM_CUDA(ensure_dynamic_smem<k_panel>((int)smem));
        void *args[] = {&a};
        GFFM_CUDA(cudaLaunchCooperativeKernel((void *)k_panel, dim3(G), dim3(PANEL_THREADS), args, smem, s));
    }
    // pivot rows, values and the status: consecutive workspace regions, one copy into
    // pinned memory
    const char *b0 = reinterpret_cast<const char *>(w.piv_row);
    const size_t span = (size_t)(reinterpret_cast<const char *>(w.result + 2) - b0);
    GFFM_CUDA(cudaMemcpyAsync(stage, b0, span, cudaMemcpyDeviceToHost, s));
    GFFM_CUDA(cudaStreamSynchronize(s));
    const char *sb = static_cast<const char *>(stage);
    std::memcpy(h_prow.data(), sb, NB * sizeof(int32_t));
    std::memcpy(h_pv.data(), sb + (reinterpret_cast<const char *>(w.piv_val) - b0), NB * sizeof(int32_t));
    std::memcpy(h_res, sb + (reinterpret_cast<const char *>(w.result) - b0), 2 * sizeof(int));
    return GFFM_OK;
}

// Forward elimination shared by PLUQ / LU / RREF.
// Lookahead: while the next panel factors on a few CTAs (one CTA once its rows fit
// one), the trailing update of the
// columns past it runs beside it on the other SMs (a second stream).  The next
// panel's own columns are updated first, on the whole GPU.
// The panel beside a side update takes at least 64 rows a CTA and at most 48 CTAs unless
// its rows need more (48 measured best on a 16384^2 factorization among caps 24 to 64).
static int look_ctas(int rows) {
    const int gmin = (rows + PANEL_MAX_R - 1) / PANEL_MAX_R;   // the panel's rows per CTA
    return std::max(gmin, std::min(48, (rows + 63) / 64));
}

struct Lookahead {
    cudaStream_t s = nullptr, s2 = nullptr;
    cudaEvent_t ea = nullptr, eb = nullptr;
    bool pending = false;   // the side update is in flight on s2
    int next_g = 0;         // CTA cap of the panel that runs beside it
    // the side update's product, for a second launch on the panel's SMs once the panel is
    // done: both launches draw tiles from one counter
    limb::Layout g;
    int rest = 0, rows_b = 0, k = 0;
    int32_t *C = nullptr;
    int *tiles = nullptr;
    ~Lookahead() {          // every exit path: s (and the workspace's release on it) follows s2
        if (pending) cudaStreamWaitEvent(s, eb, 0);
        if (ea) cudaEventDestroy(ea);
        if (eb) cudaEventDestroy(eb);
        if (s2) cudaStreamDestroy(s2);
    }
    int join() {
        if (pending) GFFM_CUDA(cudaStreamWaitEvent(s, eb, 0));
        pending = false;
        next_g = 0;
        return GFFM_OK;
    }
};

// A22 -= L21 U12 for the rows below the panel: the next panel's NB columns on s with
// every SM, then the remaining columns on s2 with all SMs but the next panel's.  The
// digit planes of L21 are split once and shared.
static int update_lookahead(Work &w, int64_t N, int row, int t, int col, int cs, int m, int n, int look,
                            Lookahead &la) {
    const int rows_b = m - row - t, rest = n - cs - look;
    const int32_t *X = w.W + (int64_t)(row + t) * w.ldw + col;   // L21: rows_b x t
    const int32_t *Y = w.W + (int64_t)row * w.ldw + cs;          // U12: t x (n - cs)
    int32_t *C = w.W + (int64_t)(row + t) * w.ldw + cs;
    const limb::Layout ga = limb::layout(look, rows_b, t, N), gb = limb::layout(rest, rows_b, t, N);
    int st = limb::split_b<int32_t>(X, w.ldw, t, rows_b, w.dB, gb, N, la.s);
    if (st) return st;
    st = limb::split_a<int32_t>(Y, w.ldw, look, t, w.dA2, ga, N, la.s);
    if (st) return st;
    st = limb::split_a<int32_t>(Y + look, w.ldw, rest, t, w.dA, gb, N, la.s);
    if (st) return st;
    st = limb::gemm_digits(ga, w.dA2, w.dB, look, rows_b, t, N, C, w.ldw, limb::EPI_SUB_I32, 0, la.s);
    if (st) return st;
    if (!la.s2) {
        GFFM_CUDA(cudaStreamCreateWithFlags(&la.s2, cudaStreamNonBlocking));
        GFFM_CUDA(cudaEventCreateWithFlags(&la.ea, cudaEventDisableTiming));
        GFFM_CUDA(cudaEventCreateWithFlags(&la.eb, cudaEventDisableTiming));
    }
    GFFM_CUDA(cudaEventRecord(la.ea, la.s));
    GFFM_CUDA(cudaStreamWaitEvent(la.s2, la.ea, 0));
    la.next_g = rows_b <= P1_MAX_ROWS ? 1 : look_ctas(rows_b);   // the next panel's CTAs
    // the side update takes its tiles from a counter: once the panel is done, a second launch
    // on the panel's SMs (help_side_update) shares the rest
    la.tiles = w.result + 8;
    GFFM_CUDA(cudaMemsetAsync(la.tiles, 0, sizeof(int), la.s2));
    la.g = gb;
    la.rest = rest;
    la.rows_b = rows_b;
    la.k = t;
    la.C = C + look;
    st = limb::gemm_digits(gb, w.dA, w.dB, rest, rows_b, t, N, C + look, w.ldw, limb::EPI_SUB_I32,
                           gffm::sm_count() - la.next_g, la.s2, nullptr, nullptr, la.tiles);
    if (st) return st;
    GFFM_CUDA(cudaEventRecord(la.eb, la.s2));
    la.pending = true;
    return GFFM_OK;
}

// After the panel that ran beside a side update: the same product again on the panel's SMs
// (stream s), drawing the tiles the side update has not taken yet.
static int help_side_update(Work &w, int64_t N, Lookahead &la) {
    if (!la.pending || !la.tiles || la.next_g <= 0) return GFFM_OK;
    return limb::gemm_digits(la.g, w.dA, w.dB, la.rest, la.rows_b, la.k, N, la.C, w.ldw, limb::EPI_SUB_I32, la.next_g,
                             la.s, nullptr, nullptr, la.tiles);
}

static int forward(Work &w, int m, int n, int64_t N, int mode, int lcols, cudaStream_t s, Result &res) {
    using namespace gffm;
    ModP M{(uint32_t)N, ~uint64_t(0) / (uint64_t)N};
    const int last = n - 1;
    std::vector<int> skipped;  // PLUQ: columns holding a swapped-in column that is never eliminated
    std::vector<int32_t> h_prow(NB), h_pv(NB);
    int h_res[2];
    // pinned staging for the panel results (pivot rows, values, inverses, status),
    // allocated once per host thread
    struct Stage {
        void *p = nullptr;
        ~Stage() {
            if (p) cudaFreeHost(p);
        }
    };
    static thread_local Stage stage;
    if ((size_t)(reinterpret_cast<const char *>(w.result + 2) - reinterpret_cast<const char *>(w.piv_row)) > 4096 ||
        reinterpret_cast<const char *>(w.piv_val) < reinterpret_cast<const char *>(w.piv_row) ||
        reinterpret_cast<const char *>(w.result) < reinterpret_cast<const char *>(w.piv_val))
        return set_error(GFFM_ERR_WORKSPACE, "elimination: panel result regions are not consecutive");
    if (!stage.p) GFFM_CUDA(cudaMallocHost(&stage.p, 4096));
    int row = 0, col = 0;
    res.perm.resize(m);
    for (int i = 0; i < m; i++) res.perm[i] = i;
    Lookahead la;   // its stream and events are created on first use
    la.s = s;
    const bool use_look = !w.plain;
    while (row < m && col < n) {
        // panels of 32 in one CTA once the rows fit it, of NB across CTAs before, of
        // TALL_NB in global memory while the rows exceed the cooperative panel's capacity
        const int nbw = std::min(panel_width(m - row), n - col);
        int st = run_panel(w, m, n, row, col, nbw, M, mode == MODE_PLUQ ? lcols : 0, s, stage.p, h_res, h_prow, h_pv,
                           la.pending ? la.next_g : 0);
        if (st) return st;
        // the panel's SMs are free: they take over the side update's remaining tiles
        st = help_side_update(w, N, la);
        if (st) return st;
        // everything after the panel may touch the columns the side update writes
        st = la.join();
        if (st) return st;
        const int t = h_res[0], status = h_res[1];
        if (status == PS_TIMEOUT) return set_error(GFFM_ERR_TIMEOUT, "elimination panel: a device-side wait gave up");
        for (int q = 0; q < t; q++) {
            const int r = row + q, p = h_prow[q];
            if (p != r) {
                res.row_swaps.push_back(r + 1);
                res.row_swaps.push_back(p + 1);
                res.swap_step.push_back((int)res.piv_r.size());
                std::swap(res.perm[r], res.perm[p]);
            }
            res.piv_r.push_back(r);
            res.piv_c.push_back(col + q);
            res.piv_v.push_back(h_pv[q]);
        }
        if (t > 0) {
            // the panel's row swaps composed into one permutation of the rows involved
            PermArgs perm;
            {
                // rows row .. row+t-1 sit at positions 0 .. t-1; the (at most t) rows
                // below them that a swap touches follow, found through a small map
                std::vector<int32_t> rows_inv;
                std::unordered_map<int32_t, int> extra;
                for (int q = 0; q < t; q++) rows_inv.push_back(row + q);
                for (int q = 0; q < t; q++)
                    if (h_prow[q] >= row + t && extra.emplace(h_prow[q], (int)rows_inv.size()).second)
                        rows_inv.push_back(h_prow[q]);
                std::vector<int32_t> content(rows_inv.size());
                for (size_t k = 0; k < rows_inv.size(); k++) content[k] = (int32_t)k;
                auto pos = [&](int32_t rr) { return rr < row + t ? (int)(rr - row) : extra.at(rr); };
                for (int q = 0; q < t; q++) std::swap(content[pos(row + q)], content[pos(h_prow[q])]);
                perm.K = (int)rows_inv.size();
                for (int k = 0; k < perm.K; k++) {
                    perm.rows[k] = rows_inv[k];
                    perm.src[k] = content[k];
                }
            }
            // columns left of the panel: multipliers of earlier pivots and skipped columns
            // (W keeps every multiplier column permuted for the arithmetic; the reference's
            // narrower L swap width is restored when L is extracted)
            // and the trailing columns: one launch
            const int left_hi = col;
            const int cs = col + nbw;
            st = permute_rows2(w, perm, left_hi, cs, n, s);
            if (st) return st;
            if (!skipped.empty()) {
                // skipped columns hold A values: row swaps at every width, then the
                // pivot-row scaling (later swaps never touch a finished pivot row)
                const int nq = (int)skipped.size();
                k_skipped<<<(nq + 127) / 128, 128, 0, s>>>(w.W, w.ldw, w.qlist, nq, left_hi, row, t, w.piv_row,
                                                             w.piv_inv, M);
                GFFM_LAUNCH_CHECK("k_skipped");
            }
            // trailing columns (swapped above): triangular solve, update of the rows below
            if (cs < n) {
                // U12 = L11^{-1} P A12 (the panel has written L11^{-1})
                st = rowmajor_gemm(w, N, w.W + (int64_t)row * w.ldw + cs, w.ldw, w.linv, NB,
                                   w.W + (int64_t)row * w.ldw + cs, w.ldw, t, n - cs, t, limb::EPI_STORE_I32, s);
                if (st) return st;
                if (row + t < m) {
                    const int look = panel_width(m - row - t);   // the next panel's width
                    if (use_look && t == nbw && n - cs > look && m - row - t >= 1024 &&
                        m - row - t <= panel_capacity())
                        st = update_lookahead(w, N, row, t, col, cs, m, n, look, la);
                    else
                        st = rowmajor_gemm(w, N, w.W + (int64_t)(row + t) * w.ldw + cs, w.ldw,
                                           w.W + (int64_t)(row + t) * w.ldw + col, w.ldw,
                                           w.W + (int64_t)row * w.ldw + cs, w.ldw, m - row - t, n - cs, t,
                                           limb::EPI_SUB_I32, s);
                    if (st) return st;
                }
            }
            row += t;
            col += t;
        }
        if (status == PS_BOUNDS)
            return set_error(GFFM_ERR_BOUNDS, "pluq: pivot column %d is outside L's padded width %d (the reference "
                                              "raises a BoundsError here)", col + 1, lcols);
        if (status == PS_ZERO_COL && t == 0 && row < m) {
            // A zero column with nothing eliminated: if everything below `row` is zero (a
            // rank-deficient tail) every remaining column is a zero column -- finish in one
            // step: the swap sequence (col, last), (col+1, last), ... as one permutation.
            const int ncols = n - col;
            if ((size_t)ncols * 4 <= 200 * 1024) {
                GFFM_CUDA(cudaMemsetAsync(w.result, 0, sizeof(int), s));
                const int64_t total = (int64_t)(m - row) * ncols;
                const unsigned blocks = (unsigned)std::min<int64_t>((total + 255) / 256, 4 * sm_count());
                k_any_nonzero<<<blocks, 256, 0, s>>>(w.W, w.ldw, row, m, col, n, w.result);
                GFFM_LAUNCH_CHECK("k_any_nonzero");
                int nz = 1;
                GFFM_CUDA(cudaMemcpyAsync(&nz, w.result, sizeof(int), cudaMemcpyDeviceToHost, s));
                GFFM_CUDA(cudaStreamSynchronize(s));
                if (!nz) {
                    if (mode == MODE_PLUQ) {
                        std::vector<int32_t> src(ncols);
                        for (int j = 0; j < ncols; j++) src[j] = col + j;
                        for (int c = col; c <= last; c++) {
                            std::swap(src[c - col], src[last - col]);
                            res.col_swaps.push_back(c + 1);
                            res.col_swaps.push_back(last + 1);
                            skipped.push_back(c);
                        }
                        GFFM_CUDA(cudaMemcpyAsync(w.qlist, src.data(), ncols * sizeof(int32_t),
                                                  cudaMemcpyHostToDevice, s));
                        GFFM_CUDA(cudaFuncSetAttribute(k_permute_cols, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                       ncols * 4));
                        k_permute_cols<<<m, 256, (size_t)ncols * 4, s>>>(w.W, w.ldw, col, ncols, w.qlist);
                        GFFM_LAUNCH_CHECK("k_permute_cols");
                        GFFM_CUDA(cudaStreamSynchronize(s));     // src outlives the copy
                    }
                    col = n;
                    continue;
                }
            }
        }
        if (status == PS_ZERO_COL && t == 0) {
            if (mode == MODE_PLUQ) {
                // find_pivot: swap the zero column with the last column, push (col, cols), skip
                k_colswap<<<(m + 255) / 256, 256, 0, s>>>(w.W, w.ldw, m, col, last);
                GFFM_LAUNCH_CHECK("k_colswap");
                res.col_swaps.push_back(col + 1);
                res.col_swaps.push_back(last + 1);
                skipped.push_back(col);
                const int32_t q = col;
                GFFM_CUDA(cudaMemcpyAsync(w.qlist + skipped.size() - 1, &q, sizeof(int32_t), cudaMemcpyHostToDevice, s));
                GFFM_CUDA(cudaStreamSynchronize(s));
            }
            col += 1;
        }
    }
    res.rank = (int)res.piv_r.size();
    return GFFM_OK;
}

// RREF backward phase on W (multipliers already zeroed): blocks of NB pivots
// from the bottom; each block is reduced in place, then the rows above lose
// their entries in the block's pivot columns through one GEMM update.
static int backward(Work &w, int m, int n, int64_t N, const Result &res, cudaStream_t s) {
    using namespace gffm;
    ModP M{(uint32_t)N, ~uint64_t(0) / (uint64_t)N};
    const int r = res.rank;
    for (int end = r; end > 0; end -= RB) {
        const int p0 = std::max(0, end - RB);
        const int nbp = end - p0;
        std::vector<int32_t> pc(nbp);
        for (int i = 0; i < nbp; i++) pc[i] = res.piv_c[p0 + i];
        GFFM_CUDA(cudaMemcpyAsync(w.pcol, pc.data(), nbp * sizeof(int32_t), cudaMemcpyHostToDevice, s));
        k_gather_cols<<<1, 64, 0, s>>>(w.W, w.ldw, p0, nbp, nbp, w.pcol, w.coef);
        GFFM_LAUNCH_CHECK("k_gather_cols(coef)");
        const int c0 = pc[0];
        k_rref_block<<<(n - c0 + 127) / 128, 128, 0, s>>>(w.W, w.ldw, p0, nbp, w.pcol, w.coef, n, M);
        GFFM_LAUNCH_CHECK("k_rref_block");
        if (p0 > 0) {
            k_gather_cols<<<(p0 + 127) / 128, 128, 0, s>>>(w.W, w.ldw, 0, p0, nbp, w.pcol, w.gather);
            GFFM_LAUNCH_CHECK("k_gather_cols");
            int st = rowmajor_gemm(w, N, w.W + c0, w.ldw, w.gather, RB, w.W + (int64_t)p0 * w.ldw + c0, w.ldw,
                                   p0, n - c0, nbp, limb::EPI_SUB_I32, s);
            if (st) return st;
        }
        // the host vector pc must outlive the async copy
        GFFM_CUDA(cudaStreamSynchronize(s));
    }
    return GFFM_OK;
}

static int check_common(int64_t m, int64_t n, int64_t lda, int64_t N) {
    using gffm::set_error;
    if (m < 0 || n < 0) return set_error(GFFM_ERR_ARG, "negative matrix size");
    if (m > (int64_t(1) << 24) || n > (int64_t(1) << 24)) return set_error(GFFM_ERR_ARG, "matrix dimension above 2^24");
    if (lda < (m > 1 ? m : 1)) return set_error(GFFM_ERR_ARG, "leading dimension smaller than the number of rows");
    if (N < 2 || N >= (int64_t(1) << 26))
        return set_error(GFFM_ERR_MODULUS, "elimination needs 2 <= N < 2^26 (got %lld)", (long long)N);
    return GFFM_OK;
}

template <typename T>
static int load(Work &w, const T *A, int64_t lda, int64_t m, int64_t n, int64_t N, cudaStream_t s) {
    ModP M{(uint32_t)N, ~uint64_t(0) / (uint64_t)N};
    dim3 grid((unsigned)((n + 31) / 32), (unsigned)((m + 31) / 32));
    k_to_rowmajor<T><<<grid, 256, 0, s>>>(A, lda, (int)m, (int)n, w.W, w.ldw, M);
    GFFM_LAUNCH_CHECK("k_to_rowmajor");
    return GFFM_OK;
}

template <typename T>
static int extract_u(Work &w, int64_t m, int64_t n, const Result &res, bool zero_multipliers, T *U, int64_t ldu,
                     cudaStream_t s) {
    std::vector<int32_t> colpiv(n > 0 ? n : 1, -1);
    if (zero_multipliers)
        for (size_t q = 0; q < res.piv_c.size(); q++) colpiv[res.piv_c[q]] = res.piv_r[q];
    GFFM_CUDA(cudaMemcpyAsync(w.colpiv, colpiv.data(), colpiv.size() * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    dim3 grid((unsigned)((n + 31) / 32), (unsigned)((m + 31) / 32));
    k_extract_u<T><<<grid, 256, 0, s>>>(w.W, w.ldw, (int)m, (int)n, w.colpiv, U, ldu);
    GFFM_LAUNCH_CHECK("k_extract_u");
    GFFM_CUDA(cudaStreamSynchronize(s));
    return GFFM_OK;
}

// mode PLUQ: L column c_s <- pivot s;  mode LU: L column s <- pivot s
template <typename T>
static int extract_l(Work &w, int64_t m, int64_t lcols, const Result &res, int mode, T *L, int64_t ldl,
                     cudaStream_t s) {
    if (m == 0 || lcols == 0) return GFFM_OK;
    std::vector<int32_t> h(3 * lcols, -1);
    for (size_t q = 0; q < res.piv_c.size(); q++) {
        const int64_t c = mode == MODE_PLUQ ? res.piv_c[q] : (int64_t)q;
        if (c >= lcols) continue;
        h[c] = res.piv_c[q];
        h[lcols + c] = res.piv_r[q];
        h[2 * lcols + c] = res.piv_v[q];
    }
    GFFM_CUDA(cudaMemcpyAsync(w.lsrc, h.data(), lcols * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    GFFM_CUDA(cudaMemcpyAsync(w.lrow, h.data() + lcols, lcols * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    GFFM_CUDA(cudaMemcpyAsync(w.lpv, h.data() + 2 * lcols, lcols * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    dim3 grid((unsigned)((m + 255) / 256), (unsigned)std::min<int64_t>(lcols, 4096));
    k_extract_l<T><<<grid, 256, 0, s>>>(w.W, w.ldw, (int)m, (int)lcols, w.lsrc, w.lrow, w.lpv, L, ldl);
    GFFM_LAUNCH_CHECK("k_extract_l");
    GFFM_CUDA(cudaStreamSynchronize(s));
    return GFFM_OK;
}

template <typename T>
int pluq(int64_t m, int64_t n, const T *A, int64_t lda, T *U, int64_t ldu, T *L, int64_t ldl, int64_t lcols,
         int64_t N, int64_t *row_swaps, int64_t *n_row_swaps, int64_t *col_swaps, int64_t *n_col_swaps,
         int64_t *rank, void *ws, size_t ws_bytes, gffm_stream_t stream, int mode, int64_t *perm,
         bool plain = false) {
    using namespace gffm;
    int st = check_common(m, n, lda, N);
    if (st) return st;
    if (ldu < (m > 1 ? m : 1) || (L && ldl < (m > 1 ? m : 1)))
        return set_error(GFFM_ERR_ARG, "leading dimension smaller than the number of rows");
    if (lcols < 0 || (L && lcols < m)) return set_error(GFFM_ERR_ARG, "L needs at least m columns");
    if (!rank) return set_error(GFFM_ERR_ARG, "rank is NULL");
    if (mode == MODE_PLUQ && (!row_swaps || !n_row_swaps || !col_swaps || !n_col_swaps))
        return set_error(GFFM_ERR_ARG, "swap stack buffers are NULL");
    if (mode == MODE_LU && !perm) return set_error(GFFM_ERR_ARG, "perm is NULL");
    if (mode == MODE_RREF && !is_prime_u32((uint32_t)N))
        return set_error(GFFM_ERR_NOT_PRIME, "the reduced row echelon form needs a prime modulus (%lld is composite)",
                         (long long)N);
    if ((m > 0 && n > 0) && (!A || !U)) return set_error(GFFM_ERR_ARG, "null data pointer");
    *rank = 0;
    if (n_row_swaps) *n_row_swaps = 0;
    if (n_col_swaps) *n_col_swaps = 0;
    if (mode == MODE_LU)
        for (int64_t i = 0; i < m; i++) perm[i] = i + 1;
    st = check_device();
    if (st) return st;
    cudaStream_t s = as_stream(stream);
    if (m == 0 || n == 0) {
        if (L && m > 0 && lcols > 0)
            GFFM_CUDA(cudaMemset2DAsync(L, (size_t)ldl * sizeof(T), 0, (size_t)m * sizeof(T), (size_t)lcols, s));
        GFFM_CUDA(cudaStreamSynchronize(s));
        return GFFM_OK;
    }
    Scratch scr;
    st = scr.acquire(ws, ws_bytes, workspace_bytes(m, n, std::max<int64_t>(lcols, 1)), s);
    if (st) return st;
    Work w;
    bind_ws(scr.ptr, m, n, std::max<int64_t>(lcols, 1), &w);
    w.plain = plain ? 1 : 0;
    if (plain) {
        // find_max_stripe_ops(Float64, N) = floor((2^53 - 1) / (N - 1)^2) - 1 (stripe_mul.jl:13-27)
        const unsigned __int128 den = (unsigned __int128)(N - 1) * (unsigned __int128)(N - 1);
        w.stripe = std::max<int64_t>(1, (int64_t)((((unsigned __int128)1 << 53) - 1) / den) - 1);
    }
    st = load<T>(w, A, lda, m, n, N, s);
    if (st) return st;
    Result res;
    st = forward(w, (int)m, (int)n, N, mode, (int)(mode == MODE_PLUQ ? lcols : 0), s, res);
    if (st) {
        cudaStreamSynchronize(s);
        return st;
    }
    if (mode == MODE_RREF) {
        std::vector<int32_t> colpiv(n, -1);
        for (size_t q = 0; q < res.piv_c.size(); q++) colpiv[res.piv_c[q]] = res.piv_r[q];
        GFFM_CUDA(cudaMemcpyAsync(w.colpiv, colpiv.data(), n * sizeof(int32_t), cudaMemcpyHostToDevice, s));
        dim3 grid((unsigned)((m + 255) / 256), (unsigned)std::min<int64_t>(n, 4096));
        k_zero_below<<<grid, 256, 0, s>>>(w.W, w.ldw, (int)m, (int)n, w.colpiv);
        GFFM_LAUNCH_CHECK("k_zero_below");
        GFFM_CUDA(cudaStreamSynchronize(s));
        st = backward(w, (int)m, (int)n, N, res, s);
        if (st) return st;
        st = extract_u<T>(w, m, n, res, false, U, ldu, s);
        if (st) return st;
        if (row_swaps) {  // pivot columns (1-based), when asked for
            for (int q = 0; q < res.rank; q++) row_swaps[q] = res.piv_c[q] + 1;
        }
    } else {
        st = extract_u<T>(w, m, n, res, true, U, ldu, s);
        if (st) return st;
        if (L) {
            st = extract_l<T>(w, m, lcols, res, mode, L, ldl, s);
            if (st) return st;
            if (mode == MODE_PLUQ) {
                // The reference swaps L's rows only over columns 1..32*cld(rows, 32)
                // (swap_rows launch, pluq_kernels.jl:254): a pivot column past that width
                // keeps the row order of its own step.  W permuted every column, so undo
                // the later swaps on those (rare) columns.
                const int64_t lsw = std::min<int64_t>((m + 31) / 32 * 32, lcols);
                std::vector<T> colbuf(m);
                for (size_t q = 0; q < res.piv_c.size(); q++) {
                    const int64_t c = res.piv_c[q];
                    if (c < lsw || c >= lcols) continue;
                    GFFM_CUDA(cudaMemcpy(colbuf.data(), L + c * ldl, m * sizeof(T), cudaMemcpyDeviceToHost));
                    for (int64_t k = (int64_t)res.swap_step.size() - 1; k >= 0; k--) {
                        if (res.swap_step[k] <= (int)q) break;
                        std::swap(colbuf[res.row_swaps[2 * k] - 1], colbuf[res.row_swaps[2 * k + 1] - 1]);
                    }
                    GFFM_CUDA(cudaMemcpy(L + c * ldl, colbuf.data(), m * sizeof(T), cudaMemcpyHostToDevice));
                }
            }
        }
        if (mode == MODE_PLUQ) {
            std::copy(res.row_swaps.begin(), res.row_swaps.end(), row_swaps);
            std::copy(res.col_swaps.begin(), res.col_swaps.end(), col_swaps);
            *n_row_swaps = (int64_t)res.row_swaps.size() / 2;
            *n_col_swaps = (int64_t)res.col_swaps.size() / 2;
        } else {
            for (int64_t i = 0; i < m; i++) perm[i] = res.perm[i] + 1;
        }
    }
    *rank = res.rank;
    return GFFM_OK;
}

// A^{-1} mod N from the reduced row echelon form of [A | I]: A is invertible exactly when
// the pivots of the RREF are the first n columns, and then the right half is A^{-1}
// (unique, so any elimination order gives the reference's result).
template <typename T>
int inverse(int64_t n, const T *A, int64_t lda, T *Ainv, int64_t ldi, int64_t N, int *invertible, void *ws,
            size_t ws_bytes, gffm_stream_t stream) {
    using namespace gffm;
    if (!invertible) return set_error(GFFM_ERR_ARG, "invertible is NULL");
    *invertible = 0;
    if (n < 0) return set_error(GFFM_ERR_ARG, "negative size");
    if (lda < std::max<int64_t>(n, 1) || ldi < std::max<int64_t>(n, 1))
        return set_error(GFFM_ERR_ARG, "leading dimension smaller than the number of rows");
    if (n == 0) {
        *invertible = 1;
        return GFFM_OK;
    }
    if (!A || !Ainv) return set_error(GFFM_ERR_ARG, "null data pointer");
    int st = check_device();
    if (st) return st;
    cudaStream_t s = as_stream(stream);
    const int64_t ld = n;
    const size_t aug_bytes = gffm::round_up((int64_t)((size_t)n * 2 * n * sizeof(T)), 256);
    const size_t el_bytes = workspace_bytes(n, 2 * n, 1);
    Scratch scr;
    st = scr.acquire(ws, ws_bytes, aug_bytes + el_bytes, s);
    if (st) return st;
    T *X = static_cast<T *>(scr.ptr);
    void *ews = static_cast<uint8_t *>(scr.ptr) + aug_bytes;
    const int64_t total = n * 2 * n;
    k_build_augmented<T><<<(unsigned)((total + 255) / 256), 256, 0, s>>>(A, lda, (int)n, X, ld);
    GFFM_LAUNCH_CHECK("k_build_augmented");
    std::vector<int64_t> piv((size_t)n);
    int64_t rank = 0;
    st = pluq<T>(n, 2 * n, X, ld, X, ld, nullptr, 1, 0, N, piv.data(), nullptr, nullptr, nullptr, &rank, ews,
                 el_bytes, stream, MODE_RREF, nullptr);
    if (st) return st;
    bool ok = rank >= n;
    for (int64_t i = 0; ok && i < n; i++) ok = piv[(size_t)i] == i + 1;
    if (ok) {
        GFFM_CUDA(cudaMemcpy2DAsync(Ainv, (size_t)ldi * sizeof(T), X + n * ld, (size_t)ld * sizeof(T),
                                    (size_t)n * sizeof(T), (size_t)n, cudaMemcpyDeviceToDevice, s));
    }
    *invertible = ok ? 1 : 0;
    return GFFM_OK;
}

}  // namespace elim

extern "C" {

int gffm_inverse_workspace_size(int64_t n, size_t *bytes) {
    if (!bytes) return gffm::set_error(GFFM_ERR_ARG, "bytes is NULL");
    if (n < 0) return gffm::set_error(GFFM_ERR_ARG, "negative size");
    *bytes = n == 0 ? 0
                    : gffm::round_up((int64_t)((size_t)n * 2 * n * sizeof(double)), 256) +
                          elim::workspace_bytes(n, 2 * n, 1);
    return GFFM_OK;
}

int gffm_inverse_f64(int64_t n, const double *A, int64_t lda, double *Ainv, int64_t ldi, int64_t N, int *invertible,
                     void *ws, size_t ws_bytes, gffm_stream_t s) {
    return elim::inverse<double>(n, A, lda, Ainv, ldi, N, invertible, ws, ws_bytes, s);
}

int gffm_inverse_f32(int64_t n, const float *A, int64_t lda, float *Ainv, int64_t ldi, int64_t N, int *invertible,
                     void *ws, size_t ws_bytes, gffm_stream_t s) {
    return elim::inverse<float>(n, A, lda, Ainv, ldi, N, invertible, ws, ws_bytes, s);
}

int gffm_elim_workspace_size(int64_t m, int64_t n, int64_t l_cols, size_t *bytes) {
    if (!bytes) return gffm::set_error(GFFM_ERR_ARG, "bytes is NULL");
    if (m < 0 || n < 0 || l_cols < 0) return gffm::set_error(GFFM_ERR_ARG, "negative size");
    *bytes = (m == 0 || n == 0) ? 0 : elim::workspace_bytes(m, n, std::max<int64_t>(l_cols, 1));
    return GFFM_OK;
}

int gffm_pluq_f64(int64_t m, int64_t n, const double *A, int64_t lda, double *U, int64_t ldu, double *L, int64_t ldl,
                  int64_t l_cols, int64_t N, int64_t *row_swaps, int64_t *n_row_swaps, int64_t *col_swaps,
                  int64_t *n_col_swaps, int64_t *rank, void *ws, size_t ws_bytes, gffm_stream_t s) {
    if (!L) return gffm::set_error(GFFM_ERR_ARG, "L is NULL");
    return elim::pluq<double>(m, n, A, lda, U, ldu, L, ldl, l_cols, N, row_swaps, n_row_swaps, col_swaps, n_col_swaps,
                              rank, ws, ws_bytes, s, elim::MODE_PLUQ, nullptr);
}

int gffm_pluq_plain_f64(int64_t m, int64_t n, const double *A, int64_t lda, double *U, int64_t ldu, double *L,
                        int64_t ldl, int64_t l_cols, int64_t N, int64_t *row_swaps, int64_t *n_row_swaps,
                        int64_t *col_swaps, int64_t *n_col_swaps, int64_t *rank, void *ws, size_t ws_bytes,
                        gffm_stream_t s) {
    if (!L) return gffm::set_error(GFFM_ERR_ARG, "L is NULL");
    return elim::pluq<double>(m, n, A, lda, U, ldu, L, ldl, l_cols, N, row_swaps, n_row_swaps, col_swaps, n_col_swaps,
                              rank, ws, ws_bytes, s, elim::MODE_PLUQ, nullptr, true);
}

int gffm_pluq_f32(int64_t m, int64_t n, const float *A, int64_t lda, float *U, int64_t ldu, float *L, int64_t ldl,
                  int64_t l_cols, int64_t N, int64_t *row_swaps, int64_t *n_row_swaps, int64_t *col_swaps,
                  int64_t *n_col_swaps, int64_t *rank, void *ws, size_t ws_bytes, gffm_stream_t s) {
    if (!L) return gffm::set_error(GFFM_ERR_ARG, "L is NULL");
    return elim::pluq<float>(m, n, A, lda, U, ldu, L, ldl, l_cols, N, row_swaps, n_row_swaps, col_swaps, n_col_swaps,
                             rank, ws, ws_bytes, s, elim::MODE_PLUQ, nullptr);
}

int gffm_lu_f64(int64_t m, int64_t n, const double *A, int64_t lda, double *U, int64_t ldu, double *L, int64_t ldl,
                int64_t N, int64_t *perm, int64_t *rank, void *ws, size_t ws_bytes, gffm_stream_t s) {
    if (!L) return gffm::set_error(GFFM_ERR_ARG, "L is NULL");
    return elim::pluq<double>(m, n, A, lda, U, ldu, L, ldl, m, N, nullptr, nullptr, nullptr, nullptr, rank, ws,
                              ws_bytes, s, elim::MODE_LU, perm);
}

int gffm_lu_f32(int64_t m, int64_t n, const float *A, int64_t lda, float *U, int64_t ldu, float *L, int64_t ldl,
                int64_t N, int64_t *perm, int64_t *rank, void *ws, size_t ws_bytes, gffm_stream_t s) {
    if (!L) return gffm::set_error(GFFM_ERR_ARG, "L is NULL");
    return elim::pluq<float>(m, n, A, lda, U, ldu, L, ldl, m, N, nullptr, nullptr, nullptr, nullptr, rank, ws,
                             ws_bytes, s, elim::MODE_LU, perm);
}

int gffm_rref_f64(int64_t m, int64_t n, const double *A, int64_t lda, double *R, int64_t ldr, int64_t N,
                  int64_t *rank, int64_t *pivot_cols, void *ws, size_t ws_bytes, gffm_stream_t s) {
    return elim::pluq<double>(m, n, A, lda, R, ldr, nullptr, 1, 0, N, pivot_cols, nullptr, nullptr, nullptr, rank,
                              ws, ws_bytes, s, elim::MODE_RREF, nullptr);
}

int gffm_rref_f32(int64_t m, int64_t n, const float *A, int64_t lda, float *R, int64_t ldr, int64_t N, int64_t *rank,
                  int64_t *pivot_cols, void *ws, size_t ws_bytes, gffm_stream_t s) {
    return elim::pluq<float>(m, n, A, lda, R, ldr, nullptr, 1, 0, N, pivot_cols, nullptr, nullptr, nullptr, rank, ws,
                             ws_bytes, s, elim::MODE_RREF, nullptr);
}

}  // extern "C"
