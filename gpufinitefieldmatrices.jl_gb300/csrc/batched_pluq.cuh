// batched_pluq.cuh -- PLUQ of many independent small matrices with their own
// primes, one CTA per instance at a time (persistent, dynamically scheduled).
//
// Semantics are those of pluq_gpu_kernel (src/CuModMatrix/rref_lu_pluq/
// pluq_kernels.jl:46-157), step for step: the pivot is the largest residue of
// the column below the current row (lowest row on ties); a zero column is
// swapped with the last column, the swap pushed, and the column after it taken
// next; the pivot row is swapped in and scaled by the pivot inverse across every
// column; L receives the pivot at (row, col) and the raw column below; L's row
// swaps cover only its first 32*cld(m, 32) columns; a pivot column at or past
// L's width is the reference's BoundsError (status 8).
//
// Blocking.  The instance lives in global memory as a row-major int32 copy W
// (and LW for L).  A panel of nb columns is copied into shared memory and
// eliminated step by step there (pivot search, row swap, scaling and the
// rank-1 updates restricted to the panel).  The rest of every row is brought
// up to date once per panel: the panel's row swaps composed into one set of
// row moves, then the pivot rows of the trailing columns by forward
// substitution
//     U[t][c] = inv_t * (W[t][c] - sum_{s<t} l[t][s] U[s][c]),
// then the rows below by one K = nb product accumulated exactly in 64 bits
// (products below 2^52, at most 32 of them) and reduced once.  Columns left of
// the panel only see the moves and the pivot-row scaling (they matter for the
// stale columns a zero-column swap leaves behind).  A zero column ends the
// panel early: the pending updates are applied first, so the last column it is
// swapped with is current.
#pragma once

#include "gffm_common.cuh"
#include "modarith.cuh"

namespace batched {

constexpr int PQ_THREADS = 256;
constexpr int PQ_CW = 128;          // trailing columns per chunk
constexpr int PQ_MAX_NB = 32;
constexpr int PQ_MAX_MOVES = 2 * PQ_MAX_NB;

struct PQInst {
    int m, n, l_cols, lsw;       // lsw = min(32*cld(m, 32), l_cols): L's row-swap width
    elim::ModP M;                // N, floor((2^64-1)/N)
    elim::Mont mont;             // pivot inverse (Fermat for prime N, else the reference's Euclid)
    const double *A;
    int64_t lda;
    double *U;
    int64_t ldu;
    double *L;
    int64_t ldl;
    int32_t *W;                  // m x ldw row-major working copy of A
    int32_t *LW;                 // m x ldlw row-major working copy of L's first lwc columns
    int ldw, ldlw, lwc, pad_;
    int64_t *row_swaps, *col_swaps, *info;
};

struct PQArgs {
    const PQInst *inst;
    const int *order;            // instances, largest first
    int count;
    int nb;                      // panel width, <= PQ_MAX_NB
    int rcap;                    // rows of the shared panel (>= every m), multiple of 4
    int *next;                   // dynamic scheduling counter (zeroed before the launch)
    int32_t *tmp;                // per-CTA row-move buffers: PQ_MAX_MOVES rows of W, then of LW
    int tmp_ldw, tmp_ldlw;       // their row strides (>= every ldw / ldlw)
};

// shared-memory words a CTA needs for panel height rcap
__host__ __device__ constexpr size_t pq_smem_words(int rcap) {
    return (size_t)PQ_MAX_NB * (rcap + 4) + (size_t)PQ_MAX_NB * PQ_CW;
}

struct PQShared {
    int piv_prow[PQ_MAX_NB];     // absolute row swapped into pivot row r0 + t
    uint32_t piv_val[PQ_MAX_NB];
    uint32_t piv_inv[PQ_MAX_NB];
    int mv_dst[PQ_MAX_MOVES], mv_src[PQ_MAX_MOVES];
    uint32_t mv_scale[PQ_MAX_MOVES];   // 0: plain move; else the pivot inverse of a pivot row
    unsigned long long red[PQ_THREADS / 32];
    int nmv, inst, stop, zero_hit;
};

__device__ __forceinline__ uint32_t reduce_u64(uint64_t x, const elim::ModP &M) {
    return (uint32_t)gffm_dev::barrett64(x, M.n, M.minv);
}

__device__ __forceinline__ uint32_t residue_of(double v, const elim::ModP &M) {
    const int64_t x = (int64_t)v;
    if (x >= 0 && x < (int64_t)M.n) return (uint32_t)x;
    if (x >= 0) return (uint32_t)gffm_dev::barrett64((uint64_t)x, M.n, M.minv);
    const uint32_t q = (uint32_t)gffm_dev::barrett64((uint64_t)(-x), M.n, M.minv);
    return q ? M.n - q : 0;
}

// Column-major Float64 (m x n, ld) <-> row-major int32 (m x n, ldw) through 32 x 32
// shared tiles (tile = 32 x 33 words of scratch).
__device__ void to_rowmajor(const double *A, int64_t lda, int32_t *W, int ldw, int m, int n, const elim::ModP &M,
                            int32_t *tile) {
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;   // 8 rows of 32 threads
    for (int r0 = 0; r0 < m; r0 += 32)
        for (int c0 = 0; c0 < n; c0 += 32) {
            for (int cc = ty; cc < 32; cc += 8) {
                const int r = r0 + tx, c = c0 + cc;
                tile[cc * 33 + tx] = (r < m && c < n) ? (int32_t)residue_of(A[r + (int64_t)c * lda], M) : 0;
            }
            __syncthreads();
            for (int rr = ty; rr < 32; rr += 8) {
                const int r = r0 + rr, c = c0 + tx;
                if (r < m && c < n) W[(int64_t)r * ldw + c] = tile[tx * 33 + rr];
            }
            __syncthreads();
        }
}

__device__ void to_colmajor(const int32_t *W, int ldw, int wcols, double *A, int64_t lda, int m, int n,
                            int32_t *tile) {
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int r0 = 0; r0 < m; r0 += 32)
        for (int c0 = 0; c0 < n; c0 += 32) {
            for (int rr = ty; rr < 32; rr += 8) {
                const int r = r0 + rr, c = c0 + tx;
                tile[rr * 33 + tx] = (r < m && c < wcols) ? W[(int64_t)r * ldw + c] : 0;
            }
            __syncthreads();
            for (int cc = ty; cc < 32; cc += 8) {
                const int r = r0 + tx, c = c0 + cc;
                if (r < m && c < n) A[r + (int64_t)c * lda] = (double)tile[tx * 33 + cc];
            }
            __syncthreads();
        }
}

// Gather the source rows of the composed row moves (columns [c_lo, c_hi) of a
// row-major int32 matrix) into T (nmv rows of stride ldt) ...
__device__ __forceinline__ void gather_moves(const int32_t *X, int ldx, int c_lo, int c_hi, int32_t *T, int ldt,
                                             const PQShared &S) {
    const int w = c_hi - c_lo;
    if (w <= 0) return;
    for (int idx = threadIdx.x; idx < S.nmv * w; idx += blockDim.x) {
        const int k = idx / w, c = c_lo + (idx - k * w);
        T[(int64_t)k * ldt + c] = X[(int64_t)S.mv_src[k] * ldx + c];
    }
}
// ... and write them to their destinations (times the pivot inverse for pivot rows when `scale`).
__device__ __forceinline__ void scatter_moves(int32_t *X, int ldx, int c_lo, int c_hi, const int32_t *T, int ldt,
                                              const PQShared &S, bool scale, const elim::ModP &M) {
    const int w = c_hi - c_lo;
    if (w <= 0) return;
    for (int idx = threadIdx.x; idx < S.nmv * w; idx += blockDim.x) {
        const int k = idx / w, c = c_lo + (idx - k * w);
        const int32_t v = T[(int64_t)k * ldt + c];
        const uint32_t sc = S.mv_scale[k];
        X[(int64_t)S.mv_dst[k] * ldx + c] = (scale && sc) ? (int32_t)elim::mulmod((uint32_t)v, sc, M) : v;
    }
}

__global__ void __launch_bounds__(PQ_THREADS) k_pluq_batched(PQArgs a) {
    extern __shared__ __align__(16) int32_t pq_smem[];
    __shared__ PQShared S;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int rs = a.rcap + 4;                        // panel column stride (words)
    int32_t *P = pq_smem;                             // P[j * rs + lr]: panel column j, local row lr
    int32_t *Us = pq_smem + (size_t)PQ_MAX_NB * rs;   // Us[t * PQ_CW + c]: pivot rows of a trailing chunk

    for (;;) {
        if (tid == 0) {
            const int k = atomicAdd(a.next, 1);
            S.inst = k < a.count ? a.order[k] : -1;
        }
        __syncthreads();
        const int ii = S.inst;
        if (ii < 0) break;
        const PQInst I = a.inst[ii];
        const int m = I.m, n = I.n;
        const uint32_t N = I.M.n;
        to_rowmajor(I.A, I.lda, I.W, I.ldw, m, n, I.M, Us);
        for (int64_t idx = tid; idx < (int64_t)m * I.ldlw; idx += blockDim.x) I.LW[idx] = 0;
        __syncthreads();

        int row = 0, col = 0, nr = 0, nc = 0, status = 0;
        while (row < m && col < n) {
            const int r0 = row, c0 = col;
            const int R = m - r0;
            const int nbc = min(a.nb, n - c0);
            // ---- panel load: W[r0 + lr][c0 + j] -> P[j][lr] ----
            for (int idx = tid; idx < R * nbc; idx += blockDim.x) {
                const int lr = idx / nbc, j = idx - lr * nbc;
                P[j * rs + lr] = I.W[(int64_t)(r0 + lr) * I.ldw + c0 + j];
            }
            if (tid == 0) {
                S.stop = 0;
                S.zero_hit = 0;
            }
            __syncthreads();
            int npiv = 0;
            for (int j = 0; j < nbc && r0 + npiv < m; j++) {
                // ---- pivot search: largest value, then lowest row ----
                unsigned long long best = 0;
                for (int lr = npiv + tid; lr < R; lr += blockDim.x) {
                    const uint32_t v = (uint32_t)P[j * rs + lr];
                    const unsigned long long key = ((unsigned long long)v << 32) | (0xFFFFFFFFu - (uint32_t)lr);
                    best = key > best ? key : best;
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    const unsigned long long other = __shfl_xor_sync(0xffffffffu, best, o);
                    best = other > best ? other : best;
                }
                if (lane == 0) S.red[warp] = best;
                __syncthreads();
                if (tid == 0) {
                    unsigned long long b = 0;
                    for (int w = 0; w < PQ_THREADS / 32; w++) b = S.red[w] > b ? S.red[w] : b;
                    const uint32_t pv = (uint32_t)(b >> 32);
                    if (pv == 0) {
                        S.zero_hit = 1;
                    } else if (c0 + j >= I.l_cols) {
                        S.stop = 8;              // the reference indexes L out of bounds here
                    } else {
                        S.piv_prow[npiv] = r0 + (int)(0xFFFFFFFFu - (uint32_t)(b & 0xFFFFFFFFu));
                        S.piv_val[npiv] = pv;
                        S.piv_inv[npiv] = elim::mod_inverse(pv, I.mont);
                    }
                }
                __syncthreads();
                if (S.zero_hit || S.stop) break;
                const int plr = S.piv_prow[npiv] - r0;
                const uint32_t inv = S.piv_inv[npiv];
                // ---- swap panel rows npiv <-> plr over every panel column, scaling the pivot
                //      row of the columns not eliminated yet ----
                for (int jj = tid; jj < nbc; jj += blockDim.x) {
                    const int32_t x = P[jj * rs + plr];
                    const int32_t y = P[jj * rs + npiv];
                    P[jj * rs + plr] = y;
                    P[jj * rs + npiv] = jj >= j ? (int32_t)elim::mulmod((uint32_t)x, inv, I.M) : x;
                }
                __syncthreads();
                // ---- rank-1 update of the panel: rows below the pivot, columns right of j ----
                for (int lr = npiv + 1 + tid; lr < R; lr += blockDim.x) {
                    const uint32_t l = (uint32_t)P[j * rs + lr];
                    if (!l) continue;
                    const uint32_t nl = N - l;
                    for (int jj = j + 1; jj < nbc; jj++) {
                        const uint32_t u = (uint32_t)P[jj * rs + npiv];
                        const uint32_t v = (uint32_t)P[jj * rs + lr] + elim::mulmod(nl, u, I.M);
                        P[jj * rs + lr] = (int32_t)(v >= N ? v - N : v);
                    }
                }
                npiv++;
                __syncthreads();
            }
            const int zero_hit = S.zero_hit;
            const int stop = S.stop;
            // ---- compose the panel's swaps into row moves; push the swap stack ----
            if (tid == 0) {
                int rows_[PQ_MAX_MOVES], at[PQ_MAX_MOVES], nrows = 0;
                auto slot = [&](int r) {
                    for (int k = 0; k < nrows; k++)
                        if (rows_[k] == r) return k;
                    rows_[nrows] = r;
                    at[nrows] = r;
                    return nrows++;
                };
                for (int t = 0; t < npiv; t++) {
                    const int r = r0 + t, pr = S.piv_prow[t];
                    const int a1 = slot(r), a2 = slot(pr);
                    const int x = at[a1];
                    at[a1] = at[a2];
                    at[a2] = x;
                    if (pr != r) {
                        I.row_swaps[2 * nr] = r + 1;
                        I.row_swaps[2 * nr + 1] = pr + 1;
                        nr++;
                    }
                }
                int k = 0;
                for (int q = 0; q < nrows; q++) {
                    const int dst = rows_[q];
                    const uint32_t sc = (dst >= r0 && dst < r0 + npiv) ? S.piv_inv[dst - r0] : 0u;
                    if (at[q] == dst && sc == 0) continue;
                    S.mv_dst[k] = dst;
                    S.mv_src[k] = at[q];
                    S.mv_scale[k] = sc;
                    k++;
                }
                S.nmv = k;
            }
            // ---- panel back to W: eliminated columns keep the pivot and above, zero below ----
            for (int idx = tid; idx < R * nbc; idx += blockDim.x) {
                const int lr = idx / nbc, j = idx - lr * nbc;
                I.W[(int64_t)(r0 + lr) * I.ldw + c0 + j] = (j < npiv && lr > j) ? 0 : P[j * rs + lr];
            }
            // ---- L: this panel's columns (pivot, then the multipliers as swapped so far) ----
            for (int idx = tid; idx < R * npiv; idx += blockDim.x) {
                const int t = idx / R, lr = idx - t * R;
                if (lr >= t) I.LW[(int64_t)(r0 + lr) * I.ldlw + c0 + t] = lr == t ? (int32_t)S.piv_val[t] : P[t * rs + lr];
            }
            __syncthreads();
            if (npiv > 0) {
                // the rows the panel's swaps moved, outside the panel: columns left of it (with the
                // pivot-row scaling), trailing columns (moves only; their scaling comes with the
                // substitution below), and L inside its swap width
                int32_t *TW = a.tmp + (size_t)blockIdx.x * PQ_MAX_MOVES * (a.tmp_ldw + a.tmp_ldlw);
                int32_t *TL = TW + (size_t)PQ_MAX_MOVES * a.tmp_ldw;
                const int lsw_left = min(c0, I.lsw);
                gather_moves(I.W, I.ldw, 0, c0, TW, a.tmp_ldw, S);
                gather_moves(I.W, I.ldw, c0 + nbc, n, TW, a.tmp_ldw, S);
                gather_moves(I.LW, I.ldlw, 0, lsw_left, TL, a.tmp_ldlw, S);
                __syncthreads();
                scatter_moves(I.W, I.ldw, 0, c0, TW, a.tmp_ldw, S, true, I.M);
                scatter_moves(I.W, I.ldw, c0 + nbc, n, TW, a.tmp_ldw, S, false, I.M);
                scatter_moves(I.LW, I.ldlw, 0, lsw_left, TL, a.tmp_ldlw, S, false, I.M);
            }
            // L columns at or past the swap width must not see the swaps after their own step
            if (tid == 0) {
                for (int t = 0; t < npiv; t++) {
                    const int c = c0 + t;
                    if (c < I.lsw) continue;
                    for (int s = npiv - 1; s > t; s--) {
                        const int r = r0 + s, pr = S.piv_prow[s];
                        if (pr == r) continue;
                        int32_t *x = I.LW + (int64_t)r * I.ldlw + c;
                        int32_t *y = I.LW + (int64_t)pr * I.ldlw + c;
                        const int32_t tmp = *y;
                        *y = *x;
                        *x = tmp;
                    }
                }
            }
            __syncthreads();
            // ---- trailing columns: pivot rows by substitution, rows below by one product ----
            const int ct0 = c0 + nbc;
            for (int cb = ct0; npiv > 0 && cb < n; cb += PQ_CW) {
                const int cw = min(PQ_CW, n - cb);
                for (int idx = tid; idx < npiv * cw; idx += blockDim.x) {
                    const int t = idx / cw, c = idx - t * cw;
                    Us[t * PQ_CW + c] = I.W[(int64_t)(r0 + t) * I.ldw + cb + c];
                }
                __syncthreads();
                if (tid < cw) {
                    for (int t = 0; t < npiv; t++) {
                        uint64_t acc = (uint32_t)Us[t * PQ_CW + tid];
                        for (int s = 0; s < t; s++) {
                            const uint32_t l = (uint32_t)P[s * rs + t];
                            acc += (uint64_t)(l ? N - l : 0u) * (uint32_t)Us[s * PQ_CW + tid];
                        }
                        Us[t * PQ_CW + tid] = (int32_t)elim::mulmod(reduce_u64(acc, I.M), S.piv_inv[t], I.M);
                    }
                }
                __syncthreads();
                for (int idx = tid; idx < npiv * cw; idx += blockDim.x) {
                    const int t = idx / cw, c = idx - t * cw;
                    I.W[(int64_t)(r0 + t) * I.ldw + cb + c] = Us[t * PQ_CW + c];
                }
                // rows below the pivots: W += (N - l) u over 4 x 4 tiles per thread
                const int rows = R - npiv;
                const int trows = (rows + 3) >> 2, tcols = (cw + 3) >> 2;
                for (int tile = tid; tile < trows * tcols; tile += blockDim.x) {
                    const int tc = tile / trows, tr = tile - tc * trows;
                    const int lr0 = npiv + 4 * tr, cc0 = 4 * tc;
                    uint64_t acc[4][4];
#pragma unroll
                    for (int x = 0; x < 4; x++)
#pragma unroll
                        for (int y = 0; y < 4; y++) acc[x][y] = 0;
                    for (int t = 0; t < npiv; t++) {
                        uint32_t lv[4], uv[4];
#pragma unroll
                        for (int x = 0; x < 4; x++) {
                            const uint32_t l = (lr0 + x < R) ? (uint32_t)P[t * rs + lr0 + x] : 0u;
                            lv[x] = l ? N - l : 0u;
                        }
#pragma unroll
                        for (int y = 0; y < 4; y++) uv[y] = (cc0 + y < cw) ? (uint32_t)Us[t * PQ_CW + cc0 + y] : 0u;
#pragma unroll
                        for (int x = 0; x < 4; x++)
#pragma unroll
                            for (int y = 0; y < 4; y++) acc[x][y] += (uint64_t)lv[x] * uv[y];
                    }
#pragma unroll
                    for (int x = 0; x < 4; x++) {
                        if (lr0 + x < R) {
                            int32_t *wrow = I.W + (int64_t)(r0 + lr0 + x) * I.ldw + cb + cc0;
#pragma unroll
                            for (int y = 0; y < 4; y++)
                                if (cc0 + y < cw) wrow[y] = (int32_t)reduce_u64(acc[x][y] + (uint32_t)wrow[y], I.M);
                        }
                    }
                }
                __syncthreads();
            }
            row = r0 + npiv;
            col = c0 + npiv;
            if (stop) {
                status = stop;
                break;
            }
            if (zero_hit) {
                // zero column at col: swap it with the last column over every row, push, move on
                const int last = n - 1;
                if (col != last) {
                    for (int r = tid; r < m; r += blockDim.x) {
                        int32_t *w = I.W + (int64_t)r * I.ldw;
                        const int32_t x = w[col];
                        w[col] = w[last];
                        w[last] = x;
                    }
                }
                if (tid == 0) {
                    I.col_swaps[2 * nc] = col + 1;
                    I.col_swaps[2 * nc + 1] = last + 1;
                }
                nc++;
                col++;
            }
            __syncthreads();
        }
        __syncthreads();
        to_colmajor(I.W, I.ldw, n, I.U, I.ldu, m, n, Us);
        to_colmajor(I.LW, I.ldlw, I.lwc, I.L, I.ldl, m, I.l_cols, Us);
        if (tid == 0) {
            I.info[0] = nr;
            I.info[1] = nc;
            I.info[2] = row;
            I.info[3] = status;
        }
        __syncthreads();
    }
}

}  // namespace batched
