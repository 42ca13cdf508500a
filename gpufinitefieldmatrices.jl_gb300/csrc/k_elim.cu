// k_elim.cu -- blocked right-looking PLUQ / LU / RREF over Z/N (N < 2^26) with
// the exact step semantics of the reference's pluq_gpu_kernel
// (src/CuModMatrix/rref_lu_pluq/pluq_kernels.jl:46-440).
//
// Working copy.  A is copied into W, a row-major int32 matrix of residues, so
// that row swaps are contiguous copies.  Multipliers are kept below each pivot
// in W (LAPACK style) and moved into L at the end.
//
// One panel = up to NB consecutive pivot columns starting at (R0, C0).  The
// panel kernel is a cooperative grid: CTA b keeps rows [R0 + b*R, R0 + (b+1)*R)
// of the panel in shared memory.  Per pivot step it
//   1. finds its local maximum residue of the pivot column (lowest row on ties),
//   2. publishes the key, that row and (if it owns it) the current pivot row
//      into a parity-double-buffered global slot,
//   3. meets the other CTAs at a counting grid barrier (bounded wait),
//   4. picks the global winner, computes the inverse with the reference's
//      extended Euclid, swaps / scales the two rows it owns, and eliminates its
//      rows below the pivot:  W[i][j] = (W[i][j] + (N - l_i) * u_j) mod N.
// Everything the reference does to columns outside the panel is deferred and
// applied after the panel in the same order-independent form:
//   - columns left of the panel: the panel's row swaps (L's multipliers only
//     below the reference's L swap width 32*cld(m, 32); skipped columns always,
//     then the pivot-row scaling),
//   - trailing columns: the row swaps, a triangular solve for the panel rows
//     (x_t = inv_t * (a_t - sum_{s<t} L[r_t, c_s] x_s), the reference's
//     scaling and updates in closed form) and the update of the rows below,
//     A22 -= L21 * U12 mod N, on the limb tensor-core GEMM.
// A zero pivot column ends the panel when the panel already has pivots; at the
// start of a panel it triggers the reference's swap with the last column
// (PLUQ) or is skipped (LU / RREF).  Exact modular arithmetic makes every
// pivot search see the same values as the unblocked reference, so the pivot
// sequence, P, L, U, Q and the swap stacks are identical.
#include "gffm_common.cuh"
#include "limb_host.h"

#include <algorithm>
#include <vector>

namespace elim {

constexpr int NB = 64;              // panel width (pivot columns per panel)
constexpr int PANEL_THREADS = 256;

enum PanelStatus { PS_DONE = 0, PS_ZERO_COL = 1, PS_TIMEOUT = 2, PS_BOUNDS = 3 };
enum Mode { MODE_PLUQ = 0, MODE_LU = 1, MODE_RREF = 2 };

struct ModP {
    uint32_t n;
    uint64_t minv;
};

__device__ __forceinline__ uint32_t mulmod(uint32_t a, uint32_t b, const ModP &M) {
    return (uint32_t)gffm_dev::barrett64((uint64_t)a * b, M.n, M.minv);
}

// mod_inv(p, P), src/CuModMatrix/rref_lu_pluq/pluq_kernels.jl:11-31
__device__ __forceinline__ uint32_t mod_inv_euclid(int64_t p, int64_t P) {
    int64_t inv = 0, new_inv = 1, rem = P, new_rem = p;
    while (new_rem != 0) {
        int64_t q = (int64_t)((uint32_t)rem / (uint32_t)new_rem);  // both in [0, 2^26)
        int64_t t = inv - q * new_inv;
        inv = new_inv;
        new_inv = t;
        t = rem - q * new_rem;
        rem = new_rem;
        new_rem = t;
    }
    if (inv < 0) inv += P;
    return (uint32_t)inv;
}

struct PanelArgs {
    int32_t *W;
    int64_t ldw;
    int m, n;
    int R0, C0, nbw;   // first pivot row / column, panel width
    int R;             // rows per CTA
    ModP M;
    int lsw;           // L row swaps reach columns [0, lsw) only
    int l_cols;        // L's padded width (PLUQ bound check), <= 0: no check
    unsigned long long *cand_key;  // [2][G]
    int32_t *cand_row;             // [2][G][NB]
    int32_t *old_row;              // [2][NB]
    unsigned int *bar;             // barrier counter, zero at launch
    int32_t *piv_row, *piv_val, *piv_inv;  // [NB]
    int *result;                           // [0] pivots, [1] status
    int *err;
};

__global__ void __launch_bounds__(PANEL_THREADS) k_panel(PanelArgs a) {
    extern __shared__ int32_t P[];  // R x NB
    __shared__ int32_t piv[NB], oldr[NB], u[NB];
    __shared__ unsigned long long red[PANEL_THREADS / 32];
    __shared__ int s_stop, s_status;
    __shared__ int32_t s_prow, s_pv, s_inv;
    const int b = blockIdx.x, G = gridDim.x, tid = threadIdx.x;
    const int lane = tid & 31, wid = tid >> 5;
    const int rbeg = a.R0 + b * a.R;
    const int rend = min(rbeg + a.R, a.m);
    const int nr = max(rend - rbeg, 0);
    const int nbw = a.nbw;

    for (int e = tid; e < nr * NB; e += blockDim.x) {
        int i = e / NB, j = e - (e / NB) * NB;
        P[e] = (j < nbw) ? a.W[(int64_t)(rbeg + i) * a.ldw + a.C0 + j] : 0;
    }
    if (tid == 0) {
        s_stop = 0;
        s_status = PS_DONE;
    }
    __syncthreads();

    const int tmax = min(nbw, a.m - a.R0);
    int t = 0;
    for (; t < tmax; t++) {
        const int r = a.R0 + t;
        const int par = t & 1;
        // 1. local arg-max of column t over rows >= r (key: value, then lowest row)
        unsigned long long best = 0;
        for (int i = max(r - rbeg, 0) + tid; i < nr; i += blockDim.x) {
            unsigned long long key = ((unsigned long long)(uint32_t)P[i * NB + t] << 32) |
                                     (unsigned long long)(0xFFFFFFFFu - (uint32_t)(rbeg + i));
            best = key > best ? key : best;
        }
        for (int o = 16; o; o >>= 1) {
            unsigned long long v = __shfl_xor_sync(0xffffffffu, best, o);
            best = v > best ? v : best;
        }
        if (lane == 0) red[wid] = best;
        __syncthreads();
        if (tid == 0) {
            for (int w = 1; w < PANEL_THREADS / 32; w++) best = red[w] > best ? red[w] : best;
            best = red[0] > best ? red[0] : best;
            a.cand_key[par * G + b] = best;
            s_prow = best ? (int)(0xFFFFFFFFu - (uint32_t)best) : -1;
        }
        __syncthreads();
        // 2. publish the candidate row and, from its owner, the current row r
        {
            const int li = s_prow >= 0 ? s_prow - rbeg : -1;
            int32_t *cr = a.cand_row + ((size_t)par * G + b) * NB;
            if (li >= 0)
                for (int j = tid; j < nbw; j += blockDim.x) cr[j] = P[li * NB + j];
            if (r >= rbeg && r < rend)
                for (int j = tid; j < nbw; j += blockDim.x) a.old_row[par * NB + j] = P[(r - rbeg) * NB + j];
        }
        __syncthreads();
        // 3. grid barrier (bounded)
        if (tid == 0) {
            __threadfence();
            atomicAdd(a.bar, 1u);
            const unsigned int target = (unsigned int)(t + 1) * (unsigned int)G;
            if (*(volatile unsigned int *)a.bar < target) {
                const unsigned long long t0 = gffm_dev::globaltimer();
                while (*(volatile unsigned int *)a.bar < target) {
                    if (gffm_dev::globaltimer() - t0 > gffm_dev::kWaitLimitNs) {
                        atomicOr(a.err, 16);
                        s_stop = 1;
                        s_status = PS_TIMEOUT;
                        break;
                    }
                }
            }
            __threadfence();
        }
        __syncthreads();
        if (s_stop) break;
        // 4. the global pivot
        unsigned long long wk = 0;
        for (int g = tid; g < G; g += blockDim.x) {
            unsigned long long v = *(volatile unsigned long long *)&a.cand_key[par * G + g];
            wk = v > wk ? v : wk;
        }
        for (int o = 16; o; o >>= 1) {
            unsigned long long v = __shfl_xor_sync(0xffffffffu, wk, o);
            wk = v > wk ? v : wk;
        }
        if (lane == 0) red[wid] = wk;
        __syncthreads();
        if (tid == 0) {
            for (int w = 0; w < PANEL_THREADS / 32; w++) wk = red[w] > wk ? red[w] : wk;
            const uint32_t pv = (uint32_t)(wk >> 32);
            if (pv == 0) {
                s_stop = 1;
                s_status = PS_ZERO_COL;
            } else if (a.l_cols > 0 && a.C0 + t >= a.l_cols) {
                s_stop = 1;
                s_status = PS_BOUNDS;
            } else {
                s_pv = (int32_t)pv;
                s_prow = (int)(0xFFFFFFFFu - (uint32_t)wk);
            }
        }
        __syncthreads();
        if (s_stop) break;
        const int prow = s_prow;
        const int bw = (prow - a.R0) / a.R;
        {
            const volatile int32_t *cr = a.cand_row + ((size_t)par * G + bw) * NB;
            const volatile int32_t *orow = a.old_row + par * NB;
            for (int j = tid; j < nbw; j += blockDim.x) {
                piv[j] = cr[j];
                oldr[j] = orow[j];
            }
        }
        if (tid == 0) s_inv = (int32_t)mod_inv_euclid(s_pv, a.M.n);
        __syncthreads();
        const uint32_t inv = (uint32_t)s_inv;
        for (int j = tid; j < nbw; j += blockDim.x) u[j] = (int32_t)mulmod((uint32_t)piv[j], inv, a.M);
        __syncthreads();
        // 5. swap_rows_and_mod restricted to the panel: row r <- pivot row * inv,
        //    row prow <- old row r; multiplier columns (j < t) swap unscaled, only below lsw
        if (r >= rbeg && r < rend) {
            int32_t *pr = P + (r - rbeg) * NB;
            for (int j = tid; j < nbw; j += blockDim.x) {
                if (j >= t)
                    pr[j] = u[j];
                else if (a.C0 + j < a.lsw)
                    pr[j] = piv[j];
            }
        }
        if (prow != r && prow >= rbeg && prow < rend) {
            int32_t *pp = P + (prow - rbeg) * NB;
            for (int j = tid; j < nbw; j += blockDim.x) {
                if (j >= t || a.C0 + j < a.lsw) pp[j] = oldr[j];
            }
        }
        __syncthreads();
        // 6. eliminate rows below the pivot (the multiplier stays in column t)
        {
            const int i0 = max(r + 1 - rbeg, 0);
            const int ncol = nbw - t - 1;
            if (ncol > 0 && i0 < nr) {
                const int total = (nr - i0) * ncol;
                for (int e = tid; e < total; e += blockDim.x) {
                    const int i = i0 + e / ncol;
                    const int j = t + 1 + e % ncol;
                    const uint32_t l = (uint32_t)P[i * NB + t];
                    if (l != 0) {
                        const uint64_t v = (uint64_t)(uint32_t)P[i * NB + j] + (uint64_t)(a.M.n - l) * (uint32_t)u[j];
                        P[i * NB + j] = (int32_t)gffm_dev::barrett64(v, a.M.n, a.M.minv);
                    }
                }
            }
        }
        if (b == 0 && tid == 0) {
            a.piv_row[t] = prow;
            a.piv_val[t] = s_pv;
            a.piv_inv[t] = (int32_t)inv;
        }
        __syncthreads();
    }
    for (int e = tid; e < nr * NB; e += blockDim.x) {
        int i = e / NB, j = e - (e / NB) * NB;
        if (j < nbw) a.W[(int64_t)(rbeg + i) * a.ldw + a.C0 + j] = P[e];
    }
    if (b == 0 && tid == 0) {
        a.result[0] = t;
        a.result[1] = s_status;
    }
}

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

// Apply the panel's row swaps (pivot s: rows R0+s <-> prow[s]), in order, to
// columns [c_lo, c_hi); with inv != nullptr also scale the new pivot row.
__global__ void __launch_bounds__(256) k_laswp(int32_t *W, int64_t ldw, int c_lo, int c_hi, int R0, int t,
                                               const int32_t *prow, const int32_t *inv, ModP M) {
    const int j = c_lo + blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= c_hi) return;
    for (int s = 0; s < t; s++) {
        const int r = R0 + s, p = prow[s];
        if (p != r) {
            int32_t x = W[(int64_t)r * ldw + j];
            W[(int64_t)r * ldw + j] = W[(int64_t)p * ldw + j];
            W[(int64_t)p * ldw + j] = x;
        }
        if (inv) W[(int64_t)r * ldw + j] = (int32_t)mulmod((uint32_t)W[(int64_t)r * ldw + j], (uint32_t)inv[s], M);
    }
}

// Skipped (swapped-in, never eliminated) columns: the panel's row swaps for
// columns at or beyond lo (those below lo were covered by k_laswp), then the
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

// Rows R0..R0+t-1 of the trailing columns [cs, n):
//   x_i = inv_i * (a_i - sum_{s<i} L11[i][s] x_s)  mod N,
// L11[i][s] = W[R0+i][C0+s] (the multipliers of this panel).  Sums of up to NB
// products below 2^52 are exact in 64 bits before one reduction.
__global__ void __launch_bounds__(128) k_trsm(int32_t *W, int64_t ldw, int R0, int C0, int t, int cs, int n,
                                              const int32_t *inv, ModP M) {
    __shared__ uint32_t L11[NB][NB + 1];
    __shared__ uint32_t sinv[NB];
    for (int e = threadIdx.x; e < t * t; e += blockDim.x) {
        int i = e / t, s = e % t;
        L11[i][s] = (s < i) ? (M.n - (uint32_t)W[(int64_t)(R0 + i) * ldw + C0 + s]) % M.n : 0;
    }
    for (int e = threadIdx.x; e < t; e += blockDim.x) sinv[e] = (uint32_t)inv[e];
    __syncthreads();
    const int j = cs + blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    uint32_t x[NB];
#pragma unroll
    for (int i = 0; i < NB; i++) {
        if (i < t) {
            uint64_t acc = (uint32_t)W[(int64_t)(R0 + i) * ldw + j];
#pragma unroll
            for (int s = 0; s < NB; s++)
                if (s < i) acc += (uint64_t)L11[i][s] * x[s];
            const uint32_t v = (uint32_t)gffm_dev::barrett64(acc, M.n, M.minv);
            x[i] = mulmod(v, sinv[i], M);
            W[(int64_t)(R0 + i) * ldw + j] = (int32_t)x[i];
        }
    }
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
    __shared__ uint32_t coef[NB][NB + 1];
    for (int e = threadIdx.x; e < NB * NB; e += blockDim.x) {
        int k = e / NB, i = e % NB;
        coef[k][i] = (k < nbp && i < nbp && i > k) ? (M.n - (uint32_t)coefbuf[k * NB + i]) % M.n : 0;
    }
    __syncthreads();
    const int j = pcol[0] + blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    uint32_t y[NB];
#pragma unroll
    for (int kk = NB - 1; kk >= 0; kk--) {
        y[kk] = 0;
        if (kk < nbp) {
            uint64_t acc = (uint32_t)W[(int64_t)(p0 + kk) * ldw + j];
#pragma unroll
            for (int i = NB - 1; i > kk; i--) acc += (uint64_t)coef[kk][i] * y[i];
            y[kk] = (uint32_t)gffm_dev::barrett64(acc, M.n, M.minv);
        }
    }
#pragma unroll
    for (int kk = 0; kk < NB; kk++)
        if (kk < nbp) W[(int64_t)(p0 + kk) * ldw + j] = (int32_t)y[kk];
}

// out[k][i] = W[row0 + k][pcol[i]] for k < rows (row-major, ld NB; zero past nbp)
__global__ void k_gather_cols(const int32_t *W, int64_t ldw, int row0, int rows, int nbp, const int32_t *pcol,
                              int32_t *out) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= rows) return;
    for (int i = 0; i < NB; i++) out[k * NB + i] = i < nbp ? W[(row0 + k) * ldw + pcol[i]] : 0;
}

// ---------------------------------------------------------------------------
// Host driver
// ---------------------------------------------------------------------------
struct Work {
    int32_t *W;
    int64_t ldw;
    unsigned long long *cand_key;
    int32_t *cand_row, *old_row;
    unsigned int *bar;
    int32_t *piv_row, *piv_val, *piv_inv;
    int *result;
    int32_t *colpiv, *lsrc, *lrow, *lpv, *pcol;  // [n], [lcols] x3, [min(m,n)]
    int32_t *gather;                             // m x NB
    int32_t *coef;                               // NB x NB
    int32_t *qlist;                              // [n] skipped columns
    __half *dA, *dB;                             // digit planes
    limb::Layout gl;
};

static size_t al(size_t x) { return (x + 255) & ~size_t(255); }

static void layout_ws(int64_t m, int64_t n, int64_t lcols, size_t *total, size_t off[16], limb::Layout *gl) {
    const int G = 160;
    const int64_t ldw = gffm::round_up(n > 0 ? n : 1, 32);
    // digit planes large enough for any trailing update / back substitution of
    // this problem: operands n x NB and NB x m (4 digits)
    *gl = limb::layout(std::max<int64_t>(n, 1), std::max<int64_t>(m, 1), NB, int64_t(1) << 25);
    size_t sizes[16] = {
        (size_t)std::max<int64_t>(m, 1) * ldw * 4,      // W
        (size_t)2 * G * 8,                              // cand_key
        (size_t)2 * G * NB * 4,                         // cand_row
        (size_t)2 * NB * 4,                             // old_row
        256,                                            // bar
        NB * 4, NB * 4, NB * 4,                         // piv_row/val/inv
        64,                                             // result
        (size_t)std::max<int64_t>(n, 1) * 4,            // colpiv
        (size_t)std::max<int64_t>(lcols, 1) * 4 * 3,    // lsrc/lrow/lpv
        (size_t)std::max<int64_t>(std::min(m, n), 1) * 4,  // pcol
        (size_t)std::max<int64_t>(m, 1) * NB * 4,       // gather
        gl->a_bytes, gl->b_bytes,
        (size_t)NB * NB * 4 + (size_t)std::max<int64_t>(n, 1) * 4};  // coef, qlist
    size_t o = 0;
    for (int i = 0; i < 16; i++) {
        off[i] = o;
        o += al(sizes[i]);
    }
    *total = o;
}

static void bind_ws(void *base, int64_t m, int64_t n, int64_t lcols, Work *w) {
    size_t total, off[16];
    layout_ws(m, n, lcols, &total, off, &w->gl);
    uint8_t *b = static_cast<uint8_t *>(base);
    w->W = (int32_t *)(b + off[0]);
    w->ldw = gffm::round_up(n > 0 ? n : 1, 32);
    w->cand_key = (unsigned long long *)(b + off[1]);
    w->cand_row = (int32_t *)(b + off[2]);
    w->old_row = (int32_t *)(b + off[3]);
    w->bar = (unsigned int *)(b + off[4]);
    w->piv_row = (int32_t *)(b + off[5]);
    w->piv_val = (int32_t *)(b + off[6]);
    w->piv_inv = (int32_t *)(b + off[7]);
    w->result = (int *)(b + off[8]);
    w->colpiv = (int32_t *)(b + off[9]);
    w->lsrc = (int32_t *)(b + off[10]);
    w->lrow = w->lsrc + std::max<int64_t>(lcols, 1);
    w->lpv = w->lrow + std::max<int64_t>(lcols, 1);
    w->pcol = (int32_t *)(b + off[11]);
    w->gather = (int32_t *)(b + off[12]);
    w->dA = (__half *)(b + off[13]);
    w->dB = (__half *)(b + off[14]);
    w->coef = (int32_t *)(b + off[15]);
    w->qlist = w->coef + NB * NB;
}

size_t workspace_bytes(int64_t m, int64_t n, int64_t lcols) {
    size_t total, off[16];
    limb::Layout gl;
    layout_ws(m, n, lcols, &total, off, &gl);
    return total;
}

struct Result {
    std::vector<int64_t> row_swaps, col_swaps;  // flattened 1-based pairs
    std::vector<int> piv_r, piv_c, piv_v;       // pivots in order
    std::vector<int> perm;                      // LU: final row order (0-based original index)
    int rank = 0;
};

// W -= L21 * U12 (or the RREF back update) on the limb GEMM, in row-major terms:
// C (rows x cols, row-major, ldc) -= X (rows x k, row-major, ldx) * Y (k x cols, row-major, ldy)
static int rowmajor_sub_gemm(Work &w, int64_t N, int32_t *C, int64_t ldc, const int32_t *X, int64_t ldx,
                             const int32_t *Y, int64_t ldy, int64_t rows, int64_t cols, int64_t k, cudaStream_t s) {
    if (rows <= 0 || cols <= 0 || k <= 0) return GFFM_OK;
    // column-major view: C^T (cols x rows) -= Y^T (cols x k) * X^T (k x rows)
    limb::Layout g = limb::layout(cols, rows, k, N);
    int st = limb::split_a<int32_t>(Y, ldy, cols, k, w.dA, g, N, s);
    if (st) return st;
    st = limb::split_b<int32_t>(X, ldx, k, rows, w.dB, g, N, s);
    if (st) return st;
    return limb::gemm_digits(g, w.dA, w.dB, cols, rows, k, N, C, ldc, 2 /* EPI_SUB_I32 */, 0, s);
}

static int run_panel(Work &w, int m, int n, int R0, int C0, int nbw, const ModP &M, int lsw, int lcols_check,
                     cudaStream_t s, int h_res[2], std::vector<int32_t> &h_prow, std::vector<int32_t> &h_pv) {
    using namespace gffm;
    const int rows = m - R0;
    int sms = sm_count();
    int R = 64;
    while ((rows + R - 1) / R > sms || (rows + R - 1) / R > 150) R += 32;
    if (R > 768)
        return set_error(GFFM_ERR_UNSUPPORTED, "elimination panel: %d rows exceed the panel kernel's capacity", rows);
    const int G = std::max(1, (rows + R - 1) / R);
    const size_t smem = (size_t)R * NB * 4;
    GFFM_CUDA(cudaMemsetAsync(w.bar, 0, sizeof(unsigned int), s));
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
    a.lsw = lsw;
    a.l_cols = lcols_check;
    a.cand_key = w.cand_key;
    a.cand_row = w.cand_row;
    a.old_row = w.old_row;
    a.bar = w.bar;
    a.piv_row = w.piv_row;
    a.piv_val = w.piv_val;
    a.piv_inv = w.piv_inv;
    a.result = w.result;
    a.err = device_error_flag();
    if (smem > 48 * 1024) GFFM_CUDA(cudaFuncSetAttribute(k_panel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    void *args[] = {&a};
    GFFM_CUDA(cudaLaunchCooperativeKernel((void *)k_panel, dim3(G), dim3(PANEL_THREADS), args, smem, s));
    GFFM_CUDA(cudaMemcpyAsync(h_res, w.result, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
    GFFM_CUDA(cudaMemcpyAsync(h_prow.data(), w.piv_row, NB * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    GFFM_CUDA(cudaMemcpyAsync(h_pv.data(), w.piv_val, NB * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    GFFM_CUDA(cudaStreamSynchronize(s));
    return GFFM_OK;
}

// Forward elimination shared by PLUQ / LU / RREF.
static int forward(Work &w, int m, int n, int64_t N, int mode, int lcols, cudaStream_t s, Result &res) {
    using namespace gffm;
    ModP M{(uint32_t)N, ~uint64_t(0) / (uint64_t)N};
    const int lsw = (mode == MODE_PLUQ) ? std::min<int64_t>(((int64_t)m + 31) / 32 * 32, lcols) : n;
    const int last = n - 1;
    std::vector<int> skipped;  // PLUQ: columns holding a swapped-in column that is never eliminated
    std::vector<int32_t> h_prow(NB), h_pv(NB);
    int h_res[2];
    int row = 0, col = 0;
    res.perm.resize(m);
    for (int i = 0; i < m; i++) res.perm[i] = i;
    while (row < m && col < n) {
        const int nbw = std::min(NB, n - col);
        int st = run_panel(w, m, n, row, col, nbw, M, lsw, mode == MODE_PLUQ ? lcols : 0, s, h_res, h_prow, h_pv);
        if (st) return st;
        const int t = h_res[0], status = h_res[1];
        if (status == PS_TIMEOUT) return set_error(GFFM_ERR_TIMEOUT, "elimination panel: a device-side wait gave up");
        for (int q = 0; q < t; q++) {
            const int r = row + q, p = h_prow[q];
            if (p != r) {
                res.row_swaps.push_back(r + 1);
                res.row_swaps.push_back(p + 1);
                std::swap(res.perm[r], res.perm[p]);
            }
            res.piv_r.push_back(r);
            res.piv_c.push_back(col + q);
            res.piv_v.push_back(h_pv[q]);
        }
        if (t > 0) {
            // columns left of the panel: L multipliers (below lsw) and skipped columns
            const int left_hi = std::min(col, lsw);
            if (left_hi > 0) {
                k_laswp<<<(left_hi + 255) / 256, 256, 0, s>>>(w.W, w.ldw, 0, left_hi, row, t, w.piv_row, nullptr, M);
                GFFM_LAUNCH_CHECK("k_laswp(left)");
            }
            if (!skipped.empty()) {
                // skipped columns hold A values: row swaps at every width, then the
                // pivot-row scaling (later swaps never touch a finished pivot row)
                const int nq = (int)skipped.size();
                k_skipped<<<(nq + 127) / 128, 128, 0, s>>>(w.W, w.ldw, w.qlist, nq, left_hi, row, t, w.piv_row,
                                                             w.piv_inv, M);
                GFFM_LAUNCH_CHECK("k_skipped");
            }
            // trailing columns: swaps, triangular solve, update of the rows below
            const int cs = col + nbw;
            if (cs < n) {
                k_laswp<<<(n - cs + 255) / 256, 256, 0, s>>>(w.W, w.ldw, cs, n, row, t, w.piv_row, nullptr, M);
                GFFM_LAUNCH_CHECK("k_laswp(trailing)");
                k_trsm<<<(n - cs + 127) / 128, 128, 0, s>>>(w.W, w.ldw, row, col, t, cs, n, w.piv_inv, M);
                GFFM_LAUNCH_CHECK("k_trsm");
                if (row + t < m) {
                    st = rowmajor_sub_gemm(w, N, w.W + (int64_t)(row + t) * w.ldw + cs, w.ldw,
                                           w.W + (int64_t)(row + t) * w.ldw + col, w.ldw,
                                           w.W + (int64_t)row * w.ldw + cs, w.ldw, m - row - t, n - cs, t, s);
                    if (st) return st;
                }
            }
            row += t;
            col += t;
        }
        if (status == PS_BOUNDS)
            return set_error(GFFM_ERR_BOUNDS, "pluq: pivot column %d is outside L's padded width %d (the reference "
                                              "raises a BoundsError here)", col + 1, lcols);
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
    for (int end = r; end > 0; end -= NB) {
        const int p0 = std::max(0, end - NB);
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
            int st = rowmajor_sub_gemm(w, N, w.W + c0, w.ldw, w.gather, NB, w.W + (int64_t)p0 * w.ldw + c0, w.ldw,
                                       p0, n - c0, nbp, s);
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
         int64_t *rank, void *ws, size_t ws_bytes, gffm_stream_t stream, int mode, int64_t *perm) {
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

}  // namespace elim

extern "C" {

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
