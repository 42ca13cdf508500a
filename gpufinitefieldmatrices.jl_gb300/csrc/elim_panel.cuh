// elim_panel.cuh -- the elimination's panel factorization kernel and the
// row-permutation kernel that follows each panel.
#pragma once

#include "gffm_common.cuh"

namespace elim {

constexpr int NB = 64;              // panel width (pivot columns per panel)
constexpr int PANEL_THREADS = 256;
constexpr int PANEL_WARPS = PANEL_THREADS / 32;
constexpr int MAX_PANEL_CTAS = 160;
constexpr int MAX_PERM_ROWS = 2 * NB;

enum PanelStatus { PS_DONE = 0, PS_ZERO_COL = 1, PS_TIMEOUT = 2, PS_BOUNDS = 3 };

struct ModP {
    uint32_t n;
    uint64_t minv;
};

__device__ __forceinline__ uint32_t mulmod(uint32_t a, uint32_t b, const ModP &M) {
    return (uint32_t)gffm_dev::barrett64((uint64_t)a * b, M.n, M.minv);
}

// floor(a / b) for 0 <= a < 2^26, b >= 1: float estimate, corrected to the exact quotient
__device__ __forceinline__ uint32_t udiv26(uint32_t a, uint32_t b) {
    int64_t q = (int64_t)__fdividef((float)a, (float)b);
    int64_t r = (int64_t)a - q * (int64_t)b;
    while (r < 0) {
        q--;
        r += b;
    }
    while (r >= (int64_t)b) {
        q++;
        r -= b;
    }
    return (uint32_t)q;
}

// mod_inv(p, P), src/CuModMatrix/rref_lu_pluq/pluq_kernels.jl:11-31: the same
// extended Euclid sequence (exact quotients), so the same result for any P.
__device__ __forceinline__ uint32_t mod_inv_euclid(uint32_t p, uint32_t P) {
    int64_t inv = 0, new_inv = 1;
    uint32_t rem = P, new_rem = p;
    while (new_rem != 0) {
        const uint32_t q = udiv26(rem, new_rem);
        const int64_t t = inv - (int64_t)q * new_inv;
        inv = new_inv;
        new_inv = t;
        const uint32_t r2 = rem - q * new_rem;
        rem = new_rem;
        new_rem = r2;
    }
    if (inv < 0) inv += P;
    return (uint32_t)inv;
}

// Pivot key: value (26 bits) | (0x3FFFFF - row) (22 bits) | step tag (16 bits).
// The largest key is the largest residue, then the lowest row.
__device__ __forceinline__ unsigned long long pkey(uint32_t v, int row) {
    return ((unsigned long long)v << 38) | ((unsigned long long)(0x3FFFFFu - (uint32_t)row) << 16);
}
__device__ __forceinline__ uint32_t pkey_val(unsigned long long k) { return (uint32_t)(k >> 38); }
__device__ __forceinline__ int pkey_row(unsigned long long k) { return (int)(0x3FFFFFu - (uint32_t)((k >> 16) & 0x3FFFFFu)); }

// One published candidate: the CTA's best row of the panel and the inverse of
// its leading value (computed while the row is written).
struct alignas(16) Rec {
    unsigned long long key;   // written last
    unsigned long long inv;
    int32_t row[NB];
};

struct PanelArgs {
    int32_t *W;
    int64_t ldw;
    int m, n;
    int R0, C0, nbw;   // first pivot row / column, panel width
    int R;             // rows per CTA
    ModP M;
    int l_cols;        // L's padded width (PLUQ bound check), <= 0: no check
    Rec *rec;          // [2][G], keys zero at launch
    int32_t *old_row;  // [2][NB]
    int32_t *piv_row, *piv_val, *piv_inv;  // [NB]
    int *result;       // [0] pivots, [1] status
    int *err;
};

__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
    for (int o = 16; o; o >>= 1) {
        const unsigned long long x = __shfl_xor_sync(0xffffffffu, v, o);
        v = x > v ? x : v;
    }
    return v;
}

// Cooperative panel factorization.  CTA b owns rows [R0 + b*R, R0 + (b+1)*R)
// of columns [C0, C0 + nbw) in shared memory.  Per pivot step the CTAs
// exchange one record each (their best candidate row with its inverse, tagged
// with the step) through a parity-double-buffered global slot; polling the G
// tags is the grid barrier, and every CTA then holds every candidate row.
__global__ void __launch_bounds__(PANEL_THREADS) k_panel(PanelArgs a) {
    extern __shared__ int32_t smem_dyn[];
    int32_t *P = smem_dyn;                           // R x NB
    int32_t *crow = smem_dyn + (size_t)a.R * NB;     // G x NB candidate rows
    __shared__ unsigned long long keys[MAX_PANEL_CTAS];
    __shared__ uint32_t invs[MAX_PANEL_CTAS];
    __shared__ int32_t oldr[NB], u[NB];
    __shared__ unsigned long long red[PANEL_WARPS];
    __shared__ int s_stop, s_status, s_prow, s_bw;
    __shared__ uint32_t s_pv, s_inv, s_cinv;
    const int b = blockIdx.x, G = gridDim.x, tid = threadIdx.x;
    const int lane = tid & 31, wid = tid >> 5;
    const int rbeg = a.R0 + b * a.R;
    const int rend = min(rbeg + a.R, a.m);
    const int nr = max(rend - rbeg, 0);
    const int nbw = a.nbw;

    for (int e = tid; e < nr * NB; e += blockDim.x) {
        const int i = e / NB, j = e - (e / NB) * NB;
        P[e] = (j < nbw) ? a.W[(int64_t)(rbeg + i) * a.ldw + a.C0 + j] : 0;
    }
    if (tid == 0) {
        s_stop = 0;
        s_status = PS_DONE;
    }
    __syncthreads();
    // candidate for step 0: column 0 over all own rows
    unsigned long long best = 0;
    for (int i = tid; i < nr; i += blockDim.x) {
        const unsigned long long k = pkey((uint32_t)P[i * NB], rbeg + i);
        best = k > best ? k : best;
    }
    best = warp_max_u64(best);
    if (lane == 0) red[wid] = best;

    const int tmax = min(nbw, a.m - a.R0);
    int t = 0;
    for (; t < tmax; t++) {
        const int r = a.R0 + t;
        const int par = t & 1;
        const unsigned long long tag = (unsigned long long)(t + 1);
        Rec *mine = a.rec + par * G + b;
        __syncthreads();  // red[] complete, previous step done
        // 1. publish: candidate row (and the current row r from its owner); thread 0
        //    computes the candidate's inverse meanwhile, then writes inverse and tagged key
        best = 0;
        for (int w = 0; w < PANEL_WARPS; w++) best = red[w] > best ? red[w] : best;
        if (best) {
            const int li = pkey_row(best) - rbeg;
            for (int j = tid; j < NB; j += blockDim.x) mine->row[j] = P[li * NB + j];
        }
        if (r >= rbeg && r < rend)
            for (int j = tid; j < NB; j += blockDim.x) a.old_row[par * NB + j] = P[(r - rbeg) * NB + j];
        if (tid == 0) s_cinv = pkey_val(best) ? mod_inv_euclid(pkey_val(best), a.M.n) : 0;
        __syncthreads();
        if (tid == 0) {
            mine->inv = s_cinv;
            __threadfence();
            *(volatile unsigned long long *)&mine->key = best | tag;
        }
        // 2. gather every record (this is the grid barrier)
        const int owner = (r - a.R0) / a.R;
        for (int g = tid; g < G; g += blockDim.x) {
            const volatile unsigned long long *kp = &a.rec[par * G + g].key;
            unsigned long long k = *kp;
            if ((k & 0xFFFFull) != tag) {
                const unsigned long long t0 = gffm_dev::globaltimer();
                while (((k = *kp) & 0xFFFFull) != tag) {
                    if (gffm_dev::globaltimer() - t0 > gffm_dev::kWaitLimitNs) {
                        atomicOr(a.err, 16);
                        s_stop = 1;
                        s_status = PS_TIMEOUT;
                        k = 0;
                        break;
                    }
                }
            }
            __threadfence();
            keys[g] = k & ~0xFFFFull;
            invs[g] = (uint32_t)__ldcg(&a.rec[par * G + g].inv);
            const int4 *src = reinterpret_cast<const int4 *>(a.rec[par * G + g].row);
            int4 *dst = reinterpret_cast<int4 *>(crow + (size_t)g * NB);
#pragma unroll
            for (int q = 0; q < NB / 4; q++) dst[q] = __ldcg(src + q);
            if (g == owner) {
                const int4 *os = reinterpret_cast<const int4 *>(a.old_row + par * NB);
                int4 *od = reinterpret_cast<int4 *>(oldr);
#pragma unroll
                for (int q = 0; q < NB / 4; q++) od[q] = __ldcg(os + q);
            }
        }
        __syncthreads();
        if (s_stop) break;
        // 3. the global pivot (every CTA decides the same)
        if (wid == 0) {
            unsigned long long wk = 0;
            int wg = 0;
            for (int g = lane; g < G; g += 32)
                if (keys[g] > wk) {
                    wk = keys[g];
                    wg = g;
                }
            for (int o = 16; o; o >>= 1) {
                const unsigned long long x = __shfl_xor_sync(0xffffffffu, wk, o);
                const int xg = __shfl_xor_sync(0xffffffffu, wg, o);
                if (x > wk) {
                    wk = x;
                    wg = xg;
                }
            }
            if (lane == 0) {
                const uint32_t pv = pkey_val(wk);
                if (pv == 0) {
                    s_stop = 1;
                    s_status = PS_ZERO_COL;
                } else if (a.l_cols > 0 && a.C0 + t >= a.l_cols) {
                    s_stop = 1;
                    s_status = PS_BOUNDS;
                } else {
                    s_pv = pv;
                    s_prow = pkey_row(wk);
                    s_bw = wg;
                    s_inv = invs[wg];
                }
            }
        }
        __syncthreads();
        if (s_stop) break;
        const int prow = s_prow;
        const uint32_t inv = s_inv;
        const int32_t *piv = crow + (size_t)s_bw * NB;
        for (int j = tid; j < NB; j += blockDim.x) u[j] = (int32_t)mulmod((uint32_t)piv[j], inv, a.M);
        __syncthreads();
        // 4. swap_rows_and_mod restricted to the panel: row r <- pivot row (scaled from
        //    column t on), row prow <- old row r; the multiplier columns swap unscaled
        if (r >= rbeg && r < rend) {
            int32_t *pr = P + (r - rbeg) * NB;
            for (int j = tid; j < nbw; j += blockDim.x) pr[j] = j >= t ? u[j] : piv[j];
        }
        if (prow != r && prow >= rbeg && prow < rend) {
            int32_t *pp = P + (prow - rbeg) * NB;
            for (int j = tid; j < nbw; j += blockDim.x) pp[j] = oldr[j];
        }
        __syncthreads();
        // 5. eliminate the rows below the pivot (warps over rows, lanes over columns);
        //    the multiplier stays in column t; column t+1 gives the next candidate
        best = 0;
        {
            const int i0 = max(r + 1 - rbeg, 0);
            const int jb = t + 1;
            if (jb < nbw) {
                for (int i = i0 + wid; i < nr; i += PANEL_WARPS) {
                    int32_t *pi = P + i * NB;
                    const uint32_t l = (uint32_t)pi[t];
                    for (int j = jb + lane; j < nbw; j += 32) {
                        uint32_t x = (uint32_t)pi[j];
                        if (l != 0) {
                            x = (uint32_t)gffm_dev::barrett64((uint64_t)x + (uint64_t)(a.M.n - l) * (uint32_t)u[j],
                                                              a.M.n, a.M.minv);
                            pi[j] = (int32_t)x;
                        }
                        if (j == jb) {
                            const unsigned long long k = pkey(x, rbeg + i);
                            best = k > best ? k : best;
                        }
                    }
                }
            }
        }
        if (b == 0 && tid == 0) {
            a.piv_row[t] = prow;
            a.piv_val[t] = (int32_t)s_pv;
            a.piv_inv[t] = (int32_t)inv;
        }
        best = warp_max_u64(best);
        if (lane == 0) red[wid] = best;
    }
    __syncthreads();
    for (int e = tid; e < nr * NB; e += blockDim.x) {
        const int i = e / NB, j = e - (e / NB) * NB;
        if (j < nbw) a.W[(int64_t)(rbeg + i) * a.ldw + a.C0 + j] = P[e];
    }
    if (b == 0 && tid == 0) {
        a.result[0] = t;
        a.result[1] = s_status;
    }
}

// L11^{-1} of a panel with t pivots (rows R0.., pivot columns C0..; L11 has the
// pivot values on the diagonal and the multipliers W[R0+i][C0+s] below), one
// warp per column j by forward substitution:
//   X[i][j] = inv_i * (delta_ij - sum_{j<=s<i} L11[i][s] X[s][j]).
// Lanes hold X[s][j] for s = lane, lane + 32; each dot product is a warp sum.
// Output row-major, ld NB, zero above the diagonal.
__global__ void __launch_bounds__(1024) k_linv(const int32_t *W, int64_t ldw, int R0, int C0, int t,
                                               const int32_t *inv, int32_t *linv, ModP M) {
    __shared__ uint32_t L11[NB][NB + 1];
    for (int e = threadIdx.x; e < NB * NB; e += blockDim.x) {
        const int i = e / NB, s = e % NB;
        L11[i][s] = (s < i && i < t) ? (uint32_t)W[(int64_t)(R0 + i) * ldw + C0 + s] : 0;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int j = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (j >= NB) return;
    uint32_t x0 = 0, x1 = 0;  // X[lane][j], X[lane + 32][j]
    for (int i = 0; i < NB; i++) {
        uint32_t xi = 0;
        if (i < t && i >= j) {
            if (i == j) {
                xi = (uint32_t)inv[i];
            } else {
                uint64_t part = 0;
                if (lane >= j && lane < i) part += (uint64_t)L11[i][lane] * x0;
                if (lane + 32 >= j && lane + 32 < i) part += (uint64_t)L11[i][lane + 32] * x1;
                for (int o = 16; o; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
                const uint32_t a = (uint32_t)gffm_dev::barrett64(part, M.n, M.minv);
                xi = mulmod(a ? M.n - a : 0, (uint32_t)inv[i], M);
            }
        }
        if (lane == (i & 31)) {
            if (i < 32)
                x0 = xi;
            else
                x1 = xi;
        }
        if (lane == 0 && i < t) linv[i * NB + j] = (int32_t)xi;
    }
}

// Row permutation of columns [c_lo, c_hi): row rows[k] receives the old row
// rows[src[k]] (the composition of a panel's swaps, computed on the host).
struct PermArgs {
    int K;
    int32_t rows[MAX_PERM_ROWS];
    int32_t src[MAX_PERM_ROWS];
};

__global__ void __launch_bounds__(64) k_permute_rows(int32_t *W, int64_t ldw, int c_lo, int c_hi,
                                                     const __grid_constant__ PermArgs p) {
    __shared__ int32_t buf[MAX_PERM_ROWS][64];
    const int j = c_lo + blockIdx.x * 64 + threadIdx.x;
    const bool ok = j < c_hi;
    for (int k = 0; k < p.K; k++) buf[k][threadIdx.x] = ok ? W[(int64_t)p.rows[k] * ldw + j] : 0;
    __syncthreads();
    if (!ok) return;
    for (int k = 0; k < p.K; k++) W[(int64_t)p.rows[k] * ldw + j] = buf[p.src[k]][threadIdx.x];
}

}  // namespace elim
