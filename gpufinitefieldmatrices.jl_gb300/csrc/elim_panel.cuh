// elim_panel.cuh -- the elimination's panel factorization kernel and the
// row-permutation kernel that follows each panel.
#pragma once

#include "gffm_common.cuh"
#include "modarith.cuh"

namespace elim {

constexpr int NB = 128;             // panel width (pivot columns per panel)
constexpr int CPL = NB / 32;        // panel columns per lane in the elimination
constexpr int PANEL_THREADS = 512;
constexpr int PANEL_WARPS = PANEL_THREADS / 32;
constexpr int MAX_PANEL_CTAS = 160;
constexpr int MAX_PERM_ROWS = 2 * NB;

enum PanelStatus { PS_DONE = 0, PS_ZERO_COL = 1, PS_TIMEOUT = 2, PS_BOUNDS = 3 };

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
    Mont mont;         // for the pivot inverses
    Rec *rec;          // [2][G], keys zero at launch
    int32_t *old_row;  // [2][NB]
    int32_t *piv_row, *piv_val, *piv_inv;  // [NB]
    int *result;       // [0] pivots, [1] status
    int *err;
};

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

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
// with the step) through a parity-double-buffered global slot: polling the G
// tags is the grid barrier, then every CTA loads the winning row.  The next
// pivot column is eliminated first, so the next candidate's inverse (warp 0)
// overlaps the elimination of the remaining columns (the other warps).
__global__ void __launch_bounds__(PANEL_THREADS, 1) k_panel(PanelArgs a) {
    extern __shared__ int32_t smem_dyn[];
    int32_t *P = smem_dyn;  // R x NB
    __shared__ unsigned long long keys[MAX_PANEL_CTAS];
    __shared__ uint32_t invs[MAX_PANEL_CTAS];
    __shared__ __align__(16) int32_t piv[NB];
    __shared__ __align__(16) int32_t oldr[NB];
    __shared__ int32_t u[NB];
    __shared__ unsigned long long red[PANEL_WARPS];
    __shared__ unsigned long long s_best;
    __shared__ int s_stop, s_status, s_prow, s_bw;
    __shared__ uint32_t s_inv, s_cinv;
    const int b = blockIdx.x, G = gridDim.x, tid = threadIdx.x;
    const int lane = tid & 31, wid = tid >> 5;
    const int rbeg = a.R0 + b * a.R;
    const int rend = min(rbeg + a.R, a.m);
    const int nr = max(rend - rbeg, 0);
    const int nbw = a.nbw;
    const uint32_t n = a.M.n;

    for (int e = tid; e < nr * NB; e += blockDim.x) {
        const int i = e / NB, j = e - (e / NB) * NB;
        P[e] = (j < nbw) ? a.W[(int64_t)(rbeg + i) * a.ldw + a.C0 + j] : 0;
    }
    if (tid == 0) {
        s_stop = 0;
        s_status = PS_DONE;
    }
    __syncthreads();
    // candidate for step 0: column 0 over all own rows, and its inverse
    {
        unsigned long long best = 0;
        for (int i = tid; i < nr; i += blockDim.x) {
            const unsigned long long k = pkey((uint32_t)P[i * NB], rbeg + i);
            best = k > best ? k : best;
        }
        best = warp_max_u64(best);
        if (lane == 0) red[wid] = best;
        __syncthreads();
        if (wid == 0) {
            best = lane < PANEL_WARPS ? red[lane] : 0ull;
            best = warp_max_u64(best);
            if (lane == 0) {
                s_best = best;
                s_cinv = pkey_val(best) ? mod_inverse(pkey_val(best), a.mont) : 0u;
            }
        }
        __syncthreads();
    }

    const int tmax = min(nbw, a.m - a.R0);
    int t = 0;
    for (; t < tmax; t++) {
        const int r = a.R0 + t;
        const int par = t & 1;
        const unsigned long long tag = (unsigned long long)(t + 1);
        Rec *mine = a.rec + par * G + b;
        // 1. publish the candidate row (and the current row r from its owner), then
        //    the inverse and the tagged key with release semantics
        const unsigned long long best0 = s_best;
        if (best0) {
            const int li = pkey_row(best0) - rbeg;
            for (int j = tid; j < NB; j += blockDim.x) mine->row[j] = P[li * NB + j];
        }
        if (r >= rbeg && r < rend)
            for (int j = tid; j < NB; j += blockDim.x) a.old_row[par * NB + j] = P[(r - rbeg) * NB + j];
        __syncthreads();
        if (tid == 0) {
            mine->inv = s_cinv;
            asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(&mine->key), "l"(best0 | tag) : "memory");
        }
        // 2. poll the G tagged keys (the grid barrier)
        for (int g = tid; g < G; g += blockDim.x) {
            const unsigned long long *kp = &a.rec[par * G + g].key;
            unsigned long long k = ld_acquire_u64(kp);
            if ((k & 0xFFFFull) != tag) {
                const unsigned long long t0 = gffm_dev::globaltimer();
                while (((k = ld_acquire_u64(kp)) & 0xFFFFull) != tag) {
                    if (gffm_dev::globaltimer() - t0 > gffm_dev::kWaitLimitNs) {
                        atomicOr(a.err, 16);
                        s_stop = 1;
                        s_status = PS_TIMEOUT;
                        k = 0;
                        break;
                    }
                }
            }
            keys[g] = k & ~0xFFFFull;
            invs[g] = (uint32_t)__ldcg(&a.rec[par * G + g].inv);
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
                    s_prow = pkey_row(wk);
                    s_bw = wg;
                    s_inv = invs[wg];
                    if (b == 0) {
                        a.piv_row[t] = s_prow;
                        a.piv_val[t] = (int32_t)pv;
                        a.piv_inv[t] = (int32_t)s_inv;
                    }
                }
            }
        }
        __syncthreads();
        if (s_stop) break;
        // 4. the winning row and the current row r
        {
            const int owner = (r - a.R0) / a.R;
            if (tid < NB / 4)
                reinterpret_cast<int4 *>(piv)[tid] =
                    __ldcg(reinterpret_cast<const int4 *>(a.rec[par * G + s_bw].row) + tid);
            else if (tid < NB / 2 && owner != b)
                reinterpret_cast<int4 *>(oldr)[tid - NB / 4] =
                    __ldcg(reinterpret_cast<const int4 *>(a.old_row + par * NB) + (tid - NB / 4));
            else if (tid < NB / 2)
                for (int q = 0; q < 4; q++) oldr[(tid - NB / 4) * 4 + q] = P[(r - rbeg) * NB + (tid - NB / 4) * 4 + q];
        }
        __syncthreads();
        const int prow = s_prow;
        const uint32_t inv = s_inv;
        for (int j = tid; j < NB; j += blockDim.x) u[j] = (int32_t)mulmod((uint32_t)piv[j], inv, a.M);
        __syncthreads();
        // 5. swap_rows_and_mod restricted to the panel: row r <- pivot row (scaled from
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
        // 6. eliminate the rows below the pivot (the multiplier stays in column t).
        //    a) the next pivot column, one thread per row, and the next candidate
        const int i0 = max(r + 1 - rbeg, 0);
        const int jb = t + 1;
        {
            unsigned long long best = 0;
            if (jb < nbw) {
                const uint32_t ub = (uint32_t)u[jb], sb = shoup_pre(ub, a.M);
                for (int i = i0 + tid; i < nr; i += blockDim.x) {
                    const uint32_t l = (uint32_t)P[i * NB + t];
                    uint32_t x = (uint32_t)P[i * NB + jb];
                    const uint32_t d = shoup_mul(l, ub, sb, n);
                    x = x >= d ? x - d : x + n - d;
                    P[i * NB + jb] = (int32_t)x;
                    const unsigned long long k = pkey(x, rbeg + i);
                    best = k > best ? k : best;
                }
            }
            best = warp_max_u64(best);
            if (lane == 0) red[wid] = best;
            __syncthreads();
            if (wid == 0) {
                best = lane < PANEL_WARPS ? red[lane] : 0ull;
                best = warp_max_u64(best);
                if (lane == 0) s_best = best;
            }
            __syncthreads();
        }
        //    b) warp 0: the inverse of the next candidate; warps 1..: columns jb+1..
        if (wid == 0) {
            if (lane == 0) {
                const uint32_t v = pkey_val(s_best);
                s_cinv = (jb < nbw && v) ? mod_inverse(v, a.mont) : 0u;
            }
        } else if (jb + 1 < nbw) {
            uint32_t uc[CPL], us[CPL];
#pragma unroll
            for (int c = 0; c < CPL; c++) {
                const int j = jb + 1 + lane + 32 * c;
                uc[c] = j < nbw ? (uint32_t)u[j] : 0u;
                us[c] = shoup_pre(uc[c], a.M);
            }
            for (int i = i0 + wid - 1; i < nr; i += PANEL_WARPS - 1) {
                int32_t *pi = P + i * NB;
                const uint32_t l = (uint32_t)pi[t];
                uint32_t x[CPL];
#pragma unroll
                for (int c = 0; c < CPL; c++) {
                    const int j = jb + 1 + lane + 32 * c;
                    x[c] = j < nbw ? (uint32_t)pi[j] : 0u;
                }
#pragma unroll
                for (int c = 0; c < CPL; c++) {
                    const int j = jb + 1 + lane + 32 * c;
                    if (j < nbw) {
                        const uint32_t d = shoup_mul(l, uc[c], us[c], n);
                        pi[j] = (int32_t)(x[c] >= d ? x[c] - d : x[c] + n - d);
                    }
                }
            }
        }
        __syncthreads();
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
// Lanes hold X[s][j] for s = lane + 32c; each dot product is a warp sum.
// Output row-major, ld NB, zero above the diagonal.  Dynamic shared memory:
// NB x (NB + 1) words for L11.
constexpr size_t LINV_SMEM = (size_t)NB * (NB + 1) * 4;
__global__ void __launch_bounds__(1024) k_linv(const int32_t *W, int64_t ldw, int R0, int C0, int t,
                                               const int32_t *inv, int32_t *linv, ModP M) {
    extern __shared__ uint32_t L11s[];
    auto L11 = [&](int i, int s) -> uint32_t & { return L11s[i * (NB + 1) + s]; };
    for (int e = threadIdx.x; e < NB * NB; e += blockDim.x) {
        const int i = e / NB, s = e % NB;
        L11(i, s) = (s < i && i < t) ? (uint32_t)W[(int64_t)(R0 + i) * ldw + C0 + s] : 0;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int j = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (j >= NB) return;
    uint32_t x[CPL];  // X[lane + 32c][j]
#pragma unroll
    for (int c = 0; c < CPL; c++) x[c] = 0;
    for (int i = 0; i < NB; i++) {
        uint32_t xi = 0;
        if (i < t && i >= j) {
            if (i == j) {
                xi = (uint32_t)inv[i];
            } else {
                uint64_t part = 0;
#pragma unroll
                for (int c = 0; c < CPL; c++) {
                    const int s = lane + 32 * c;
                    if (s >= j && s < i) part += (uint64_t)L11(i, s) * x[c];
                }
                // reduce each lane's part first: the warp sum of 32 residues fits 32 bits
                uint32_t p32 = (uint32_t)gffm_dev::barrett64(part, M.n, M.minv);
                for (int o = 16; o; o >>= 1) p32 += __shfl_xor_sync(0xffffffffu, p32, o);
                const uint32_t a = (uint32_t)gffm_dev::barrett64(p32, M.n, M.minv);
                xi = mulmod(a ? M.n - a : 0, (uint32_t)inv[i], M);
            }
        }
#pragma unroll
        for (int c = 0; c < CPL; c++)
            if (lane + 32 * c == i) x[c] = xi;
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

// Two passes through a K x ncols scratch copy (both fully parallel and coalesced):
// k_rows_gather: tmp[k][j] = W[rows[k]][c_lo + j];  k_rows_scatter: W[rows[k]][c_lo + j] = tmp[src[k]][j].
__global__ void __launch_bounds__(256) k_rows_gather(const int32_t *__restrict__ W, int64_t ldw, int c_lo, int ncols,
                                                     int32_t *__restrict__ tmp, const __grid_constant__ PermArgs p) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (int64_t)p.K * ncols) return;
    const int k = (int)(e / ncols), j = (int)(e - (int64_t)k * ncols);
    tmp[e] = W[(int64_t)p.rows[k] * ldw + c_lo + j];
}
__global__ void __launch_bounds__(256) k_rows_scatter(int32_t *__restrict__ W, int64_t ldw, int c_lo, int ncols,
                                                      const int32_t *__restrict__ tmp,
                                                      const __grid_constant__ PermArgs p) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (int64_t)p.K * ncols) return;
    const int k = (int)(e / ncols), j = (int)(e - (int64_t)k * ncols);
    W[(int64_t)p.rows[k] * ldw + c_lo + j] = tmp[(int64_t)p.src[k] * ncols + j];
}

}  // namespace elim
