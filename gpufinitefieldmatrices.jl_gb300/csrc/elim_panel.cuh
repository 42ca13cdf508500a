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
    int32_t *linv;     // k_panel1: L11^{-1} of the panel's pivots, row-major, ld NB
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

// ---------------------------------------------------------------------------
// Single-CTA panel: the same factorization step as k_panel for a panel of at
// most P1_NB columns whose rows (at most P1_MAX_ROWS) fit one CTA's shared
// memory, without the grid-wide exchange.  Left-looking: column t is brought up
// to date when the pivot search reaches it,
//   U[0:t][t] = Linv W[0:t][t],    v[r] = W[r][t] + sum_{s<t} (N - l[r][s]) U[s][t],
// Linv the inverse of the panel's lower-triangular factor (pivots on its
// diagonal), grown by one row per pivot.  Pivot t-1 is applied while column t is
// prepared: warp 7 computes its inverse, warps 0 and 2 swap the rows, warp 1
// forms U[s][t] for s < t-1, warp 2 Linv's new row before scaling, warps 0-6 the
// partial values of column t.  The panel is written back as k_panel leaves it:
// pivot rows scaled (U), the multipliers unscaled below the pivots, the columns
// after a stop brought up to date.  No waits outside CTA barriers.
constexpr int P1_NB = 32;
constexpr int P1_THREADS = 256;
constexpr int P1_INV_WARP = 7;
constexpr int P1_MAX_ROWS = 1536;
__host__ __device__ constexpr size_t p1_smem_bytes(int rows) { return (size_t)P1_NB * (size_t)(rows + 4) * 4; }

__device__ __forceinline__ uint32_t p1_red(uint64_t x, const ModP &M) {
    return (uint32_t)gffm_dev::barrett64(x, M.n, M.minv);
}
// sum_{s < n8} a[s * sa] * b[s * sb], n8 a multiple of 8, at most 32 products below 2^52
__device__ __forceinline__ uint64_t p1_dot8(const uint32_t *a, int sa, const uint32_t *b, int sb, int n8) {
    uint64_t x0 = 0, x1 = 0, x2 = 0, x3 = 0;
    for (int q = 0; q < n8; q += 8) {
        uint32_t va[8], vb[8];
#pragma unroll
        for (int k = 0; k < 8; k++) {
            va[k] = a[(q + k) * sa];
            vb[k] = b[(q + k) * sb];
        }
        x0 += (uint64_t)va[0] * vb[0] + (uint64_t)va[4] * vb[4];
        x1 += (uint64_t)va[1] * vb[1] + (uint64_t)va[5] * vb[5];
        x2 += (uint64_t)va[2] * vb[2] + (uint64_t)va[6] * vb[6];
        x3 += (uint64_t)va[3] * vb[3] + (uint64_t)va[7] * vb[7];
    }
    return (x0 + x1) + (x2 + x3);
}
__device__ __forceinline__ void p1_named_sync(int id, int nthreads) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

__global__ void __launch_bounds__(P1_THREADS, 1) k_panel1(PanelArgs a) {
    extern __shared__ __align__(16) int32_t p1s[];
    __shared__ uint32_t Lv[P1_NB * 33];   // Linv[t][s] at Lv[t * 33 + s], zero above the diagonal
    __shared__ uint32_t s_ut[P1_NB];
    __shared__ unsigned long long red[P1_THREADS / 32];
    __shared__ uint32_t s_inv;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int r0 = a.R0, c0 = a.C0, m = a.m, R = m - r0, nbc = a.nbw;
    const int rs = R + 4;
    const ModP M = a.M;
    const uint32_t N = M.n;
    int32_t *P = p1s;                       // P[j * rs + lr]: panel column j, local row lr
    const uint32_t *Pu = reinterpret_cast<const uint32_t *>(P);
    for (int idx = tid; idx < R * nbc; idx += blockDim.x) {
        const int lr = idx / nbc, j = idx - lr * nbc;
        P[j * rs + lr] = a.W[(int64_t)(r0 + lr) * a.ldw + c0 + j];
    }
    for (int idx = tid; idx < P1_NB * 33; idx += blockDim.x) Lv[idx] = 0;
    __syncthreads();

    int npiv = 0, status = PS_DONE;
    uint32_t ppv = 0;
    int pplr = 0;
    for (int t = 0;; t++) {
        uint32_t g = 0;   // U[t-1][t]
        if (t > 0) {
            const int tp = t - 1;
            const bool nxt = t < nbc && r0 + t < m;
            const int tp8 = (tp + 7) & ~7;
            uint64_t lsum = 0;
            if (warp == P1_INV_WARP) {
                const uint32_t inv = mod_inv_euclid_alu(ppv, N);
                if (lane == 0) s_inv = inv;
            } else {
                if (warp == 0) {
                    if (lane >= tp && lane < nbc) {
                        int32_t *colp = P + lane * rs;
                        if (lane == tp) {
                            colp[pplr] = colp[tp];
                        } else if (pplr != tp) {
                            const int32_t x = colp[tp];
                            colp[tp] = colp[pplr];
                            colp[pplr] = x;
                        }
                    }
                } else if (warp == 1) {
                    if (nxt) {
                        const uint64_t acc = p1_dot8(Lv + lane * 33, 1, Pu + t * rs, 1, tp8);
                        s_ut[lane] = lane < tp ? p1_red(acc, M) : 0u;
                    }
                } else if (warp == 2) {
                    if (lane < tp && pplr != tp) {
                        int32_t *colp = P + lane * rs;
                        const int32_t x = colp[tp];
                        colp[tp] = colp[pplr];
                        colp[pplr] = x;
                    }
                    __syncwarp();
                    lsum = p1_dot8(Pu + tp, rs, Lv + lane, 33, tp8);
                }
                if (nxt) {
                    p1_named_sync(1, P1_INV_WARP * 32);
                    for (int lr = tp + tid; lr < R; lr += P1_INV_WARP * 32)
                        P[t * rs + lr] = (int32_t)p1_red((uint32_t)P[t * rs + lr] + p1_dot8(Pu + lr, rs, s_ut, 1, tp8), M);
                }
            }
            __syncthreads();
            const uint32_t inv = s_inv;
            if (warp == 2)
                Lv[tp * 33 + lane] = lane < tp ? mulmod(p1_red(lsum, M), inv, M) : (lane == tp ? inv : 0u);
            if (tid == 0) {
                P[tp * rs + tp] = (int32_t)mulmod(ppv, inv, M);   // U's diagonal
                a.piv_inv[tp] = (int32_t)inv;
            }
            if (!nxt) break;
            g = mulmod((uint32_t)P[t * rs + tp], inv, M);
            if (warp == 0 && lane == 0) s_ut[tp] = g;
        }
        // column t below its pivot rows, and its largest residue (lowest row on ties)
        unsigned long long best = 0;
        for (int lr = t + tid; lr < R; lr += P1_THREADS) {
            uint32_t v = (uint32_t)P[t * rs + lr];
            if (t > 0) v = p1_red((uint64_t)v + (uint64_t)(uint32_t)P[(t - 1) * rs + lr] * g, M);
            P[t * rs + lr] = v ? (int32_t)(N - v) : 0;
            const unsigned long long key = ((unsigned long long)v << 32) | (0xFFFFFFFFu - (uint32_t)lr);
            best = key > best ? key : best;
        }
        best = warp_max_u64(best);
        if (lane == 0) red[warp] = best;
        __syncthreads();
        best = lane < P1_THREADS / 32 ? red[lane] : 0ull;
#pragma unroll
        for (int o = 4; o > 0; o >>= 1) {
            const unsigned long long x = __shfl_xor_sync(0xffffffffu, best, o);
            best = x > best ? x : best;
        }
        best = __shfl_sync(0xffffffffu, best, 0);
        const uint32_t pv = (uint32_t)(best >> 32);
        if (warp == 0 && lane < t) P[t * rs + lane] = (int32_t)s_ut[lane];
        if (pv == 0) {
            status = PS_ZERO_COL;
            break;
        }
        if (a.l_cols > 0 && c0 + t >= a.l_cols) {
            status = PS_BOUNDS;
            break;
        }
        pplr = (int)(0xFFFFFFFFu - (uint32_t)(best & 0xFFFFFFFFu));
        ppv = pv;
        if (tid == 0) {
            a.piv_row[t] = r0 + pplr;
            a.piv_val[t] = (int32_t)pv;
        }
        npiv = t + 1;
    }
    __syncthreads();
    // the columns after a stop (a zero column is final already): values above the
    // pivot rows by Linv, the rows below by the multipliers
    const int np8 = (npiv + 7) & ~7;
    for (int j = npiv + (status == PS_ZERO_COL ? 1 : 0); npiv > 0 && j < nbc; j++) {
        if (warp == 0) {
            const uint64_t acc = p1_dot8(Lv + lane * 33, 1, Pu + j * rs, 1, np8);
            s_ut[lane] = lane < npiv ? p1_red(acc, M) : 0u;
        }
        __syncthreads();
        for (int lr = npiv + tid; lr < R; lr += P1_THREADS)
            P[j * rs + lr] = (int32_t)p1_red((uint32_t)P[j * rs + lr] + p1_dot8(Pu + lr, rs, s_ut, 1, np8), M);
        if (tid < npiv) P[j * rs + tid] = (int32_t)s_ut[tid];
        __syncthreads();
    }
    // back to W: pivot columns hold U on and above the diagonal and the unscaled
    // multipliers below it; the other columns their current residues
    for (int idx = tid; idx < R * nbc; idx += blockDim.x) {
        const int lr = idx / nbc, j = idx - lr * nbc;
        uint32_t x = (uint32_t)P[j * rs + lr];
        if (j < npiv && lr > j) x = x ? N - x : 0u;
        a.W[(int64_t)(r0 + lr) * a.ldw + c0 + j] = (int32_t)x;
    }
    // L11^{-1} for the U12 product (what k_linv computes for the cooperative panel)
    for (int idx = tid; idx < npiv * npiv; idx += blockDim.x) {
        const int i = idx / npiv, j = idx - i * npiv;
        a.linv[i * NB + j] = (int32_t)Lv[i * 33 + j];
    }
    if (tid == 0) {
        a.result[0] = npiv;
        a.result[1] = status;
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

// Columns [0, c_left) and [c_lo, c_hi) in one launch: block b stages the K moved
// rows' values of 32 consecutive columns in shared memory (K x 32 words), then
// writes row rows[k] <- staged row src[k].
__global__ void __launch_bounds__(256) k_rows_permute(int32_t *__restrict__ W, int64_t ldw, int c_left, int c_lo,
                                                      int c_hi, const __grid_constant__ PermArgs p) {
    extern __shared__ int32_t staged[];
    const int nleft = (c_left + 31) / 32;
    const int g = blockIdx.x;
    const int cbase = g < nleft ? 32 * g : c_lo + 32 * (g - nleft);
    const int width = min(32, (g < nleft ? c_left : c_hi) - cbase);
    for (int e = threadIdx.x; e < p.K * 32; e += blockDim.x) {
        const int k = e >> 5, j = e & 31;
        if (j < width) staged[e] = W[(int64_t)p.rows[k] * ldw + cbase + j];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < p.K * 32; e += blockDim.x) {
        const int k = e >> 5, j = e & 31;
        if (j < width) W[(int64_t)p.rows[k] * ldw + cbase + j] = staged[p.src[k] * 32 + j];
    }
}

}  // namespace elim
