// elim_panel.cuh -- the elimination's panel factorization kernels and the
// row-permutation kernel that follows each panel.
#pragma once

#include "gffm_common.cuh"
#include "modarith.cuh"

namespace elim {

constexpr int NB = 128;             // panel width (pivot columns per panel)
constexpr int PANEL_THREADS = 512;
constexpr int PANEL_WARPS = PANEL_THREADS / 32;
constexpr int MAX_PANEL_CTAS = 160;
constexpr int MAX_PERM_ROWS = 2 * NB;
constexpr int PANEL_MAX_R = 288;    // rows per CTA: threads 0..287 own one row each
constexpr int PANEL_AUX0 = PANEL_MAX_R;              // threads 288..511: publication, polling, Linv rows
constexpr int PANEL_NAUX = PANEL_THREADS - PANEL_AUX0;
constexpr int LU_LD = NB + 1;
// Dynamic shared memory of k_panel: the CTA's rows (NB columns x (R + 1) words,
// column-major) and the square of the panel's U rows and Linv (NB x LU_LD words).
__host__ __device__ constexpr size_t panel_smem_bytes(int R) {
    return ((size_t)NB * (size_t)(R + 1) + (size_t)NB * LU_LD) * 4;
}

enum PanelStatus { PS_DONE = 0, PS_ZERO_COL = 1, PS_TIMEOUT = 2, PS_BOUNDS = 3 };

// Pivot key: value (26 bits) | (0x3FFFFF - row) (22 bits) | step tag (16 bits).
// The largest key is the largest residue, then the lowest row.
__device__ __forceinline__ unsigned long long pkey(uint32_t v, int row) {
    return ((unsigned long long)v << 38) | ((unsigned long long)(0x3FFFFFu - (uint32_t)row) << 16);
}
__device__ __forceinline__ uint32_t pkey_val(unsigned long long k) { return (uint32_t)(k >> 38); }
__device__ __forceinline__ int pkey_row(unsigned long long k) { return (int)(0x3FFFFFu - (uint32_t)((k >> 16) & 0x3FFFFFu)); }

// One CTA's published candidate for a pivot step.  Every word carries the
// step's tag (the key in its low 16 bits, the row words in their high 32 bits),
// so a reader that sees the tag sees the value: no fence between writer and
// reader, and each word is polled on its own.
struct alignas(16) Rec {
    unsigned long long key;      // pkey | tag
    unsigned long long row[NB];  // (tag << 32) | residue
    unsigned long long inv;      // (tag << 32) | the candidate's inverse (the reference's Euclid)
};
// The exchange area: the displaced row's words (two parities), then the records.
constexpr size_t OLD_ROW_WORDS = (size_t)2 * (NB + 1);
__host__ __device__ constexpr size_t exchange_bytes(int G) {
    return OLD_ROW_WORDS * 8 + (size_t)2 * G * sizeof(Rec);
}

struct PanelArgs {
    int32_t *W;
    int64_t ldw;
    int m, n;
    int R0, C0, nbw;   // first pivot row / column, panel width
    int R;             // rows per CTA
    ModP M;
    int l_cols;        // L's padded width (PLUQ bound check), <= 0: no check
    Rec *rec;          // [2][G], zero at launch
    unsigned long long *old_row;  // [2][NB + 1], zero at launch
    int32_t *piv_row, *piv_val, *piv_inv;  // [NB]
    int32_t *linv;     // L11^{-1} of the panel's pivots, row-major, ld NB
    int *result;       // [0] pivots, [1] status
    int *err;
};

__device__ __forceinline__ void st_relaxed_u64(unsigned long long *p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
// The value of a row word once it carries `tag` (bounded wait; false when it gave up).
__device__ __forceinline__ bool wait_row_word(const unsigned long long *p, uint32_t tag, uint32_t &val) {
    unsigned long long w = ld_relaxed_u64(p);
    if ((uint32_t)(w >> 32) != tag) {
        const unsigned long long t0 = gffm_dev::globaltimer();
        while ((uint32_t)((w = ld_relaxed_u64(p)) >> 32) != tag)
            if (gffm_dev::globaltimer() - t0 > gffm_dev::kWaitLimitNs) return false;
    }
    val = (uint32_t)w;
    return true;
}

__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
    const unsigned hi = __reduce_max_sync(0xffffffffu, (unsigned)(v >> 32));
    const unsigned lo = __reduce_max_sync(0xffffffffu, (unsigned)(v >> 32) == hi ? (unsigned)v : 0u);
    return ((unsigned long long)hi << 32) | lo;
}

__device__ __forceinline__ uint32_t p1_red(uint64_t x, const ModP &M) {
    return (uint32_t)gffm_dev::barrett64(x, M.n, M.minv);
}
// sum_{s < n8} a[s * sa] * b[s * sb], n8 a multiple of 8, at most 128 products below 2^52
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

// Row tp of the inverse of the panel's lower-triangular factor (pivot values on
// the diagonal, negated multipliers Lneg = N - l below), thread s < tp:
//   Linv[tp][s] = inv * sum_{s <= q < tp} Lneg_tp[q] Linv[q][s],   Linv[tp][tp] = inv.
// lp: Lneg_tp, zero from tp on.  LU[q][s] for q < s holds U, hence the mask.
__device__ __forceinline__ void linv_row(uint32_t *LU, const uint32_t *lp, int tp, uint32_t inv, int s,
                                         const ModP &M) {
    if (s < tp) {
        uint64_t x0 = 0, x1 = 0;
        for (int q = s & ~7; q < tp; q += 8) {
            uint32_t va[8], vb[8];
#pragma unroll
            for (int k = 0; k < 8; k++) {
                va[k] = q + k >= s ? lp[q + k] : 0u;
                vb[k] = LU[(q + k) * LU_LD + s];
            }
#pragma unroll
            for (int k = 0; k < 8; k += 2) {
                x0 += (uint64_t)va[k] * vb[k];
                x1 += (uint64_t)va[k + 1] * vb[k + 1];
            }
        }
        LU[tp * LU_LD + s] = mulmod(p1_red(x0 + x1, M), inv, M);
    } else if (s == tp) {
        LU[tp * LU_LD + tp] = inv;
    }
}
// Row tp of U for column c > tp + 1 (thread c):
//   U[tp][c] = inv * (W_tp[c] + sum_{s < tp} Lneg_tp[s] U[s][c]),
// W_tp the pivot row's residues, lp its negated multipliers (zero from tp on).
__device__ __forceinline__ void u_row(uint32_t *LU, const uint32_t *piv, const uint32_t *lp, int tp, uint32_t inv,
                                      int c, const ModP &M) {
    const uint64_t acc = p1_dot8(lp, 1, LU + c, LU_LD, (tp + 7) & ~7);
    LU[tp * LU_LD + c] = mulmod(p1_red(acc + piv[c], M), inv, M);
}

// Cooperative left-looking panel factorization.  CTA b keeps rows
// [R0 + b*R, R0 + (b+1)*R) of columns [C0, C0 + nbw) in shared memory,
// column-major, thread lr < R owning row lr.  Column t is brought up to date
// only when the pivot search reaches it:
//   v[r] = W[r][t] + sum_{s<t} Lneg[r][s] U[s][t],
// Lneg = N - l the negated multipliers -- one exact 64-bit dot product per row,
// reduced once.  Every CTA keeps the same U rows of the panel's pivots,
//   U[s][c] = inv_s (W_s[c] + sum_{s'<s} Lneg_s[s'] U[s'][c]),
// (the reference's row scaling and updates in closed form) and the inverse Linv
// of the panel's lower-triangular factor, in one square (LU).  Per pivot step t:
//   A. each CTA publishes its candidate (largest residue of column t in its rows,
//      lowest row on ties): the key and the row, as tagged words; the owner of
//      row r = R0 + t publishes that row too,
//   B. while two auxiliary warps poll the G keys (bounded waits), four form
//      Linv's row t-1 and one computes the inverse of the CTA's own candidate
//      (the reference's Euclid) and publishes it as a tagged word, the row
//      threads form U's row t-1 and the partial values
//      y[r] = W[r][t+1] + sum_{s<t} Lneg[r][s] U[s][t+1]; the owner of row r
//      publishes y[r],
//   C. every warp picks the same winner; the CTA fetches its row and its
//      inverse (and, where the winner lands, the displaced row r with y[r]):
//      every CTA inverted its own candidate during B, so the winner's inverse
//      is off the critical path,
//   D. every warp forms U[t][t+1] = inv (W_t[t+1] + sum_{s<t} Lneg_t[s] U[s][t+1]);
//      the row threads complete column t+1, v[r] = y[r] + Lneg[r][t] U[t][t+1],
//      and the CTA's next candidate is its largest v while the auxiliary warps
//      move the two rows.
// The panel is written back with the pivot rows scaled (U), the multipliers
// unscaled below the pivots and the columns after a stop brought up to date;
// CTA 0 writes L11^{-1} for the product U12 = L11^{-1} P A12.
__global__ void __launch_bounds__(PANEL_THREADS, 1) k_panel(PanelArgs a) {
    extern __shared__ __align__(16) uint32_t psm[];
    const int R = a.R, rs = R + 1;
    uint32_t *P = psm;                      // P[j * rs + lr]
    uint32_t *LU = psm + (size_t)NB * rs;   // LU[s * LU_LD + c]: Linv (c <= s), U (c > s); zero until formed
    __shared__ unsigned long long keys[MAX_PANEL_CTAS];
    __shared__ __align__(16) uint32_t s_piv[NB];     // the pivot row: Lneg (c < t), residues (c > t)
    __shared__ __align__(16) uint32_t s_lp[NB + 8];  // its negated multipliers, zero from t on
    __shared__ uint32_t s_old[NB + 1];               // the displaced row, and its partial value of column t+1
    __shared__ unsigned long long red[PANEL_WARPS];
    __shared__ int s_stop, s_stop_c, s_status;   // timeouts while polling keys / fetching the pivot row
    __shared__ uint32_t s_inv;
    __shared__ int32_t s_rec[3][NB];                 // pivot rows, values, inverses (written out after the loop)
    const int b = blockIdx.x, G = gridDim.x, tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    const int rbeg = a.R0 + b * R;
    const int rend = min(rbeg + R, a.m);
    const int nr = max(rend - rbeg, 0);
    const int nbw = a.nbw;
    const ModP M = a.M;
    const uint32_t N = M.n;
    const int lr = tid, grow = rbeg + tid;
    const bool own = tid < nr;
    const int x = tid - PANEL_AUX0;         // auxiliary thread index (>= 0)

    for (int e = tid; e < nr * nbw; e += PANEL_THREADS) {
        const int i = e / nbw, j = e - i * nbw;
        P[j * rs + i] = (uint32_t)a.W[(int64_t)(rbeg + i) * a.ldw + a.C0 + j];
    }
    for (int i = tid; i < NB * LU_LD; i += PANEL_THREADS) LU[i] = 0;
    for (int i = tid; i < NB + 8; i += PANEL_THREADS) s_lp[i] = 0;
    if (tid == 0) {
        s_stop = 0;
        s_stop_c = 0;
        s_status = PS_DONE;
    }
    __syncthreads();
    // column 0: negated multipliers and the first candidate
    unsigned long long best = 0;
    if (own) {
        const uint32_t v = P[lr];
        P[lr] = v ? N - v : 0u;
        best = pkey(v, grow);
    }
    best = warp_max_u64(best);
    if (lane == 0) red[warp] = best;
    __syncthreads();
    best = warp_max_u64(lane < PANEL_WARPS ? red[lane] : 0ull);

    const int tmax = min(nbw, a.m - a.R0);
    uint64_t y = 0;   // this row's partial value of column t+1
    int t = 0;
    for (; t < tmax; t++) {
        const int r = a.R0 + t;
        const int par = t & 1;
        const uint32_t tag = (uint32_t)(t + 1);
        const bool owner_r = r >= rbeg && r < rend;
        const bool next = t + 1 < nbw;
        unsigned long long *oldw = a.old_row + par * (NB + 1);
        Rec *recs = a.rec + par * G;
        if (x >= 0) {
            // A. publication
            if (x < NB) {
                if (best != 0 && x < nbw)
                    st_relaxed_u64(&recs[b].row[x],
                                   ((unsigned long long)tag << 32) | P[x * rs + (pkey_row(best) - rbeg)]);
                if (x == 0) st_relaxed_u64(&recs[b].key, best | tag);
            } else if (owner_r) {
                for (int j = x - NB; j < nbw; j += PANEL_NAUX - NB)
                    st_relaxed_u64(&oldw[j], ((unsigned long long)tag << 32) | P[j * rs + (r - rbeg)]);
            }
            // B. two warps poll the keys, four form Linv's row t-1
            if (x < 64) {
                const int g0 = x, g1 = x + 64, g2 = x + 128;
                unsigned pend = (g0 < G ? 1u : 0u) | (g1 < G ? 2u : 0u) | (g2 < G ? 4u : 0u);
                const unsigned long long t0 = gffm_dev::globaltimer();
                while (pend) {
                    const unsigned long long k0 = (pend & 1u) ? ld_relaxed_u64(&recs[g0].key) : 0ull;
                    const unsigned long long k1 = (pend & 2u) ? ld_relaxed_u64(&recs[g1].key) : 0ull;
                    const unsigned long long k2 = (pend & 4u) ? ld_relaxed_u64(&recs[g2].key) : 0ull;
                    if ((pend & 1u) && (k0 & 0xFFFFull) == tag) { keys[g0] = k0 & ~0xFFFFull; pend &= ~1u; }
                    if ((pend & 2u) && (k1 & 0xFFFFull) == tag) { keys[g1] = k1 & ~0xFFFFull; pend &= ~2u; }
                    if ((pend & 4u) && (k2 & 0xFFFFull) == tag) { keys[g2] = k2 & ~0xFFFFull; pend &= ~4u; }
                    if (pend && gffm_dev::globaltimer() - t0 > gffm_dev::kWaitLimitNs) {
                        atomicOr(a.err, 16);
                        s_stop = 1;
                        s_status = PS_TIMEOUT;
                        break;
                    }
                }
            } else if (x < 64 + NB && t > 0) {
                linv_row(LU, s_lp, t - 1, s_inv, x - 64, M);
            } else if (x == 64 + NB && best != 0) {
                // the inverse of this CTA's candidate, in case it wins
                st_relaxed_u64(&recs[b].inv, ((unsigned long long)tag << 32) | mod_inv_euclid_alu(pkey_val(best), N));
            }
        } else {
            // B. the row threads: U's row t-1, then the partial values of column t+1
            if (t > 0 && tid > t && tid < nbw) u_row(LU, s_piv, s_lp, t - 1, s_inv, tid, M);
            p1_named_sync(1, PANEL_AUX0);
            if (next && own && grow >= r) {
                y = (uint64_t)P[(t + 1) * rs + lr] + p1_dot8(P + lr, rs, LU + t + 1, LU_LD, (t + 7) & ~7);
                if (grow == r) st_relaxed_u64(&oldw[NB], ((unsigned long long)tag << 32) | p1_red(y, M));
            }
        }
        __syncthreads();
        if (s_stop) break;
        // C. the global pivot (every warp decides the same)
        unsigned long long wk = 0;
        for (int g = lane; g < G; g += 32) wk = keys[g] > wk ? keys[g] : wk;
        wk = warp_max_u64(wk);
        const uint32_t pv = pkey_val(wk);
        if (pv == 0 || (a.l_cols > 0 && a.C0 + t >= a.l_cols)) {
            if (tid == 0) s_status = pv == 0 ? PS_ZERO_COL : PS_BOUNDS;
            break;
        }
        const int prow = pkey_row(wk);
        const int bw = (prow - a.R0) / R;
        const bool lands = bw == b && prow != r;   // the displaced row r moves into this CTA
        if (tid < nbw) {
            uint32_t v = 0;
            if (!wait_row_word(&a.rec[par * G + bw].row[tid], tag, v)) {
                atomicOr(a.err, 16);
                s_stop_c = 1;
                s_status = PS_TIMEOUT;
            }
            s_piv[tid] = v;
            s_lp[tid] = tid < t ? v : 0u;
        } else if (tid >= NB && tid <= 2 * NB && lands) {
            const int j = tid - NB;
            if (j < nbw || (j == NB && next)) {
                uint32_t v = 0;
                if (!wait_row_word(&oldw[j], tag, v)) {
                    atomicOr(a.err, 16);
                    s_stop_c = 1;
                    s_status = PS_TIMEOUT;
                }
                s_old[j] = v;
            }
        } else if (tid == PANEL_THREADS - 32) {
            uint32_t v = 0;
            if (!wait_row_word(&a.rec[par * G + bw].inv, tag, v)) {
                atomicOr(a.err, 16);
                s_stop_c = 1;
                s_status = PS_TIMEOUT;
            }
            s_inv = v;
        }
        __syncthreads();
        if (s_stop_c) break;
        // D. U[t][t+1] (every warp), column t+1 and the next candidate (row threads),
        //    the row moves (auxiliary threads)
        const uint32_t inv = s_inv;
        uint32_t g = 0;
        if (next) {
            uint64_t acc = 0;
            for (int s = lane; s < t; s += 32) acc += (uint64_t)s_lp[s] * LU[s * LU_LD + t + 1];
            const uint32_t part = __reduce_add_sync(0xffffffffu, p1_red(acc, M));   // 32 residues: below 2^31
            g = mulmod(p1_red((uint64_t)part + s_piv[t + 1], M), inv, M);
        }
        best = 0;
        if (x < 0) {
            if (next && own) {
                if (grow > r) {
                    const bool moved = lands && grow == prow;
                    const uint32_t lt = moved ? s_old[t] : P[t * rs + lr];
                    const uint64_t yy = moved ? (uint64_t)s_old[NB] : y;
                    const uint32_t v = p1_red(yy + (uint64_t)lt * g, M);
                    P[(t + 1) * rs + lr] = v ? N - v : 0u;
                    best = pkey(v, grow);
                } else {
                    const int s = grow - a.R0;
                    P[(t + 1) * rs + lr] = s < t ? LU[s * LU_LD + t + 1] : g;
                }
            }
        } else {
            if (owner_r)
                for (int j = x; j <= t; j += PANEL_NAUX) P[j * rs + (r - rbeg)] = j < t ? s_piv[j] : mulmod(pv, inv, M);
            if (lands)
                for (int j = x; j < nbw; j += PANEL_NAUX)
                    if (j != t + 1) P[j * rs + (prow - rbeg)] = s_old[j];
            if (x == 0) {
                if (next) LU[t * LU_LD + t + 1] = g;
                s_rec[0][t] = prow;
                s_rec[1][t] = (int32_t)pv;
                s_rec[2][t] = (int32_t)inv;
            }
        }
        best = warp_max_u64(best);
        if (lane == 0) red[warp] = best;
        __syncthreads();
        best = warp_max_u64(lane < PANEL_WARPS ? red[lane] : 0ull);
    }
    __syncthreads();
    const int npiv = t, status = s_status;
    if (npiv > 0 && (status == PS_DONE || status == PS_ZERO_COL)) {
        // the last pivot's rows of Linv and U, then the columns after a stop (the
        // column at a zero stop is final already): U above, the multipliers below
        if (x >= 0 && x < NB) linv_row(LU, s_lp, npiv - 1, s_inv, x, M);
        if (x < 0 && tid > npiv && tid < nbw) u_row(LU, s_piv, s_lp, npiv - 1, s_inv, tid, M);
        __syncthreads();
        if (own)
            for (int j = npiv + 1; j < nbw; j++) {
                if (grow >= a.R0 + npiv)
                    P[j * rs + lr] = p1_red((uint64_t)P[j * rs + lr] + p1_dot8(P + lr, rs, LU + j, LU_LD, (npiv + 7) & ~7), M);
                else
                    P[j * rs + lr] = LU[(grow - a.R0) * LU_LD + j];
            }
        __syncthreads();
    }
    // back to W: pivot columns hold U on and above the diagonal and the unscaled
    // multipliers below it; the other columns their current residues
    for (int e = tid; e < nr * nbw; e += PANEL_THREADS) {
        const int i = e / nbw, j = e - i * nbw;
        uint32_t v = P[j * rs + i];
        if (j < npiv && rbeg + i > a.R0 + j) v = v ? N - v : 0u;
        a.W[(int64_t)(rbeg + i) * a.ldw + a.C0 + j] = (int32_t)v;
    }
    if (b == 0) {
        for (int e = tid; e < npiv; e += PANEL_THREADS) {
            a.piv_row[e] = s_rec[0][e];
            a.piv_val[e] = s_rec[1][e];
            a.piv_inv[e] = s_rec[2][e];
        }
        for (int e = tid; e < npiv * npiv; e += PANEL_THREADS) {
            const int i = e / npiv, j = e - i * npiv;
            a.linv[i * NB + j] = j <= i ? (int32_t)LU[i * LU_LD + j] : 0;
        }
        if (tid == 0) {
            a.result[0] = npiv;
            a.result[1] = status;
        }
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
constexpr int P1_MAX_ROWS = 512;
__host__ __device__ constexpr size_t p1_smem_bytes(int rows) { return (size_t)P1_NB * (size_t)(rows + 4) * 4; }

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
        // warp 1 alone rewrites s_ut (for column t+1, before the next barrier): it copies
        // column t's values above the pivot rows, each lane before its own next write
        if (warp == 1 && lane < t) P[t * rs + lane] = (int32_t)s_ut[lane];
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
    // L11^{-1} for the U12 product
    for (int idx = tid; idx < npiv * npiv; idx += blockDim.x) {
        const int i = idx / npiv, j = idx - i * npiv;
        a.linv[i * NB + j] = (int32_t)Lv[i * 33 + j];
    }
    if (tid == 0) {
        a.result[0] = npiv;
        a.result[1] = status;
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

// ---------------------------------------------------------------------------
// Tall panels: more rows below the panel than the cooperative kernel holds in
// shared memory (MAX_PANEL_CTAS x PANEL_MAX_R, fewer on a GPU with fewer SMs).
// A tall panel is at most TALL_NB columns wide and factors right-looking in
// global memory, three launches per pivot step t:
//   k_tall_search  the pivot: largest residue of column t below row R0 + t,
//                  lowest row on ties (one 64-bit atomic max of
//                  value << 32 | (2^32 - 1 - row)),
//   k_tall_pivot   one warp: a zero column (or L's bound) stops the panel;
//                  otherwise the pivot's inverse (the reference's Euclid), the
//                  swap of rows R0 + t and the pivot row in the panel's
//                  columns, the new pivot row scaled from column t on,
//   k_tall_update  the rows below: W[r][c] -= l_r U[t][c] for the panel's
//                  columns c > t, l_r = W[r][t] (kept unscaled: the multiplier).
// k_tall_finish then writes the pivot count, the status and L11^{-1}.  The
// panel ends as k_panel leaves it: U on and above the diagonal, the unscaled
// multipliers below it, the columns after a stop up to date, the pivot records
// and L11^{-1}; the blocked algorithm around it is unchanged.  No waits.
constexpr int TALL_NB = 32;

struct TallArgs {
    int32_t *W;
    int64_t ldw;
    int m, R0, C0, nbw;
    ModP M;
    int l_cols;                  // L's padded width (PLUQ bound check), <= 0: no check
    unsigned long long *key;     // the step's pivot key, zero before each search
    int *state;                  // [0] stopped, [1] pivots at the stop, [2] status of the stop
    uint32_t *urow;              // [TALL_NB] the step's scaled pivot row
    int32_t *piv_row, *piv_val, *piv_inv;
    int32_t *linv;               // L11^{-1}, row-major, ld NB
    int *result;                 // [0] pivots, [1] status
};

__global__ void __launch_bounds__(256) k_tall_search(TallArgs a, int t) {
    __shared__ unsigned long long red[8];
    if (*(volatile int *)a.state) return;
    const int c = a.C0 + t;
    unsigned long long best = 0;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t r = a.R0 + t + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < a.m; r += stride) {
        const unsigned long long k =
            ((unsigned long long)(uint32_t)a.W[r * a.ldw + c] << 32) | (0xFFFFFFFFu - (uint32_t)r);
        best = k > best ? k : best;
    }
    best = warp_max_u64(best);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = best;
    __syncthreads();
    if (threadIdx.x < 32) {
        best = warp_max_u64(threadIdx.x < 8 ? red[threadIdx.x] : 0ull);
        if (threadIdx.x == 0 && best) atomicMax(a.key, best);
    }
}

__global__ void __launch_bounds__(TALL_NB) k_tall_pivot(TallArgs a, int t) {
    __shared__ uint32_t s_inv;
    if (*(volatile int *)a.state) return;
    const int tid = threadIdx.x;
    const unsigned long long key = *(volatile unsigned long long *)a.key;
    const uint32_t pv = (uint32_t)(key >> 32);
    const int prow = (int)(0xFFFFFFFFu - (uint32_t)key);
    const int r = a.R0 + t;
    __syncwarp();
    if (pv == 0 || (a.l_cols > 0 && a.C0 + t >= a.l_cols)) {
        if (tid == 0) {
            a.state[1] = t;
            a.state[2] = pv == 0 ? PS_ZERO_COL : PS_BOUNDS;
            a.state[0] = 1;
        }
        return;
    }
    if (tid == 0) s_inv = mod_inv_euclid_alu(pv, a.M.n);
    __syncwarp();
    const uint32_t inv = s_inv;
    if (tid < a.nbw) {
        int32_t *wr = a.W + (int64_t)r * a.ldw + a.C0;
        int32_t *wp = a.W + (int64_t)prow * a.ldw + a.C0;
        const uint32_t vr = (uint32_t)wr[tid], vp = (uint32_t)wp[tid];
        // earlier columns: the rows' multipliers move unscaled; from column t on the pivot row is
        // scaled (each thread reads and writes only its own column)
        const uint32_t u = tid >= t ? mulmod(vp, inv, a.M) : vp;
        wr[tid] = (int32_t)u;
        if (prow != r) wp[tid] = (int32_t)vr;
        a.urow[tid] = u;
    }
    if (tid == 0) {
        *a.key = 0;
        a.piv_row[t] = prow;
        a.piv_val[t] = (int32_t)pv;
        a.piv_inv[t] = (int32_t)inv;
    }
}

// one warp per row, lane j on column t + 1 + j
__global__ void __launch_bounds__(256) k_tall_update(TallArgs a, int t) {
    if (*(volatile int *)a.state) return;
    const int w = a.nbw - t - 1;
    if (w <= 0) return;
    const int lane = threadIdx.x & 31;
    const uint32_t N = a.M.n;
    const uint32_t u = lane < w ? a.urow[t + 1 + lane] : 0u;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t r = a.R0 + t + 1 + ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32; r < a.m; r += warps) {
        int32_t *row = a.W + r * a.ldw + a.C0;
        const uint32_t l = (uint32_t)row[t];
        if (lane < w && l != 0) {
            const uint32_t x = (uint32_t)row[t + 1 + lane];
            row[t + 1 + lane] = (int32_t)p1_red((uint64_t)x + (uint64_t)(N - l) * u, a.M);
        }
    }
}

// one warp: the pivot count and status, and L11^{-1} (pivot values on L11's diagonal,
// the unscaled multipliers below it): Linv[t][t] = inv_t,
// Linv[t][s] = inv_t * sum_{s <= q < t} (N - l_t[q]) Linv[q][s]
__global__ void __launch_bounds__(32) k_tall_finish(TallArgs a, int tmax) {
    __shared__ uint32_t Li[TALL_NB][TALL_NB + 1];
    const int s = threadIdx.x;
    const int stopped = *(volatile int *)a.state;
    const int npiv = stopped ? a.state[1] : tmax;
    const int status = stopped ? a.state[2] : PS_DONE;
    const uint32_t N = a.M.n;
    for (int t = 0; t < npiv; t++) {
        const uint32_t inv = (uint32_t)a.piv_inv[t];
        if (s < t) {
            const int32_t *lt = a.W + (int64_t)(a.R0 + t) * a.ldw + a.C0;
            uint64_t acc = 0;
            for (int q = s; q < t; q++) {
                const uint32_t l = (uint32_t)lt[q];
                acc += (uint64_t)(l ? N - l : 0u) * Li[q][s];
            }
            Li[t][s] = mulmod(p1_red(acc, a.M), inv, a.M);
        } else if (s == t) {
            Li[t][t] = inv;
        }
        __syncwarp();
    }
    for (int i = 0; i < npiv; i++)
        if (s < npiv) a.linv[i * NB + s] = s <= i ? (int32_t)Li[i][s] : 0;
    if (s == 0) {
        a.result[0] = npiv;
        a.result[1] = status;
    }
}

}  // namespace elim
