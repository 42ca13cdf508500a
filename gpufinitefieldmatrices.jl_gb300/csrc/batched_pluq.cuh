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
// (and LW for L).  A panel of nb <= 32 columns is copied into shared memory and
// factored left-looking: column t is brought up to date only when the pivot
// search reaches it, its values above the pivot rows by the inverse of the
// panel's lower-triangular factor L' (pivots on the diagonal, multipliers l
// below; its inverse Linv grows by one row per pivot) and the rows below by one
// exact dot product each,
//     U[0:t][t] = Linv W[0:t][t],      v[r] = W[r][t] - sum_{s<t} l[r][s] U[s][t],
// 64-bit sums of at most 32 products below 2^52, reduced once.  The rest of
// every row is brought up to date once per panel: the panel's row swaps
// composed into one set of row moves, the pivot rows of the trailing columns
// by the same Linv product, and the rows below by one K = nb product.  Columns
// left of the panel only see the moves and the pivot-row scaling (they matter
// for the stale columns a zero-column swap leaves behind).  A zero column ends
// the panel; it is final at that point (zero below the pivot rows), and the
// panel's columns after it join the trailing update, so the last column it is
// swapped with is current.
//
// L's columns are stored by row identity, not position: a panel writes its
// multipliers into LW at the row each position held at the start (`ident`, kept
// in shared memory and moved with the rows), and the conversion to column-major
// output reads row ident[r] for output row r.  Later panels' swaps then cost one
// move of m identities instead of a move of every earlier L column.  Columns at
// or past L's swap width keep positions (they must not see later swaps).
#pragma once

#include "gffm_common.cuh"
#include "modarith.cuh"

namespace batched {

constexpr int PQ_THREADS = 256;
constexpr int PQ_CW = 128;          // trailing columns per chunk
constexpr int PQ_MAX_NB = 32;
constexpr int PQ_MAX_MOVES = 2 * PQ_MAX_NB;
constexpr int PQ_INV_WARP = 7;       // the warp that computes pivot inverses (the last one)
static_assert(PQ_INV_WARP * 32 + 32 == PQ_THREADS, "the inverse warp is the CTA's last warp");

struct PQInst {
    int m, n, l_cols, lsw;       // lsw = min(32*cld(m, 32), l_cols): L's row-swap width
    elim::ModP M;                // N, floor((2^64-1)/N)
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
    int32_t *tmp;                // per-CTA row-move buffers: PQ_MAX_MOVES rows of W
    int tmp_ldw;                 // their row stride (>= every ldw)
    const int *flags;            // per instance: factor it only if nonzero (null: every instance)
};

// shared-memory words a CTA needs for panel height rcap: panel, trailing pivot rows
// and the panel's row source map (rcap words) -- at least the 8 transpose tiles of
// 32 x 33 words the conversions use -- then the row identities (rcap words), which
// the conversions read
__host__ __device__ constexpr size_t pq_ident_offset(int rcap) {
    return (size_t)PQ_MAX_NB * (rcap + 4) + (size_t)PQ_MAX_NB * PQ_CW + (size_t)rcap > (size_t)8 * 32 * 33
               ? (size_t)PQ_MAX_NB * (rcap + 4) + (size_t)PQ_MAX_NB * PQ_CW + (size_t)rcap
               : (size_t)8 * 32 * 33;
}
__host__ __device__ constexpr size_t pq_smem_words(int rcap) { return pq_ident_offset(rcap) + (size_t)rcap; }

struct PQShared {
    int piv_prow[PQ_MAX_NB];     // absolute row swapped into pivot row r0 + t
    uint32_t piv_val[PQ_MAX_NB];
    uint32_t piv_inv[PQ_MAX_NB];
    int mv_dst[PQ_MAX_MOVES], mv_src[PQ_MAX_MOVES];
    uint32_t mv_scale[PQ_MAX_MOVES];   // 0: plain move; else the pivot inverse of a pivot row
    unsigned long long red[PQ_THREADS / 32];
    uint32_t inv;                // the pending pivot's inverse
    int nmv, inst;
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

// Column-major Float64 (m x n, ld) <-> row-major int32 (m x n, ldw) through
// 32 x 32 shared tiles, PQ_TPR tiles per round (scratch: PQ_TPR x 32 x 33 words):
// every thread issues all 4 * PQ_TPR loads of a round before its first store.
constexpr int PQ_TPR = 8;   // pq_smem_words reserves PQ_TPR * 32 * 33 words at least

__device__ void to_rowmajor(const double *A, int64_t lda, int32_t *W, int ldw, int m, int n, const elim::ModP &M,
                            int32_t *scratch) {
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;   // 8 rows of 32 threads
    const int tc = (n + 31) >> 5, nt = ((m + 31) >> 5) * tc;
    for (int t0 = 0; t0 < nt; t0 += PQ_TPR) {
        double v[PQ_TPR][4];
#pragma unroll
        for (int q = 0; q < PQ_TPR; q++) {
            const int r0 = ((t0 + q) / tc) * 32, c0 = ((t0 + q) % tc) * 32;
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int r = r0 + tx, c = c0 + ty + 8 * i;
                v[q][i] = (t0 + q < nt && r < m && c < n) ? A[r + (int64_t)c * lda] : 0.0;
            }
        }
#pragma unroll
        for (int q = 0; q < PQ_TPR; q++)
#pragma unroll
            for (int i = 0; i < 4; i++) scratch[q * 1056 + (ty + 8 * i) * 33 + tx] = (int32_t)residue_of(v[q][i], M);
        __syncthreads();
#pragma unroll
        for (int q = 0; q < PQ_TPR; q++) {
            if (t0 + q >= nt) break;
            const int r0 = ((t0 + q) / tc) * 32, c0 = ((t0 + q) % tc) * 32;
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int r = r0 + ty + 8 * i, c = c0 + tx;
                if (r < m && c < n) W[(int64_t)r * ldw + c] = scratch[q * 1056 + tx * 33 + ty + 8 * i];
            }
        }
        __syncthreads();
    }
}

// Columns c < map_cols read row rowmap[r] for output row r (rowmap may be null when
// map_cols is 0); with tri_block > 0 such a column is zero in the rows above its block of
// tri_block columns, which are not read.
__device__ void to_colmajor(const int32_t *W, int ldw, int wcols, double *A, int64_t lda, int m, int n,
                            int32_t *scratch, const int *rowmap = nullptr, int map_cols = 0, int tri_block = 0) {
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int tc = (n + 31) >> 5, nt = ((m + 31) >> 5) * tc;
    for (int t0 = 0; t0 < nt; t0 += PQ_TPR) {
        int32_t v[PQ_TPR][4];
#pragma unroll
        for (int q = 0; q < PQ_TPR; q++) {
            const int r0 = ((t0 + q) / tc) * 32, c0 = ((t0 + q) % tc) * 32;
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int r = r0 + ty + 8 * i, c = c0 + tx;
                const bool in = t0 + q < nt && r < m && c < wcols && !(tri_block && c < map_cols && r < c - c % tri_block);
                v[q][i] = in ? W[(int64_t)(c < map_cols ? rowmap[r] : r) * ldw + c] : 0;
            }
        }
#pragma unroll
        for (int q = 0; q < PQ_TPR; q++)
#pragma unroll
            for (int i = 0; i < 4; i++) scratch[q * 1056 + (ty + 8 * i) * 33 + tx] = v[q][i];
        __syncthreads();
#pragma unroll
        for (int q = 0; q < PQ_TPR; q++) {
            if (t0 + q >= nt) break;
            const int r0 = ((t0 + q) / tc) * 32, c0 = ((t0 + q) % tc) * 32;
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int r = r0 + tx, c = c0 + ty + 8 * i;
                if (r < m && c < n) A[r + (int64_t)c * lda] = (double)scratch[q * 1056 + tx * 33 + ty + 8 * i];
            }
        }
        __syncthreads();
    }
}

// Row moves of a panel on columns [c_lo, c_hi) of a row-major int32 matrix: gather
// the sources into T (one row per move, stride ldt), then write the destinations
// (times the pivot inverse for pivot rows when `scale`).  A warp per move row.
__device__ __forceinline__ void gather_moves(const int32_t *X, int ldx, int c_lo, int c_hi, int32_t *T, int ldt,
                                             const PQShared &S) {
    const int lane = threadIdx.x & 31;
    for (int k = threadIdx.x >> 5; k < S.nmv; k += blockDim.x >> 5) {
        const int32_t *src = X + (int64_t)S.mv_src[k] * ldx;
        int32_t *dst = T + (int64_t)k * ldt;
        for (int c = c_lo + lane; c < c_hi; c += 128) {
            int32_t v[4];
#pragma unroll
            for (int u = 0; u < 4; u++) v[u] = c + 32 * u < c_hi ? src[c + 32 * u] : 0;
#pragma unroll
            for (int u = 0; u < 4; u++)
                if (c + 32 * u < c_hi) dst[c + 32 * u] = v[u];
        }
    }
}
__device__ __forceinline__ void scatter_moves(int32_t *X, int ldx, int c_lo, int c_hi, const int32_t *T, int ldt,
                                              const PQShared &S, bool scale, const elim::ModP &M) {
    const int lane = threadIdx.x & 31;
    for (int k = threadIdx.x >> 5; k < S.nmv; k += blockDim.x >> 5) {
        const int32_t *src = T + (int64_t)k * ldt;
        int32_t *dst = X + (int64_t)S.mv_dst[k] * ldx;
        const uint32_t sc = scale ? S.mv_scale[k] : 0u;
        for (int c = c_lo + lane; c < c_hi; c += 128) {
            int32_t v[4];
#pragma unroll
            for (int u = 0; u < 4; u++) v[u] = c + 32 * u < c_hi ? src[c + 32 * u] : 0;
#pragma unroll
            for (int u = 0; u < 4; u++)
                if (c + 32 * u < c_hi) dst[c + 32 * u] = sc ? (int32_t)elim::mulmod((uint32_t)v[u], sc, M) : v[u];
        }
    }
}

// sum_{s < n8} a[s * sa] * b[s * sb] for n8 a multiple of 8 (at most 32 products below
// 2^52): four accumulators, the eight loads of a chunk issued together
__device__ __forceinline__ uint64_t dot8(const uint32_t *a, int sa, const uint32_t *b, int sb, int n8) {
    uint64_t x0 = 0, x1 = 0, x2 = 0, x3 = 0;
    for (int s = 0; s < n8; s += 8) {
        uint32_t va[8], vb[8];
#pragma unroll
        for (int k = 0; k < 8; k++) {
            va[k] = a[(s + k) * sa];
            vb[k] = b[(s + k) * sb];
        }
        x0 += (uint64_t)va[0] * vb[0] + (uint64_t)va[4] * vb[4];
        x1 += (uint64_t)va[1] * vb[1] + (uint64_t)va[5] * vb[5];
        x2 += (uint64_t)va[2] * vb[2] + (uint64_t)va[6] * vb[6];
        x3 += (uint64_t)va[3] * vb[3] + (uint64_t)va[7] * vb[7];
    }
    return (x0 + x1) + (x2 + x3);
}

__device__ __forceinline__ void named_sync(int id, int nthreads) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// the largest 64-bit key of the warp, in every lane: two 32-bit max reductions
__device__ __forceinline__ unsigned long long pq_warp_max(unsigned long long v) {
    const unsigned hi = __reduce_max_sync(0xffffffffu, (unsigned)(v >> 32));
    const unsigned lo = __reduce_max_sync(0xffffffffu, (unsigned)(v >> 32) == hi ? (unsigned)v : 0u);
    return ((unsigned long long)hi << 32) | lo;
}

__device__ __forceinline__ unsigned long long pkey32(uint32_t v, int lr) {
    return ((unsigned long long)v << 32) | (0xFFFFFFFFu - (uint32_t)lr);
}

// The trailing update's 4 x 4 tiles: item i covers rows lr0 .. lr0+3 (local) and
// columns cc .. cc+3 of the current chunk, cc = 8 * (column octet) + 4 * (i & 1).
// In a chunk past the panel (moved), the columns have not seen the panel's row moves
// yet: a row's W values come from row srcmap[lr] (local rows; the identity except for
// the moved rows, whose sources are pivot-block rows still holding their old contents).
struct UpdCtx {
    int32_t *W;
    int ldw, r0, cb, npiv, R, cw, lr_base, trows;
    const int32_t *P;            // the panel; Us and srcmap follow it in shared memory
    int rs;
    bool moved;
    __device__ __forceinline__ const int32_t *us() const { return P + PQ_MAX_NB * rs; }
    __device__ __forceinline__ const int *srcmap() const { return us() + PQ_MAX_NB * PQ_CW; }
};
__device__ __forceinline__ void upd_pos(const UpdCtx &c, int item, int &lr0, int &cc) {
    const int tile = item >> 1, tc = tile / c.trows, tr = tile - tc * c.trows;
    lr0 = c.lr_base + 4 * tr;
    cc = 8 * tc + 4 * (item & 1);
}
__device__ __forceinline__ void upd_load(uint64_t (&a)[4][4], const UpdCtx &c, int item) {
    int lr0, cc;
    upd_pos(c, item, lr0, cc);
#pragma unroll
    for (int x = 0; x < 4; x++) {
        const bool rok = lr0 + x >= c.npiv && lr0 + x < c.R;
        const int lr = (rok && c.moved) ? c.srcmap()[lr0 + x] : lr0 + x;
        const int32_t *w = c.W + (int64_t)(c.r0 + lr) * c.ldw + c.cb + cc;
#pragma unroll
        for (int y = 0; y < 4; y++) a[x][y] = (rok && cc + y < c.cw) ? (uint32_t)w[y] : 0u;
    }
}
__device__ __forceinline__ void upd_mul(uint64_t (&a)[4][4], const UpdCtx &c, int item) {
    int lr0, cc;
    upd_pos(c, item, lr0, cc);
#pragma unroll 4
    for (int t = 0; t < c.npiv; t++) {
        const int4 lq = *reinterpret_cast<const int4 *>(c.P + t * c.rs + lr0);   // negated multipliers
        const int4 uq = *reinterpret_cast<const int4 *>(c.us() + t * PQ_CW + cc);
        const uint32_t lv[4] = {(uint32_t)lq.x, (uint32_t)lq.y, (uint32_t)lq.z, (uint32_t)lq.w};
        const uint32_t uv[4] = {(uint32_t)uq.x, (uint32_t)uq.y, (uint32_t)uq.z, (uint32_t)uq.w};
#pragma unroll
        for (int x = 0; x < 4; x++)
#pragma unroll
            for (int y = 0; y < 4; y++) a[x][y] += (uint64_t)lv[x] * uv[y];
    }
}
__device__ __forceinline__ void upd_store(const uint64_t (&a)[4][4], const UpdCtx &c, int item, const elim::ModP &M) {
    int lr0, cc;
    upd_pos(c, item, lr0, cc);
#pragma unroll
    for (int x = 0; x < 4; x++) {
        if (lr0 + x >= c.npiv && lr0 + x < c.R) {
            int32_t *w = c.W + (int64_t)(c.r0 + lr0 + x) * c.ldw + c.cb + cc;
#pragma unroll
            for (int y = 0; y < 4; y++)
                if (cc + y < c.cw) w[y] = (int32_t)reduce_u64(a[x][y], M);
        }
    }
}

// Left-looking factorization of the panel P (columns [0, nbc), local rows [0, R), pivot
// rows from r0 of an m-row matrix; c0 is the panel's first column, l_cols L's width).
// P holds the panel on entry.  On return (after a barrier) P's columns below their pivot
// rows hold the negated multipliers, on and above them U; Lv holds Linv; S the pivots.
// Returns the pivot count; zero_hit / stop say how the panel ended early.
__device__ __forceinline__ int pq_factor_panel(int32_t *P, int rs, int R, int r0, int m, int nbc, int c0,
                                               int l_cols, const elim::ModP &M, PQShared &S, uint32_t *Lv,
                                               uint32_t *s_ut, int &zero_hit, int &stop) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t N = M.n;
    for (int idx = tid; idx < PQ_MAX_NB * 33; idx += blockDim.x) Lv[idx] = 0;   // rows not applied yet
    __syncthreads();
    int npiv = 0;
    zero_hit = 0;
    stop = 0;
    // Left-looking: column t is brought up to date only when it is reached.
    //   above the pivot rows  U[s][t] = sum_{s' <= s} Linv[s][s'] P[t][s']       (s < t)
    //   below                 v[lr]   = P[t][lr] + sum_{s < t} (N - l[lr][s]) U[s][t]
    // Linv, the inverse of the panel's lower-triangular factor (the pivots on its
    // diagonal, the multipliers below), grows by one row per pivot.  Columns left of t
    // hold U above the diagonal, pv * inv on it and the negated multipliers below it.
    // Pivot t-1 is applied while column t is prepared: warp 7 computes the pivot's
    // inverse; meanwhile warps 0 and 2 swap the rows (columns from t-1 on / left of
    // it), warp 1 forms U[s][t] for s < t-1 and warp 2 Linv's new row before scaling,
    // then warps 0-6 the partial values y[lr] = P[t][lr] + sum_{s < t-1} (N - l[lr][s])
    // U[s][t]; once the inverse is known, v = y + (N - l[lr][t-1]) * inv * y[t-1].
    uint32_t ppv = 0;     // pending pivot (value, local row); uniform over the block
    int pplr = 0;
    for (int t = 0;; t++) {
        uint32_t g = 0;   // U[t-1][t]
        if (t > 0) {
            const int tp = t - 1;
            const bool nxt = t < nbc && r0 + t < m;
            // the sums run over tp8 terms: Lv rows from tp on, and s_ut from tp on, are zero
            const int tp8 = (tp + 7) & ~7;
            const uint32_t *Pu = reinterpret_cast<const uint32_t *>(P);
            uint64_t lsum = 0;
            if (warp == PQ_INV_WARP) {
                const uint32_t inv = elim::mod_inv_euclid_alu(ppv, N);
                if (lane == 0) S.inv = inv;
            } else {
                if (warp == 0) {
                    // rows tp <-> pplr over the panel's columns from tp on
                    if (lane >= tp && lane < nbc) {
                        int32_t *col = P + lane * rs;
                        if (lane == tp) {
                            col[pplr] = col[tp];
                        } else if (pplr != tp) {
                            const int32_t x = col[tp];
                            col[tp] = col[pplr];
                            col[pplr] = x;
                        }
                    }
                } else if (warp == 1) {
                    if (nxt) {   // U[s][t] for s < t-1 (rows above the swapped ones); zero from t-1 on
                        const uint64_t acc = dot8(Lv + lane * 33, 1, Pu + t * rs, 1, tp8);
                        s_ut[lane] = lane < tp ? reduce_u64(acc, M) : 0u;
                    }
                } else if (warp == 2) {
                    // rows tp <-> pplr over the columns left of tp, then Linv's row tp before
                    // the inverse: sum_{s' < tp} (N - l[tp][s']) Linv[s'][lane]
                    if (lane < tp && pplr != tp) {
                        int32_t *col = P + lane * rs;
                        const int32_t x = col[tp];
                        col[tp] = col[pplr];
                        col[pplr] = x;
                    }
                    __syncwarp();
                    lsum = dot8(Pu + tp, rs, Lv + lane, 33, tp8);
                }
                if (nxt) {
                    named_sync(1, PQ_INV_WARP * 32);
                    for (int lr = tp + tid; lr < R; lr += PQ_INV_WARP * 32)
                        P[t * rs + lr] = (int32_t)reduce_u64((uint32_t)P[t * rs + lr] + dot8(Pu + lr, rs, s_ut, 1, tp8), M);
                }
            }
            __syncthreads();
            const uint32_t inv = S.inv;
            if (warp == 2)
                Lv[tp * 33 + lane] =
                    lane < tp ? elim::mulmod(reduce_u64(lsum, M), inv, M) : (lane == tp ? inv : 0u);
            if (tid == 0) {
                P[tp * rs + tp] = (int32_t)elim::mulmod(ppv, inv, M);   // U's diagonal
                S.piv_inv[tp] = inv;
            }
            if (!nxt) break;
            g = elim::mulmod((uint32_t)P[t * rs + tp], inv, M);
            if (warp == 0 && lane == 0) s_ut[tp] = g;
        }
        // column t below its pivot rows, and its largest residue (lowest row on ties)
        unsigned long long best = 0;
        for (int lr = t + tid; lr < R; lr += PQ_THREADS) {
            uint32_t v = (uint32_t)P[t * rs + lr];
            if (t > 0) v = reduce_u64((uint64_t)v + (uint64_t)(uint32_t)P[(t - 1) * rs + lr] * g, M);
            P[t * rs + lr] = v ? (int32_t)(N - v) : 0;
            const unsigned long long key = pkey32(v, lr);
            best = key > best ? key : best;
        }
        best = pq_warp_max(best);
        if (lane == 0) S.red[warp] = best;
        __syncthreads();
        // every warp takes the same decision from the eight warp maxima
        best = pq_warp_max(lane < PQ_THREADS / 32 ? S.red[lane] : 0ull);
        const uint32_t pv = (uint32_t)(best >> 32);
        // the column's values above the pivot rows are final either way.  Warp 1 copies
        // them: it alone rewrites s_ut (for column t+1, before the next barrier), so each
        // lane reads its entry before its own next write.
        if (warp == 1 && lane < t) P[t * rs + lane] = (int32_t)s_ut[lane];
        if (pv == 0) {
            zero_hit = 1;
            break;
        }
        if (c0 + t >= l_cols) {
            stop = 8;    // the reference indexes L out of bounds here
            break;
        }
        pplr = (int)(0xFFFFFFFFu - (uint32_t)(best & 0xFFFFFFFFu));
        ppv = pv;
        if (tid == 0) {
            S.piv_prow[t] = r0 + pplr;
            S.piv_val[t] = pv;
        }
        npiv = t + 1;
    }
    __syncthreads();
    return npiv;
}

// The panel's swaps composed into row moves (S.mv_*, S.nmv; absolute rows), and the swaps
// appended to row_swaps (1-based pairs from index nr).  One thread; scratch: 2 * rcap words.
__device__ __forceinline__ void pq_compose(PQShared &S, int npiv, int r0, int *scratch, int rcap,
                                          int64_t *row_swaps, int &nr) {
    int *at = scratch;                       // at[lr]: local row whose content sits at lr
    int *mk = scratch + rcap;              // visited marks
    for (int t = 0; t < npiv; t++) {
        const int pr = S.piv_prow[t] - r0;
        at[t] = t;
        at[pr] = pr;
        mk[t] = 0;
        mk[pr] = 0;
    }
    for (int t = 0; t < npiv; t++) {
        const int pr = S.piv_prow[t] - r0;
        const int x = at[t];
        at[t] = at[pr];
        at[pr] = x;
        if (pr != t) {
            row_swaps[2 * nr] = r0 + t + 1;
            row_swaps[2 * nr + 1] = r0 + pr + 1;
            nr++;
        }
    }
    int k = 0;
    for (int q2 = 0; q2 < 2 * npiv; q2++) {
        {
            const int d = (q2 & 1) ? S.piv_prow[q2 >> 1] - r0 : (q2 >> 1);
            if (mk[d]) continue;
            mk[d] = 1;
            const uint32_t sc = d < npiv ? S.piv_inv[d] : 0u;
            if (at[d] == d && sc == 0) continue;
            S.mv_dst[k] = r0 + d;
            S.mv_src[k] = r0 + at[d];
            S.mv_scale[k] = sc;
            k++;
        }
    }
    S.nmv = k;
}

// The pivot rows of trailing columns [cb, cb + cw): their current values (from row
// r0 + srcmap[t] when `moved`, the rows' old places) times Linv, into Us[t][0:cw].
// Called by the whole block; ends with a barrier.
// ALIGNED: cb, cw and ldw are multiples of 4 (16-byte loads).
template <bool ALIGNED = false>
__device__ __forceinline__ void pq_pivot_rows(const int32_t *W, int ldw, int r0, int cb, int cw, int npiv,
                                             bool moved, const int *srcmap, int32_t *Us, const uint32_t *Lv,
                                             const elim::ModP &M) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (ALIGNED) {
        // 16 bytes a load, every load of the block issued before the first store
        constexpr int PER = PQ_MAX_NB * PQ_CW / 4 / PQ_THREADS;
        const int w4 = cw >> 2;
        int4 v[PER];
#pragma unroll
        for (int i = 0; i < PER; i++) {
            const int idx = tid + i * PQ_THREADS, t = idx / (PQ_CW / 4), q = idx - t * (PQ_CW / 4);
            if (t < npiv && q < w4)
                v[i] = *reinterpret_cast<const int4 *>(W + (int64_t)(r0 + (moved ? srcmap[t] : t)) * ldw + cb + 4 * q);
        }
#pragma unroll
        for (int i = 0; i < PER; i++) {
            const int idx = tid + i * PQ_THREADS, t = idx / (PQ_CW / 4), q = idx - t * (PQ_CW / 4);
            if (t < npiv && q < w4) *reinterpret_cast<int4 *>(Us + t * PQ_CW + 4 * q) = v[i];
        }
    } else {
        for (int t = warp; t < npiv; t += PQ_THREADS / 32) {
            const int32_t *src = W + (int64_t)(r0 + (moved ? srcmap[t] : t)) * ldw + cb;
            for (int c = lane; c < cw; c += 32) Us[t * PQ_CW + c] = src[c];
        }
    }
    __syncthreads();
    {
        // U = Linv * (pivot rows) over 2 x 8 tiles: 16 row pairs x 16 column octets
        const int i0 = 2 * (tid & 15), cc0 = 8 * (tid >> 4);
        const bool act = i0 < npiv && cc0 < cw;
        uint64_t acc[2][8];
#pragma unroll
        for (int y = 0; y < 8; y++) acc[0][y] = acc[1][y] = 0;
        if (act) {
            const int smax = min(i0 + 1, npiv - 1);
            for (int s2 = 0; s2 <= smax; s2++) {
                const uint32_t l0 = Lv[i0 * 33 + s2], l1 = Lv[(i0 + 1) * 33 + s2];
                const int4 u0 = *reinterpret_cast<const int4 *>(Us + s2 * PQ_CW + cc0);
                const int4 u1 = *reinterpret_cast<const int4 *>(Us + s2 * PQ_CW + cc0 + 4);
                const uint32_t uv[8] = {(uint32_t)u0.x, (uint32_t)u0.y, (uint32_t)u0.z, (uint32_t)u0.w,
                                        (uint32_t)u1.x, (uint32_t)u1.y, (uint32_t)u1.z, (uint32_t)u1.w};
#pragma unroll
                for (int y = 0; y < 8; y++) {
                    acc[0][y] += (uint64_t)l0 * uv[y];
                    acc[1][y] += (uint64_t)l1 * uv[y];
                }
            }
        }
        __syncthreads();
        if (act) {
#pragma unroll
            for (int x = 0; x < 2; x++) {
                if (i0 + x >= npiv) break;
#pragma unroll
                for (int y = 0; y < 8; y++)
                    if (cc0 + y < cw) Us[(i0 + x) * PQ_CW + cc0 + y] = (int32_t)reduce_u64(acc[x][y], M);
            }
        }
    }
    __syncthreads();
}

__global__ void __launch_bounds__(PQ_THREADS, 2) k_pluq_batched(PQArgs a) {
    extern __shared__ __align__(16) int32_t pq_smem[];
    __shared__ PQShared S;
    __shared__ uint32_t Lv[PQ_MAX_NB * 33];   // Linv[t][s] at Lv[t * 33 + s], zero above the diagonal
    __shared__ uint32_t s_ut[PQ_MAX_NB];      // the current column's values above its pivot rows
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int rs = a.rcap + 4;                        // panel column stride (words), a multiple of 4
    int32_t *P = pq_smem;                             // P[j * rs + lr]: panel column j, local row lr
    int32_t *Us = pq_smem + (size_t)PQ_MAX_NB * rs;   // Us[t * PQ_CW + c]: pivot rows of a trailing chunk
    int *srcmap = Us + PQ_MAX_NB * PQ_CW;             // srcmap[lr]: the panel's row moves, local rows
    int *ident = pq_smem + pq_ident_offset(a.rcap);   // ident[r]: the row at position r at the start

    for (;;) {
        if (tid == 0) {
            int v = -1;
            for (;;) {
                const int k = atomicAdd(a.next, 1);
                if (k >= a.count) break;
                v = a.order[k];
                if (!a.flags || a.flags[v]) break;
                v = -1;
            }
            S.inst = v;
        }
        __syncthreads();
        const int ii = S.inst;
        if (ii < 0) break;
        // the instance's fields, in registers
        const PQInst *Ip = a.inst + ii;
        const int m = Ip->m, n = Ip->n, l_cols = Ip->l_cols, lsw = Ip->lsw;
        const elim::ModP M{Ip->M.n, Ip->M.minv};
        const uint32_t N = M.n;
        int32_t *const W = Ip->W;
        int32_t *const LW = Ip->LW;
        const int ldw = Ip->ldw, ldlw = Ip->ldlw;
        int64_t *const row_swaps = Ip->row_swaps;
        to_rowmajor(Ip->A, Ip->lda, W, ldw, m, n, M, pq_smem);
        for (int64_t idx = tid; idx < (int64_t)m * ldlw; idx += blockDim.x) LW[idx] = 0;
        for (int r = tid; r < m; r += blockDim.x) ident[r] = r;
        __syncthreads();

        int row = 0, col = 0, nr = 0, nc = 0, status = 0;
        while (row < m && col < n) {
            const int r0 = row, c0 = col;
            const int R = m - r0;
            const int nbc = min(a.nb, n - c0);
            // ---- panel load: W[r0 + lr][c0 + j] -> P[j][lr] ----
            for (int idx = tid; idx < R * nbc; idx += blockDim.x) {
                const int lr = idx / nbc, j = idx - lr * nbc;
                P[j * rs + lr] = W[(int64_t)(r0 + lr) * ldw + c0 + j];
            }
            int zero_hit = 0, stop = 0;
            const int npiv = pq_factor_panel(P, rs, R, r0, m, nbc, c0, l_cols, M, S, Lv, s_ut, zero_hit, stop);
            // ---- compose the panel's swaps into row moves (local rows; `at` and the marks in Us) ----
            if (tid == 0) {
                pq_compose(S, npiv, r0, Us, a.rcap, row_swaps, nr);
            }
            for (int lr = tid; lr < R; lr += blockDim.x) srcmap[lr] = lr;
            // ---- panel back to W: eliminated columns keep the pivot and above, zero below ----
            for (int idx = tid; idx < R * nbc; idx += blockDim.x) {
                const int lr = idx / nbc, j = idx - lr * nbc;
                W[(int64_t)(r0 + lr) * ldw + c0 + j] = (j < npiv && lr > j) ? 0 : P[j * rs + lr];
            }
            __syncthreads();
            int id_moved = 0;
            for (int k = tid; k < S.nmv; k += blockDim.x) srcmap[S.mv_dst[k] - r0] = S.mv_src[k] - r0;
            if (tid < S.nmv) id_moved = ident[S.mv_src[tid]];
            if (npiv > 0 && nc > 0) {
                // the rows the panel's swaps moved, left of the panel, with the pivot-row scaling:
                // only once a zero column has been skipped, the one way a column left of the
                // panel holds non-zeros below its pivot row.  (The trailing columns take their
                // moves inside the update through srcmap; L's columns follow `ident`.)
                int32_t *TW = a.tmp + (size_t)blockIdx.x * PQ_MAX_MOVES * a.tmp_ldw;
                gather_moves(W, ldw, 0, c0, TW, a.tmp_ldw, S);
                __syncthreads();
                scatter_moves(W, ldw, 0, c0, TW, a.tmp_ldw, S, true, M);
            }
            __syncthreads();
            if (tid < S.nmv) ident[S.mv_dst[tid]] = id_moved;
            __syncthreads();
            // ---- L: this panel's columns (pivot, then the multipliers as swapped so far), by
            // row identity inside the swap width, by position past it ----
            for (int idx = tid; idx < R * npiv; idx += blockDim.x) {
                const int lr = idx / npiv, t = idx - lr * npiv;
                if (lr >= t) {
                    const uint32_t x = (uint32_t)P[t * rs + lr];   // negated multiplier
                    const int c = c0 + t, r = c < lsw ? ident[r0 + lr] : r0 + lr;
                    LW[(int64_t)r * ldlw + c] = (int32_t)(lr == t ? S.piv_val[t] : (x ? N - x : 0u));
                }
            }
            __syncthreads();
            // L columns at or past the swap width must not see the swaps after their own step
            if (tid == 0) {
                for (int t = 0; t < npiv; t++) {
                    const int c = c0 + t;
                    if (c < lsw) continue;
                    for (int s2 = npiv - 1; s2 > t; s2--) {
                        const int r = r0 + s2, pr = S.piv_prow[s2];
                        if (pr == r) continue;
                        int32_t *x = LW + (int64_t)r * ldlw + c;
                        int32_t *y = LW + (int64_t)pr * ldlw + c;
                        const int32_t tmp = *y;
                        *y = *x;
                        *x = tmp;
                    }
                }
            }
            __syncthreads();
            // ---- trailing columns: pivot rows by the Linv product, rows below by one product ----
            // (a zero column that ended the panel is final already)
            const int ct0 = c0 + npiv + (zero_hit ? 1 : 0);
            // Chunks: the panel's own columns left over after an early end (already in their
            // final row order) alone, then chunks of PQ_CW from the panel's end on, whose
            // columns take the panel's row moves on the way in.
            const int cmove = c0 + nbc;
            for (int cb = ct0, cw = 0; npiv > 0 && cb < n; cb += cw) {
                const bool moved = cb >= cmove;
                cw = moved ? min(PQ_CW, n - cb) : min(cmove, n) - cb;
                pq_pivot_rows(W, ldw, r0, cb, cw, npiv, moved, srcmap, Us, Lv, M);
                // rows below the pivots: W += (N - l) u over 4 x 4 tiles, two per thread in
                // flight: the W values of the next tile load while the current one multiplies.
                // Tiles start at a multiple of 4 rows (16-byte panel and pivot-row reads).
                const int lr_base = npiv & ~3;
                const int trows = (R - lr_base + 3) >> 2;
                const int nitems = 2 * trows * ((cw + 7) >> 3);
                const UpdCtx uc{W, ldw, r0, cb, npiv, R, cw, lr_base, trows, P, rs, moved};
                uint64_t a0[4][4], a1[4][4];
                int it = tid;
                if (it < nitems) upd_load(a0, uc, it);
                for (; it < nitems; it += 2 * PQ_THREADS) {
                    const int it1 = it + PQ_THREADS;
                    if (it1 < nitems) upd_load(a1, uc, it1);
                    upd_mul(a0, uc, it);
                    upd_store(a0, uc, it, M);
                    if (it1 >= nitems) break;
                    const int it2 = it1 + PQ_THREADS;
                    if (it2 < nitems) upd_load(a0, uc, it2);
                    upd_mul(a1, uc, it1);
                    upd_store(a1, uc, it1, M);
                }
                __syncthreads();
                // U to the pivot rows, after the update has read their old contents
                for (int t = warp; t < npiv; t += PQ_THREADS / 32) {
                    int32_t *dst = W + (int64_t)(r0 + t) * ldw + cb;
                    for (int c = lane; c < cw; c += 32) dst[c] = Us[t * PQ_CW + c];
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
                        int32_t *w = W + (int64_t)r * ldw;
                        const int32_t x = w[col];
                        w[col] = w[last];
                        w[last] = x;
                    }
                }
                if (tid == 0) {
                    Ip->col_swaps[2 * nc] = col + 1;
                    Ip->col_swaps[2 * nc + 1] = last + 1;
                }
                nc++;
                col++;
            }
            __syncthreads();
        }
        __syncthreads();
        to_colmajor(W, ldw, n, Ip->U, Ip->ldu, m, n, pq_smem);
        to_colmajor(LW, ldlw, Ip->lwc, Ip->L, Ip->ldl, m, l_cols, pq_smem, ident, lsw);
        if (tid == 0) {
            Ip->info[0] = nr;
            Ip->info[1] = nc;
            Ip->info[2] = row;
            Ip->info[3] = status;
        }
        __syncthreads();
    }
}

}  // namespace batched
