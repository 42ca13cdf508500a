// batched_steps.cuh -- the batched PLUQ in panel steps, its trailing updates on the
// tensor cores.  Included by k_batched.cu after the grouped GEMM.
//
// A PLUQ instance takes this route when it is square with n a multiple of 32 (n >= 64),
// its prime is odd and L is at least n columns wide.  Step s factors panel s (columns
// [32 s, 32 s + 32)) of every instance still running, one launch for all:
//   k_pq_panel   a CTA per instance: the left-looking panel of k_pluq_batched
//                (pq_factor_panel), the panel's swaps composed into row moves, the
//                panel and L written back, then the pivot rows of the trailing columns
//                (Linv times the pivot rows, from their old places) into a side buffer
//                U12, and both factors of the trailing update as fp16 digit planes:
//                A = the negated multipliers (rows below the pivots x 32),
//                B = U12 transposed (trailing columns x 32), 7-bit balanced digits,
//                rows of 32 fp16 (64 bytes; TMA and the MMA use 64-byte swizzling).
//   k_gemm_trail a persistent tcgen05 GEMM over the 128 x 64 tiles of every instance's
//                trailing block: W[r][c] = W[src(r)][c] + sum_t A[r][t] B[c][t] mod p,
//                src(r) the row whose old contents row r receives (the panel's moves).
//                The pivot rows keep their old contents through the GEMM (they are the
//                moved rows' sources); the next step's panel kernel copies U12 into them.
// The result is the same factorization as k_pluq_batched, operation for operation: the
// same pivots, the same row moves, each entry reduced mod p once per panel.  A panel that
// finds fewer than 32 pivots (a zero column, a rank drop) flags its instance; the instance
// is then factored from its input again by k_pluq_batched, which covers every case.
#pragma once

#include "batched_pluq.cuh"
#include "gemm_limb.cuh"

namespace batched {

constexpr int ST_NB = 32;                   // panel width of the step route
constexpr int ST_BM = 128, ST_BN = 64;      // trailing GEMM tile (limb::BM x limb::BN)
constexpr int ST_KPAD = 32;                 // K of the digit planes: 64-byte rows
constexpr int ST_MAX_GROUPS = 2;            // step chains run side by side (graph branches)
constexpr int ST_GROUP_MIN = 64;            // step instances needed before a batch is split into groups
constexpr int ST_A_TILE = ST_BM * ST_KPAD * 2, ST_B_TILE = ST_BN * ST_KPAD * 2;   // one digit's tile
constexpr int ST_STAGES = 3;
constexpr int ST_STAGE_BYTES = 4 * (ST_A_TILE + ST_B_TILE);
// after the stages: two slots of 64 bytes per epilogue thread for the next tile's old values
constexpr int ST_PF_BYTES = 2 * 512 * 64;
constexpr int ST_SMEM_BYTES = ST_STAGES * ST_STAGE_BYTES + ST_PF_BYTES + 1024;
static_assert(ST_SMEM_BYTES <= 227 * 1024, "trail GEMM shared memory");
static_assert(ST_BM == limb::BM && ST_BN == limb::BN, "the step GEMM's epilogue uses the limb tile shape");

// Dynamic shared memory of k_pq_panel for panels of up to rcap rows: the panel (32 columns
// of rcap + 4 words), whose space the trailing columns' pivot rows (32 x PQ_CW words) reuse
// once the panel has been written out, then the swap composition's scratch (2 rcap words)
// and the panel's row sources (rcap words).
__host__ __device__ constexpr size_t st_panel_words(int rcap) {
    return (size_t)PQ_MAX_NB * (rcap + 4) > (size_t)PQ_MAX_NB * PQ_CW ? (size_t)PQ_MAX_NB * (rcap + 4)
                                                                       : (size_t)PQ_MAX_NB * PQ_CW;
}
__host__ __device__ constexpr size_t st_smem_words(int rcap) { return st_panel_words(rcap) + 3 * (size_t)rcap; }

struct StepInst {
    int pq;                      // index in the PLUQ instance array
    int n;                       // m = n, a multiple of 32
    int L;                       // 7-bit digits per residue
    int Mpad, Npad;              // rows per digit plane of A / B (multiples of 128 / 64, >= n - 32)
    int *srcmap;                 // [n]: the current panel's row sources (local rows)
    int *ident;                  // [n]: row identities (L is stored by identity)
    int32_t *U12;                // [32][n]: the last panel's pivot rows of its trailing columns
    int *nr;                     // running count of row swaps
    __half *Ad, *Bd;             // L planes of Mpad x 64 / Npad x 64 fp16
    // the trailing GEMM's epilogue: the grouped GEMM's fast path (odd p, one exact chunk)
    uint32_t ninv;               // -p^-1 mod 2^32
    int32_t Wm[limb::MAX_SHIFTS];  // 2^(7 s) 2^32 mod p
    int64_t fbias;
};

struct StepArgs {
    const PQInst *inst;
    const StepInst *steps;
    const int *order;            // step instances, largest first
    const int *live;             // per step: how many of `order` still factor (a prefix)
    int *next;                   // per step: scheduling counters (zero before the run)
    int *flags;                  // per PLUQ instance: nonzero = k_pluq_batched factors it
    const CUtensorMap *tmaps;    // per step instance: A planes, B planes
    int rcap;                    // rows of the shared panel (>= every n), multiple of 4
};

// the whole block, after a barrier: L 7-bit balanced digits of the 8 residues v[0..7]
// (centred mod p) packed as 8 fp16 per plane, stored 16 bytes per plane at dst + l * plane
__device__ __forceinline__ void put_digits8(const uint32_t (&v)[8], uint32_t N, int L, __half *dst, size_t plane) {
    __half d[8][4];
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const int32_t c = 2 * v[i] > N ? (int32_t)v[i] - (int32_t)N : (int32_t)v[i];
        limb::digits<4>(c, d[i], 7);
    }
#pragma unroll
    for (int l = 0; l < 4; l++) {
        if (l >= L) break;
        __half2 h[4];
#pragma unroll
        for (int i = 0; i < 4; i++) h[i] = __halves2half2(d[2 * i][l], d[2 * i + 1][l]);
        *reinterpret_cast<int4 *>(dst + l * plane) = *reinterpret_cast<const int4 *>(h);
    }
}

// ---------------------------------------------------------------------------
// prologue: the working copies, row identities and counters of every step instance
// ---------------------------------------------------------------------------
// the first `count` instances of a.order (a group's)
__global__ void __launch_bounds__(PQ_THREADS) k_pq_prologue(StepArgs a, int count) {
    extern __shared__ __align__(16) int32_t pq_smem[];
    for (int q = blockIdx.x; q < count; q += gridDim.x) {
        const StepInst J = a.steps[a.order[q]];
        const PQInst &I = a.inst[J.pq];
        const elim::ModP M{I.M.n, I.M.minv};
        to_rowmajor(I.A, I.lda, I.W, I.ldw, J.n, J.n, M, pq_smem);
        // (L's working copy is not cleared: the finish reads only the entries the steps write)
        for (int r = threadIdx.x; r < J.n; r += blockDim.x) J.ident[r] = r;
        if (threadIdx.x == 0) {
            *J.nr = 0;
            a.flags[J.pq] = 0;
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// one panel step of every running instance
// ---------------------------------------------------------------------------
// MIN_BLOCKS: CTAs per SM the registers are sized for (the plan takes 3 where a step's
// panel height lets three CTAs' shared memory fit)
template <int MIN_BLOCKS>
__global__ void __launch_bounds__(PQ_THREADS, MIN_BLOCKS) k_pq_panel(StepArgs a, int s) {
    extern __shared__ __align__(16) int32_t pq_smem[];
    __shared__ PQShared S;
    __shared__ uint32_t Lv[PQ_MAX_NB * 33];
    __shared__ uint32_t s_ut[PQ_MAX_NB];
    const int tid = threadIdx.x;
    const int rs = a.rcap + 4;
    int32_t *P = pq_smem;
    int32_t *Us = pq_smem;                                   // the panel's space, after the panel
    int *scratch = pq_smem + st_panel_words(a.rcap);         // the swap composition's
    int *srcmap = scratch + 2 * a.rcap;
    const int r0 = ST_NB * s, c0 = r0;

    for (;;) {
        if (tid == 0) {
            const int k = atomicAdd(a.next + s, 1);
            S.inst = k < a.live[s] ? a.order[k] : -1;
        }
        __syncthreads();
        const int jj = S.inst;
        if (jj < 0) break;
        const StepInst &J = a.steps[jj];
        const PQInst &I = a.inst[J.pq];
        const int n = J.n, R = n - r0, T = n - c0 - ST_NB;
        const elim::ModP M{I.M.n, I.M.minv};
        const uint32_t N = M.n;
        int32_t *const W = I.W;
        const int ldw = I.ldw;
        if (a.flags[J.pq] == 0) {
            // the previous panel's pivot rows, columns [c0, n): U12 -> W (their old contents
            // were the previous trailing update's row sources)
            if (s > 0) {
                const int w4 = (n - c0) >> 2;
                for (int idx = tid; idx < ST_NB * w4; idx += blockDim.x) {
                    const int t = idx / w4, q = idx - t * w4;
                    *reinterpret_cast<int4 *>(W + (int64_t)(r0 - ST_NB + t) * ldw + c0 + 4 * q) =
                        *reinterpret_cast<const int4 *>(J.U12 + (int64_t)t * n + 4 * q);
                }
            }
            // the panel, W[r0 + lr][c0 + j] -> P[j][lr]: 16-byte loads, four in flight a thread
            for (int base = 0; base < R * 8; base += 4 * PQ_THREADS) {
                int4 v[4];
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    const int idx = base + tid + i * PQ_THREADS, lr = idx >> 3, q = idx & 7;
                    if (idx < R * 8) v[i] = *reinterpret_cast<const int4 *>(W + (int64_t)(r0 + lr) * ldw + c0 + 4 * q);
                }
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    const int idx = base + tid + i * PQ_THREADS, lr = idx >> 3, q = idx & 7;
                    if (idx < R * 8) {
                        P[(4 * q) * rs + lr] = v[i].x;
                        P[(4 * q + 1) * rs + lr] = v[i].y;
                        P[(4 * q + 2) * rs + lr] = v[i].z;
                        P[(4 * q + 3) * rs + lr] = v[i].w;
                    }
                }
            }
            int zero_hit = 0, stop = 0;
            const int npiv = pq_factor_panel(P, rs, R, r0, n, ST_NB, c0, I.l_cols, M, S, Lv, s_ut, zero_hit, stop);
            if (npiv < ST_NB) {
                // a zero column or a rank drop: k_pluq_batched factors this instance from its input
                if (tid == 0) a.flags[J.pq] = 1;
            } else {
                if (tid == 0) {
                    int nr = *J.nr;
                    pq_compose(S, npiv, r0, scratch, a.rcap, I.row_swaps, nr);
                    *J.nr = nr;
                }
                // the panel back to W, a row a thread in 16-byte stores: U on and above the
                // diagonal, zero below
                for (int lr = tid; lr < R; lr += blockDim.x) {
                    srcmap[lr] = lr;
                    int4 *wrow = reinterpret_cast<int4 *>(W + (int64_t)(r0 + lr) * ldw + c0);
#pragma unroll
                    for (int q = 0; q < ST_NB / 4; q++) {
                        int32_t x[4];
#pragma unroll
                        for (int i = 0; i < 4; i++) x[i] = lr > 4 * q + i ? 0 : P[(4 * q + i) * rs + lr];
                        wrow[q] = make_int4(x[0], x[1], x[2], x[3]);
                    }
                }
                __syncthreads();
                int id_moved = 0;
                for (int k = tid; k < S.nmv; k += blockDim.x) srcmap[S.mv_dst[k] - r0] = S.mv_src[k] - r0;
                if (tid < S.nmv) id_moved = J.ident[S.mv_src[tid]];
                __syncthreads();
                if (tid < S.nmv) J.ident[S.mv_dst[tid]] = id_moved;
                for (int lr = tid; lr < R; lr += blockDim.x) J.srcmap[lr] = srcmap[lr];
                __syncthreads();
                // L: the pivots and the multipliers, by row identity (L's swap width covers n), a
                // row a thread in 16-byte stores (zero above the diagonal, as L is there)
                for (int lr = tid; lr < R; lr += blockDim.x) {
                    int4 *lrow = reinterpret_cast<int4 *>(I.LW + (int64_t)J.ident[r0 + lr] * I.ldlw + c0);
#pragma unroll
                    for (int q = 0; q < ST_NB / 4; q++) {
                        int32_t x[4];
#pragma unroll
                        for (int i = 0; i < 4; i++) {
                            const int t = 4 * q + i;
                            const uint32_t v = (uint32_t)P[t * rs + lr];
                            x[i] = lr < t ? 0 : (int32_t)(lr == t ? S.piv_val[t] : (v ? N - v : 0u));
                        }
                        lrow[q] = make_int4(x[0], x[1], x[2], x[3]);
                    }
                }
                // A planes: the negated multipliers of rows [32, R), 8 per thread and store
                {
                    const size_t plane = (size_t)J.Mpad * ST_KPAD;
                    for (int idx = tid; idx < (R - ST_NB) * 4; idx += blockDim.x) {
                        const int lr = ST_NB + (idx >> 2), t0 = 8 * (idx & 3);
                        uint32_t v[8];
#pragma unroll
                        for (int i = 0; i < 8; i++) v[i] = (uint32_t)P[(t0 + i) * rs + lr];
                        put_digits8(v, N, J.L, J.Ad + (size_t)(lr - ST_NB) * ST_KPAD + t0, plane);
                    }
                }
                __syncthreads();   // the panel is written out: its space takes the pivot rows
                // the pivot rows of the trailing columns, PQ_CW at a time: U12 and the B planes
                for (int cb = c0 + ST_NB; cb < n; cb += PQ_CW) {
                    const int cw = min(PQ_CW, n - cb);
                    const int cl = cb - c0 - ST_NB;   // column within the trailing block
                    pq_pivot_rows<true>(W, ldw, r0, cb, cw, ST_NB, true, srcmap, Us, Lv, M);
                    const int w4 = cw >> 2;
                    for (int idx = tid; idx < ST_NB * w4; idx += blockDim.x) {
                        const int t = idx / w4, q = idx - t * w4;
                        *reinterpret_cast<int4 *>(J.U12 + (int64_t)t * n + cl + 4 * q) =
                            *reinterpret_cast<const int4 *>(Us + t * PQ_CW + 4 * q);
                    }
                    const size_t plane = (size_t)J.Npad * ST_KPAD;
                    for (int idx = tid; idx < cw * 4; idx += blockDim.x) {
                        const int c = idx >> 2, t0 = 8 * (idx & 3);
                        uint32_t v[8];
#pragma unroll
                        for (int i = 0; i < 8; i++) v[i] = (uint32_t)Us[(t0 + i) * PQ_CW + c];
                        put_digits8(v, N, J.L, J.Bd + (size_t)(cl + c) * ST_KPAD + t0, plane);
                    }
                    __syncthreads();   // Us is refilled by the next chunk
                }
                (void)T;
            }
        }
        __syncthreads();   // every thread has read S.inst before the next pick
    }
}

// ---------------------------------------------------------------------------
// the trailing update of every running instance, tcgen05, in place
// ---------------------------------------------------------------------------
// One tile: its L x L digit products over K = 32 (two K = 16 steps), drained shift by
// shift and combined by the grouped GEMM's fast epilogue, plus the old value of the
// output row's source row, reduced and stored over the row.  A CTA takes a contiguous
// range of the step's tiles (ordered by instance, tile row, tile column), so each role
// keeps the instance's fields, and the epilogue its row pointers, across tiles instead of
// starting every tile with a chain of dependent loads.
__global__ void __launch_bounds__(G_THREADS, 1)
    k_gemm_trail(StepArgs a, int s, const WorkItem *__restrict__ items, int nitems, int *err) {
    extern __shared__ uint8_t dsmem_raw[];
    __shared__ uint64_t full_bar[ST_STAGES];
    __shared__ uint64_t empty_bar[ST_STAGES];
    __shared__ uint64_t acc_full_bar, acc_empty_bar, drain_bar;
    __shared__ uint32_t tmem_base_s;
    __shared__ int abort_sh;
    __shared__ int32_t wm_s[G_EPI_WARPS][8];   // per epilogue warp: its current instance's shift weights
    volatile int &abort_s = abort_sh;

    uint8_t *smem = (uint8_t *)(((uintptr_t)dsmem_raw + 1023) & ~(uintptr_t)1023);
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const int r0 = ST_NB * s;
    const int t_begin = (int)((int64_t)nitems * blockIdx.x / gridDim.x);
    const int t_end = (int)((int64_t)nitems * (blockIdx.x + 1) / gridDim.x);

    if (threadIdx.x == 0) {
        for (int q = 0; q < ST_STAGES; q++) {
            gffm_dev::mbar_init(&full_bar[q], 1);
            gffm_dev::mbar_init(&empty_bar[q], 1);
        }
        gffm_dev::mbar_init(&acc_full_bar, 1);
        gffm_dev::mbar_init(&acc_empty_bar, G_EPI_WARPS);
        gffm_dev::mbar_init(&drain_bar, 1);
        abort_s = 0;
        gffm_dev::fence_mbar_init();
    }
    if (warp == 1) gffm_dev::tmem_alloc(&tmem_base_s, G_TMEM_COLS);
    gffm_dev::tc_fence_before();
    __syncthreads();
    gffm_dev::tc_fence_after();
    const uint32_t tmem = tmem_base_s;

    if (warp == 0) {
        // ---------------- TMA producer ----------------
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0;
            uint32_t issued_parity_mask = 0, issued_mask = 0;
            int last = -1, L = 0, Mpad = 0, Npad = 0;
            bool skip = false;
            const CUtensorMap *tmA = nullptr, *tmB = nullptr;
            for (int t = t_begin; t < t_end && !abort_s; t++) {
                const WorkItem it = items[t];
                if (it.inst != last) {
                    last = it.inst;
                    const StepInst &J = a.steps[it.inst];
                    skip = a.flags[J.pq] != 0;
                    L = J.L;
                    Mpad = J.Mpad;
                    Npad = J.Npad;
                    tmA = a.tmaps + 2 * it.inst;
                    tmB = tmA + 1;
                    if (!skip) {
                        tmap_acquire(tmA);
                        tmap_acquire(tmB);
                    }
                }
                if (skip) continue;
                if (!gffm_dev::mbar_wait(&empty_bar[stage], phase ^ 1)) {
                    atomicOr(err, 1);
                    abort_s = 1;
                    break;
                }
                uint8_t *sa = smem + stage * ST_STAGE_BYTES;
                uint8_t *sb = sa + 4 * ST_A_TILE;
                gffm_dev::mbar_arrive_expect_tx(&full_bar[stage], (uint32_t)L * (ST_A_TILE + ST_B_TILE));
                for (int l = 0; l < L; l++)
                    gffm_dev::tma_load_2d(sa + l * ST_A_TILE, tmA, &full_bar[stage], 0, l * Mpad + it.tm * ST_BM);
                for (int l = 0; l < L; l++)
                    gffm_dev::tma_load_2d(sb + l * ST_B_TILE, tmB, &full_bar[stage], 0, l * Npad + it.tn * ST_BN);
                issued_mask |= 1u << stage;
                issued_parity_mask = (issued_parity_mask & ~(1u << stage)) | (phase << stage);
                if (++stage == ST_STAGES) {
                    stage = 0;
                    phase ^= 1;
                }
            }
            if (abort_s) {
                for (int q = 0; q < ST_STAGES; q++)
                    if (issued_mask & (1u << q)) gffm_dev::mbar_wait(&full_bar[q], (issued_parity_mask >> q) & 1);
            }
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer ----------------
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0, acc_phase = 0;
            bool issued_any = false;
            int last = -1, L = 0;
            bool skip = false;
            uint32_t idesc_full = 0, idesc_lo = 0;
            const uint32_t idesc_one = gffm_dev::idesc_f16_f32(BM, BN);
            for (int t = t_begin; t < t_end && !abort_s; t++) {
                const WorkItem it = items[t];
                if (it.inst != last) {
                    last = it.inst;
                    const StepInst &J = a.steps[it.inst];
                    skip = a.flags[J.pq] != 0;
                    L = J.L;
                    idesc_full = gffm_dev::idesc_f16_f32(BM, BN * L);
                    idesc_lo = gffm_dev::idesc_f16_f32(BM, BN * (L > 1 ? L - 1 : 1));
                }
                if (skip) continue;
                if (!gffm_dev::mbar_wait(&acc_empty_bar, acc_phase ^ 1)) {
                    atomicOr(err, 2);
                    abort_s = 1;
                    break;
                }
                gffm_dev::tc_fence_after();
                if (!gffm_dev::mbar_wait(&full_bar[stage], phase)) {
                    atomicOr(err, 4);
                    abort_s = 1;
                    break;
                }
                gffm_dev::tc_fence_after();
                const uint32_t sa = gffm_dev::smem_u32(smem + stage * ST_STAGE_BYTES);
                const uint32_t sb = sa + 4 * ST_A_TILE;
                // K = 32: two K = 16 steps along the 64-byte rows
#pragma unroll
                for (int kk = 0; kk < ST_NB / 16; kk++) {
                    const uint64_t bdesc = gffm_dev::umma_desc_sw64(sb + kk * 32);
                    if (kk == 0) {
                        gffm_dev::mma_f16(tmem, gffm_dev::umma_desc_sw64(sa), bdesc, idesc_full, 0);
                        for (int i = 1; i < L; i++) {
                            const uint64_t adesc = gffm_dev::umma_desc_sw64(sa + i * ST_A_TILE);
                            gffm_dev::mma_f16(tmem + 64 * i, adesc, bdesc, idesc_lo, 1);
                            gffm_dev::mma_f16(tmem + 64 * (i + L - 1), adesc,
                                              gffm_dev::umma_desc_sw64(sb + (L - 1) * ST_B_TILE), idesc_one, 0);
                        }
                    } else {
                        for (int i = 0; i < L; i++)
                            gffm_dev::mma_f16(tmem + 64 * i, gffm_dev::umma_desc_sw64(sa + i * ST_A_TILE + kk * 32),
                                              bdesc, idesc_full, 1);
                    }
                }
                issued_any = true;
                gffm_dev::mma_commit(&empty_bar[stage]);
                if (++stage == ST_STAGES) {
                    stage = 0;
                    phase ^= 1;
                }
                gffm_dev::mma_commit(&acc_full_bar);
                acc_phase ^= 1;
            }
            if (abort_s && issued_any) {
                gffm_dev::mma_commit(&drain_bar);
                gffm_dev::mbar_wait(&drain_bar, 0);
            }
        }
    } else {
        // ---------------- epilogue ----------------
        // A thread owns one row and 16 columns of the tile.  The row's old values are loaded
        // before the accumulator is waited for (no tile of this launch writes a row another
        // tile reads: sources are pivot rows or the row itself): a tile's by cp.async into
        // one of two shared slots while the previous tile drains, when both belong to the
        // same instance, else directly.  Every iteration commits one (possibly empty)
        // cp.async group, so waiting for all but the newest finds the current tile's.
        const int quad = warp & 3;
        const int part = (warp - 2) >> 2;   // which 16 of the tile's 64 columns
        const uint32_t tq = tmem + ((uint32_t)(quad * 32) << 16) + 16 * part;
        uint32_t acc_phase = 0;
        int last = -1, last_tm = -1, n = 0, L = 0, ldw = 0;
        bool skip = false, row_live = false;
        uint32_t ninv = 0, n32 = 0;
        int64_t fbias = 0;
        int32_t *Wm = wm_s[warp - 2];
        int32_t *W = nullptr;
        const int *srcmap = nullptr;
        const int32_t *src_row = nullptr;
        int32_t *dst_row = nullptr;
        uint8_t *pf_base = smem + ST_STAGES * ST_STAGE_BYTES + (threadIdx.x - 64) * 64;
        bool have = false;   // this tile's old values were prefetched into slot t & 1
        WorkItem nx = t_begin < t_end ? items[t_begin] : WorkItem{0, 0, 0, 0};
        for (int t = t_begin; t < t_end; t++) {
            const WorkItem it = nx;
            if (t + 1 < t_end) nx = items[t + 1];
            if (it.inst != last) {
                last = it.inst;
                last_tm = -1;
                const StepInst &J = a.steps[it.inst];
                const PQInst &I = a.inst[J.pq];
                skip = a.flags[J.pq] != 0;
                n = J.n;
                L = J.L;
                ninv = J.ninv;
                fbias = J.fbias;
                __syncwarp();
                if (lane < limb::MAX_SHIFTS) Wm[lane] = J.Wm[lane];
                __syncwarp();
                W = I.W;
                ldw = I.ldw;
                n32 = I.M.n;
                srcmap = J.srcmap;
            }
            if (!skip && it.tm != last_tm) {
                last_tm = it.tm;
                const int rt = it.tm * ST_BM + quad * 32 + lane;   // row within the trailing block
                row_live = rt < n - r0 - ST_NB;
                if (row_live) {
                    src_row = W + (int64_t)(r0 + srcmap[ST_NB + rt]) * ldw;
                    dst_row = W + (int64_t)(r0 + ST_NB + rt) * ldw;
                }
            }
            // the next tile's old values, if it belongs to this instance and is live
            const bool cur = have;
            have = false;
            if (!skip && t + 1 < t_end && nx.inst == it.inst) {
                const int rtn = nx.tm * ST_BM + quad * 32 + lane;
                const int coln = r0 + ST_NB + nx.tn * ST_BN + part * 16;
                if (rtn < n - r0 - ST_NB && coln < n) {
                    const int32_t *srcn = nx.tm == it.tm ? src_row : W + (int64_t)(r0 + srcmap[ST_NB + rtn]) * ldw;
                    uint8_t *slot = pf_base + ((t + 1) & 1) * (512 * 64);
#pragma unroll
                    for (int q = 0; q < 4; q++) gffm_dev::cp_async16(slot + 16 * q, srcn + coln + 4 * q);
                    have = true;
                }
            }
            gffm_dev::cp_async_commit();
            if (skip) continue;
            const int col = r0 + ST_NB + it.tn * ST_BN + part * 16;   // n - col is 0 or >= 16
            const bool live = row_live && col < n;
            int4 c4[4];
            if (live) {
                if (cur) {
                    gffm_dev::cp_async_wait<1>();
                    const int4 *slot = reinterpret_cast<const int4 *>(pf_base + (t & 1) * (512 * 64));
#pragma unroll
                    for (int q = 0; q < 4; q++) c4[q] = slot[q];
                } else {
#pragma unroll
                    for (int q = 0; q < 4; q++) c4[q] = *reinterpret_cast<const int4 *>(src_row + col + 4 * q);
                }
            }
            const int nshift = 2 * L - 1;
            int64_t acc[16];
#pragma unroll
            for (int j = 0; j < 16; j++) acc[j] = fbias;
            if (!gffm_dev::mbar_wait(&acc_full_bar, acc_phase)) {
                atomicOr(err, 8);
                abort_s = 1;
                break;
            }
            gffm_dev::tc_fence_after();
            // 7-bit digits: the shifts in pairs, one wide multiply-add each (limb::fast_pair),
            // 8 columns of both shifts at a time
#pragma unroll 1
            for (int q = 0; q + 1 < nshift; q += 2) {
                const int w = Wm[q];
#pragma unroll 1
                for (int h = 0; h < 16; h += 8) {
                    uint32_t v[8], u[8];
                    gffm_dev::tmem_ld_32x32b_x8(tq + 64 * q + h, v);
                    gffm_dev::tmem_ld_32x32b_x8(tq + 64 * (q + 1) + h, u);
                    gffm_dev::tmem_ld_wait();
                    if (h == 0) {
#pragma unroll
                        for (int j = 0; j < 8; j++) acc[j] += (int64_t)fast_pair(v[j], u[j]) * w;
                    } else {
#pragma unroll
                        for (int j = 0; j < 8; j++) acc[8 + j] += (int64_t)fast_pair(v[j], u[j]) * w;
                    }
                }
            }
            {
                uint32_t v[16];
                gffm_dev::tmem_ld_32x32b_x16(tq + 64 * (nshift - 1), v);
                gffm_dev::tmem_ld_wait();
                const int w = Wm[nshift - 1];
#pragma unroll
                for (int j = 0; j < 16; j++) acc[j] += (int64_t)(int32_t)fast_bits(v[j]) * w;
            }
            gffm_dev::tc_fence_before();
            __syncwarp();
            if (lane == 0) gffm_dev::mbar_arrive(&acc_empty_bar);
            acc_phase ^= 1;
            if (live) {
                int32_t *dst = dst_row + col;
                // x in (0, 2^32 p): (x + m p) / 2^32 < 2p is x 2^-32 mod p; then + the old value
                auto fin = [&](int64_t a64, int32_t old) -> int32_t {
                    const uint64_t x = (uint64_t)a64;
                    const uint32_t mq = (uint32_t)x * ninv;
                    uint32_t r = (uint32_t)((x + (uint64_t)mq * n32) >> 32);
                    r = r >= n32 ? r - n32 : r;
                    r += (uint32_t)old;
                    return (int32_t)(r >= n32 ? r - n32 : r);
                };
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int4 o = make_int4(fin(acc[4 * q], c4[q].x), fin(acc[4 * q + 1], c4[q].y),
                                             fin(acc[4 * q + 2], c4[q].z), fin(acc[4 * q + 3], c4[q].w));
                    *reinterpret_cast<int4 *>(dst + 4 * q) = o;
                }
            }
        }
        gffm_dev::cp_async_wait<0>();   // no copy into shared memory outlives the CTA
    }

    gffm_dev::tc_fence_before();
    __syncthreads();
    gffm_dev::tc_fence_after();
    if (warp == 1) gffm_dev::tmem_dealloc(tmem, G_TMEM_COLS);
}

// ---------------------------------------------------------------------------
// the outputs of every step instance that was not handed back
// ---------------------------------------------------------------------------
// dynamic shared memory: the conversions' 8 x 32 x 33 words, then the row identities
// the first `count` instances of a.order (a group's)
__global__ void __launch_bounds__(PQ_THREADS) k_pq_finish(StepArgs a, int count) {
    extern __shared__ __align__(16) int32_t pq_smem[];
    int *id_s = pq_smem + 8 * 32 * 33;
    for (int q = blockIdx.x; q < count; q += gridDim.x) {
        const StepInst J = a.steps[a.order[q]];
        if (a.flags[J.pq]) continue;   // uniform over the block; k_pluq_batched writes its outputs
        const PQInst &I = a.inst[J.pq];
        for (int r = threadIdx.x; r < J.n; r += blockDim.x) id_s[r] = J.ident[r];
        to_colmajor(I.W, I.ldw, J.n, I.U, I.ldu, J.n, J.n, pq_smem);   // its barriers order the id_s stores
        // L by row identity; a column's rows above its panel block were never written: zero
        to_colmajor(I.LW, I.ldlw, I.lwc, I.L, I.ldl, J.n, I.l_cols, pq_smem, id_s, I.lsw, ST_NB);
        if (threadIdx.x == 0) {
            I.info[0] = *J.nr;
            I.info[1] = 0;
            I.info[2] = J.n;
            I.info[3] = 0;
        }
        __syncthreads();
    }
}

}  // namespace batched
