// gemm_limb.cuh -- exact modular GEMM on the tcgen05 tensor cores.
//
// Representation.  A residue x in [0, N), N < 2^26, is centred to
// c in (-N/2, N/2] and written in L balanced base-2^7 digits
//     c = sum_{i<L} d_i 2^(7i),   d_i in [-64, 63],
// each digit held exactly in fp16.  For A (m x k) and B (k x n):
//     A*B = sum_s 2^(7s) C_s,   C_s = sum_{i+j=s} A_i B_j,   s = 0 .. 2L-2.
// A product may instead use base-2^8 digits in [-128, 127] (fewer digits for
// some moduli; |d_i d_j| <= 2^14, so chunks of 1024/L values of k, and the
// weights below become 2^(8s) mod N): the kernels below do not depend on the
// digit width, only the split and the host-side chunk and weights do.
//
// Tensor-core mapping.  The L digit tiles of B for one 64-column output tile
// are stacked along N into one operand B' = [B_0; B_1; ...; B_{L-1}] (64L
// rows).  One tcgen05.mma of A_i (128 x 16) with B' (64L x 16) produces
// [A_i B_0 | A_i B_1 | ... ] and is issued with its accumulator at TMEM
// column 64*i, so the block A_i B_j lands in columns 64*(i+j): the shift-s
// accumulator.  The 2L-1 shift accumulators (448 columns for L = 4) live side
// by side in TMEM and every mma of the main loop has N = 64L (256 for L = 4).
//
// Exactness.  |d_i d_j| <= 2^12 and a shift accumulator sums at most L digit
// products per k, so after Kc <= 4096/L values of k every partial sum is an
// integer of magnitude <= 2^24 and the fp32 accumulation is exact.  The K loop
// is therefore cut into chunks of Kc; after each chunk the epilogue warps
// drain the accumulators, convert them to int32 and add
// sum_s C_s * (2^(7s) mod N) into int64 registers; the final value is reduced
// mod N with Barrett's method and stored.
//
// Tile schedule.  A CTA's tiles are blockIdx.x, + gridDim.x, ... or, with a
// tile counter, whatever a global atomic counter hands out: then several
// launches of the same product share its tiles, and CTAs launched later (on
// SMs that became free) take over the remaining ones.  The producer draws the
// tiles and passes them to the mma issuer and the epilogue through a small ring
// in shared memory.
//
// Warp roles (576 threads): warp 0 issues TMA loads, warp 1 allocates TMEM
// and one lane issues the mma's, warps 2..17 are the epilogue (four per 32-lane
// TMEM quadrant, each owning 16 of the 64 output columns).  With one
// accumulator set the mma's of a tile wait for the drain of the previous one,
// and for short K (the elimination's K = 128 updates) the epilogue's per-tile
// chain paces the mma's; twice the epilogue warps of 8 x 32 columns halve
// both.  Every
// wait is bounded; on timeout a kernel records the failure in the library's
// error word and returns without storing.
#pragma once

#include "gffm_common.cuh"
#include "limb_host.h"

namespace limb {

constexpr int BM = 128;            // output rows per tile (tcgen05 M)
constexpr int BN = 64;             // output columns per tile
constexpr int BK = 64;             // k per pipeline stage (one 128-byte swizzle row of fp16)
constexpr int A_TILE = BM * BK * 2;
constexpr int B_TILE = BN * BK * 2;
// epilogue warps and threads per CTA for an epilogue kind (the same for all)
__host__ __device__ constexpr int epi_warps(int) { return 16; }
__host__ __device__ constexpr int gemm_threads(int epi) { return 64 + 32 * epi_warps(epi); }
constexpr int MAX_SHIFTS = 7;
constexpr int TILE_RING = 4;       // tiles the producer hands ahead to the mma issuer and the epilogue
constexpr int TILE_GROUP = 16;     // output-tile rows per raster group (L2 reuse)

// Tile width BNV: 64 (one accumulator set) or 32 (two accumulator sets in TMEM,
// half the epilogue warps per set: the drain of one tile overlaps the mma's of
// the next -- for short K, where a tile is one or two exact chunks and the
// drain is as long as the products).
template <int L, int BNV = 64>
struct Cfg {
    static constexpr int B_T = BNV * BK * 2;
    static constexpr int STAGE_BYTES = L * (A_TILE + B_T);
    static constexpr int STAGES = BNV == 64 ? ((L == 4) ? 2 : (L == 3 ? 3 : (L == 2 ? 4 : 8)))
                                            : ((L == 4) ? 2 : (L == 3 ? 3 : (L == 2 ? 5 : 8)));
    static constexpr int NSHIFT = 2 * L - 1;
    static constexpr int ACC_BUFS = BNV == 32 ? 2 : 1;
    static constexpr int BUF_COLS = BNV == 32 ? 256 : 0;   // column offset of the second accumulator set
    static constexpr int TMEM_COLS = BNV == 32 ? 512
                                               : ((64 * NSHIFT <= 64) ? 64 : (64 * NSHIFT <= 128 ? 128 : (64 * NSHIFT <= 256 ? 256 : 512)));
    static constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024;
    static_assert(STAGES * STAGE_BYTES + 1024 <= 227 * 1024, "stages exceed shared memory");
};

struct Params {
    int m, n;              // true output size
    int kblocks;           // padded K / BK
    int Mpad, Npad;        // rows per digit plane of the A / B digit arrays
    int mtiles, ntiles;
    int chunk_kb;          // k-blocks per exact chunk
    int64_t N;
    uint64_t minv;         // floor((2^64-1)/N)
    int64_t bias;          // multiple of N, >= 2^60
    int32_t W[MAX_SHIFTS]; // 2^(bits*s) mod N
    void *C;
    int64_t ldc;
    const double *X, *Y;   // EPI_KSUB_F64 subtrahends
    int *err;
    int *tile_counter;         // nullptr: static tile schedule; else tiles drawn from this counter
    // EPI_SUB_I32M (EPI_SUB_I32 with odd N, one exact chunk whose shift sums stay below 2^22):
    // the chunk values are read by adding 1.5 * 2^23 in fp32 (the integer lands in the
    // mantissa) and reduced by a 32-bit Montgomery step, the weights carrying 2^32.
    uint32_t ninv;             // -N^-1 mod 2^32
    int32_t Wm[MAX_SHIFTS];    // 2^(bits*s) * 2^32 mod N
    int64_t fbias;             // the initial value (fast_consts): takes out the magic-number bits
};

__device__ __forceinline__ void tile_coords(int t, int mtiles, int ntiles, int &tm, int &tn) {
    int group = t / (TILE_GROUP * ntiles);
    int first_m = group * TILE_GROUP;
    int gsz = mtiles - first_m < TILE_GROUP ? mtiles - first_m : TILE_GROUP;
    int local = t - group * TILE_GROUP * ntiles;
    tm = first_m + local % gsz;
    tn = local / gsz;
}

// The fast drain reads a shift sum C (|C| <= 2^22, exact in fp32) by adding 1.5 * 2^23:
// the result's bits are 0x4B400000 + C.  With 7-bit digits the weights of shifts s and
// s + 1 differ by 2^7, so the pair takes the single weight Wm[s]: bits_s + (bits_{s+1} << 7)
// in wrapping 32-bit arithmetic is C_s + 2^7 C_{s+1} + FAST_PAIR_OFFSET exactly, where
// FAST_PAIR_OFFSET = 129 * 0x4B400000 mod 2^32 read as int32 (|C_s + 2^7 C_{s+1}| <= 2^29.01,
// so the sum stays inside int32).  The constants come out through the initial value
// (fast_consts), and a 2L - 1 shift drain does L wide multiply-adds instead of 2L - 1.
constexpr int32_t FAST_MAGIC_BITS = 0x4B400000;
constexpr int32_t FAST_PAIR_OFFSET = -348127232;
__device__ __forceinline__ uint32_t fast_bits(uint32_t v) {
    return __float_as_uint(__fadd_rn(__uint_as_float(v), 12582912.0f));
}
__device__ __forceinline__ int32_t fast_pair(uint32_t lo, uint32_t hi) {
    return (int32_t)(fast_bits(lo) + (fast_bits(hi) << 7));
}

__device__ __forceinline__ int64_t reduce_signed(int64_t acc, const Params &p) {
    // acc + bias is in [0, 2^62); bias = 0 mod N
    return (int64_t)gffm_dev::barrett64((uint64_t)(acc + p.bias), (uint64_t)p.N, p.minv);
}

template <int L, int EPI, int BNV = 64>
__global__ void __launch_bounds__(gemm_threads(EPI), 1)
    k_gemm_limb(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, Params p) {
    using C_ = Cfg<L, BNV>;
    constexpr int AB = C_::ACC_BUFS;
    constexpr int EW = epi_warps(EPI);
    constexpr int EPB = EW / AB;         // epilogue warps per accumulator set
    constexpr int CW = BNV / (EPB / 4);  // output columns per epilogue warp (32 or 16)
    constexpr bool SUB = EPI == EPI_SUB_I32 || EPI == EPI_SUB_I32M;   // read-modify-write of int32 C
    constexpr bool FAST = EPI == EPI_SUB_I32M;
    extern __shared__ uint8_t dsmem_raw[];
    __shared__ uint64_t full_bar[C_::STAGES];
    __shared__ uint64_t empty_bar[C_::STAGES];
    __shared__ uint64_t acc_full_bar[AB], acc_empty_bar[AB];
    __shared__ uint64_t drain_bar;
    __shared__ uint64_t tile_full[TILE_RING], tile_empty[TILE_RING];
    __shared__ int tile_ring[TILE_RING];
    __shared__ uint32_t tmem_base_s;
    __shared__ int abort_sh;
    volatile int &abort_s = abort_sh;

    uint8_t *smem = (uint8_t *)(((uintptr_t)dsmem_raw + 1023) & ~(uintptr_t)1023);
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const int ntiles_total = p.mtiles * p.ntiles;

    if (threadIdx.x == 0) {
        for (int s = 0; s < C_::STAGES; s++) {
            gffm_dev::mbar_init(&full_bar[s], 1);
            gffm_dev::mbar_init(&empty_bar[s], 1);
        }
        for (int b = 0; b < AB; b++) {
            gffm_dev::mbar_init(&acc_full_bar[b], 1);
            gffm_dev::mbar_init(&acc_empty_bar[b], EPB);
        }
        gffm_dev::mbar_init(&drain_bar, 1);
        for (int q = 0; q < TILE_RING; q++) {
            gffm_dev::mbar_init(&tile_full[q], 1);
            gffm_dev::mbar_init(&tile_empty[q], 1 + EW);   // the mma issuer and every epilogue warp
        }
        abort_s = 0;
        gffm_dev::fence_mbar_init();
        gffm_dev::prefetch_tmap(&tmA);
        gffm_dev::prefetch_tmap(&tmB);
    }
    if (warp == 1) gffm_dev::tmem_alloc(&tmem_base_s, C_::TMEM_COLS);
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
            for (int i = 0;; i++) {
                // the next tile, handed to the consumers (-1: none left)
                int t = p.tile_counter ? atomicAdd(p.tile_counter, 1) : blockIdx.x + i * (int)gridDim.x;
                if (abort_s || t >= ntiles_total) t = -1;
                const int slot = i % TILE_RING;
                if (i >= TILE_RING && !gffm_dev::mbar_wait(&tile_empty[slot], (uint32_t)(i / TILE_RING - 1) & 1)) {
                    atomicOr(p.err, 1);
                    abort_s = 1;
                    t = -1;
                }
                tile_ring[slot] = t;
                gffm_dev::mbar_arrive(&tile_full[slot]);
                if (t < 0) break;
                int tm, tn;
                tile_coords(t, p.mtiles, p.ntiles, tm, tn);
                for (int kb = 0; kb < p.kblocks; kb++) {
                    if (!gffm_dev::mbar_wait(&empty_bar[stage], phase ^ 1)) {
                        atomicOr(p.err, 1);
                        abort_s = 1;
                        break;
                    }
                    if (abort_s) break;
                    uint8_t *sa = smem + stage * C_::STAGE_BYTES;
                    uint8_t *sb = sa + L * A_TILE;
                    gffm_dev::mbar_arrive_expect_tx(&full_bar[stage], C_::STAGE_BYTES);
#pragma unroll
                    for (int l = 0; l < L; l++)
                        gffm_dev::tma_load_2d(sa + l * A_TILE, &tmA, &full_bar[stage], kb * BK, l * p.Mpad + tm * BM);
#pragma unroll
                    for (int l = 0; l < L; l++)
                        gffm_dev::tma_load_2d(sb + l * C_::B_T, &tmB, &full_bar[stage], kb * BK, l * p.Npad + tn * BNV);
                    issued_mask |= 1u << stage;
                    issued_parity_mask = (issued_parity_mask & ~(1u << stage)) | (phase << stage);
                    if (++stage == C_::STAGES) {
                        stage = 0;
                        phase ^= 1;
                    }
                }
            }
            if (abort_s) {
                // let copies already in flight land before the CTA exits (bounded)
                for (int s = 0; s < C_::STAGES; s++)
                    if (issued_mask & (1u << s)) gffm_dev::mbar_wait(&full_bar[s], (issued_parity_mask >> s) & 1);
            }
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer ----------------
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0;
            uint32_t acc_phase[AB];
#pragma unroll
            for (int b = 0; b < AB; b++) acc_phase[b] = 0;
            bool issued_any = false;
            const uint32_t idesc_full = gffm_dev::idesc_f16_f32(BM, BNV * L);
            const uint32_t idesc_lo = gffm_dev::idesc_f16_f32(BM, BNV * (L > 1 ? L - 1 : 1));
            const uint32_t idesc_one = gffm_dev::idesc_f16_f32(BM, BNV);
            int local = 0;
            for (int i = 0; !abort_s; i++, local++) {
                const int slot = i % TILE_RING;
                if (!gffm_dev::mbar_wait(&tile_full[slot], (uint32_t)(i / TILE_RING) & 1)) {
                    atomicOr(p.err, 2);
                    abort_s = 1;
                    break;
                }
                const int t = tile_ring[slot];
                gffm_dev::mbar_arrive(&tile_empty[slot]);
                if (t < 0) break;
                const int buf = AB == 2 ? (local & 1) : 0;
                const uint32_t acc = tmem + (uint32_t)(buf * C_::BUF_COLS);
                for (int kb0 = 0; kb0 < p.kblocks && !abort_s; kb0 += p.chunk_kb) {
                    int kb1 = kb0 + p.chunk_kb < p.kblocks ? kb0 + p.chunk_kb : p.kblocks;
                    if (!gffm_dev::mbar_wait(&acc_empty_bar[buf], acc_phase[buf] ^ 1)) {
                        atomicOr(p.err, 2);
                        abort_s = 1;
                        break;
                    }
                    gffm_dev::tc_fence_after();
                    for (int kb = kb0; kb < kb1; kb++) {
                        if (!gffm_dev::mbar_wait(&full_bar[stage], phase)) {
                            atomicOr(p.err, 4);
                            abort_s = 1;
                            break;
                        }
                        gffm_dev::tc_fence_after();
                        const uint32_t sa = gffm_dev::smem_u32(smem + stage * C_::STAGE_BYTES);
                        const uint32_t sb = sa + L * A_TILE;
#pragma unroll
                        for (int kk = 0; kk < BK / 16; kk++) {
                            const uint64_t bdesc = gffm_dev::umma_desc_sw128(sb + kk * 32);
                            if (kb == kb0 && kk == 0) {
                                // first k-step of a chunk: initialise every shift accumulator once
                                gffm_dev::mma_f16(acc, gffm_dev::umma_desc_sw128(sa + kk * 32), bdesc, idesc_full, 0);
#pragma unroll
                                for (int i = 1; i < L; i++) {
                                    const uint64_t adesc = gffm_dev::umma_desc_sw128(sa + i * A_TILE + kk * 32);
                                    gffm_dev::mma_f16(acc + BNV * i, adesc, bdesc, idesc_lo, 1);
                                    gffm_dev::mma_f16(acc + BNV * (i + L - 1), adesc,
                                                      gffm_dev::umma_desc_sw128(sb + (L - 1) * C_::B_T + kk * 32),
                                                      idesc_one, 0);
                                }
                            } else {
#pragma unroll
                                for (int i = 0; i < L; i++)
                                    gffm_dev::mma_f16(acc + BNV * i, gffm_dev::umma_desc_sw128(sa + i * A_TILE + kk * 32),
                                                      bdesc, idesc_full, 1);
                            }
                        }
                        issued_any = true;
                        gffm_dev::mma_commit(&empty_bar[stage]);  // frees the stage once these mma's finish
                        if (++stage == C_::STAGES) {
                            stage = 0;
                            phase ^= 1;
                        }
                    }
                    if (abort_s) break;
                    gffm_dev::mma_commit(&acc_full_bar[buf]);
                    acc_phase[buf] ^= 1;
                }
            }
            if (abort_s && issued_any) {
                // wait (bounded) until every mma issued so far has completed
                gffm_dev::mma_commit(&drain_bar);
                gffm_dev::mbar_wait(&drain_bar, 0);
            }
        }
    } else {
        // ---------------- epilogue ----------------
        const int ew = warp - 2;
        const int quad = warp & 3;       // TMEM lane quadrant this warp may access
        // each group of four consecutive warps covers the four quadrants; a group
        // owns one accumulator set (BNV = 32) and CW of its columns
        const int grp = ew >> 2;
        const int buf = AB == 2 ? grp / (EPB / 4) : 0;
        const int part = grp % (EPB / 4);
        uint32_t acc_phase = 0;
        int local = 0;
        for (int i = 0;; i++, local++) {
            const int slot = i % TILE_RING;
            if (!gffm_dev::mbar_wait(&tile_full[slot], (uint32_t)(i / TILE_RING) & 1)) {
                atomicOr(p.err, 8);
                abort_s = 1;
                break;
            }
            const int t = tile_ring[slot];
            __syncwarp();
            if (lane == 0) gffm_dev::mbar_arrive(&tile_empty[slot]);
            if (t < 0) break;
            if (AB == 2 && (local & 1) != buf) continue;      // the other warp group's tile
            const uint32_t accb = tmem + (uint32_t)(buf * C_::BUF_COLS) + (uint32_t)(CW * part);
            int tm, tn;
            tile_coords(t, p.mtiles, p.ntiles, tm, tn);
            const int64_t row = (int64_t)tm * BM + quad * 32 + lane;
            const int64_t col0 = (int64_t)tn * BNV + CW * part;
            // read-modify-write: C's values are loaded before the accumulators are ready
            int32_t cv[SUB ? CW : 1];
            if (SUB) {
                const int32_t *cbase = (const int32_t *)p.C + row + col0 * p.ldc;
#pragma unroll
                for (int j = 0; j < CW; j++) cv[j] = (row < p.m && col0 + j < p.n) ? __ldcg(cbase + j * p.ldc) : 0;
            }
            int64_t acc[CW];
#pragma unroll
            for (int j = 0; j < CW; j++) acc[j] = FAST ? p.fbias : 0;
            int32_t dp[FAST ? (C_::NSHIFT + 1) / 2 : 1][FAST ? CW : 1];   // the fast drain's pairs
            bool ok = true;
            int chunk = 0;
            for (int kb0 = 0; kb0 < p.kblocks; kb0 += p.chunk_kb, chunk++) {
                if (!gffm_dev::mbar_wait(&acc_full_bar[buf], acc_phase)) {
                    atomicOr(p.err, 8);
                    abort_s = 1;
                    ok = false;
                    break;
                }
                gffm_dev::tc_fence_after();
                if (FAST) {
                    // shifts in pairs (fast_pair), kept as int32 until the accumulator is
                    // released; 8 columns of both shifts at a time
#pragma unroll
                    for (int s = 0; s < C_::NSHIFT; s += 2) {
#pragma unroll
                        for (int h = 0; h < CW; h += 8) {
                            uint32_t v[8], u[8];
                            const uint32_t ta = accb + ((uint32_t)(quad * 32) << 16) + BNV * s + h;
                            gffm_dev::tmem_ld_32x32b_x8(ta, v);
                            if (s + 1 < C_::NSHIFT) gffm_dev::tmem_ld_32x32b_x8(ta + BNV, u);
                            gffm_dev::tmem_ld_wait();
#pragma unroll
                            for (int j = 0; j < 8; j++)
                                dp[s / 2][h + j] = s + 1 < C_::NSHIFT ? fast_pair(v[j], u[j]) : (int32_t)fast_bits(v[j]);
                        }
                    }
                }
#pragma unroll
                for (int s = 0; s < (FAST ? 0 : C_::NSHIFT); s++) {
                    uint32_t v[CW];
                    gffm_dev::tmem_ld_32x32b<CW>(accb + ((uint32_t)(quad * 32) << 16) + BNV * s, v);
                    gffm_dev::tmem_ld_wait();
                    if (EPI == EPI_EXACT_I64) {
                        // exact chunk value sum_s C_s 2^(7s), in [0, 2^62) for raw digits: wrapping
                        // 64-bit sums are exact once every shift has been added
#pragma unroll
                        for (int j = 0; j < CW; j++)
                            acc[j] = (int64_t)((uint64_t)acc[j] +
                                               ((uint64_t)(int64_t)__float2int_rz(__uint_as_float(v[j])) << (7 * s)));
                    } else {
                        const int w = p.W[s];
#pragma unroll
                        for (int j = 0; j < CW; j++) acc[j] += (int64_t)__float2int_rz(__uint_as_float(v[j])) * w;
                    }
                }
                gffm_dev::tc_fence_before();
                __syncwarp();
                if (lane == 0) gffm_dev::mbar_arrive(&acc_empty_bar[buf]);
                acc_phase ^= 1;
                if (FAST) {
                    // the wide multiply-adds run while the next tile's mma's fill the accumulator
#pragma unroll
                    for (int i = 0; i < (C_::NSHIFT + 1) / 2; i++) {
                        const int w = p.Wm[2 * i];
#pragma unroll
                        for (int j = 0; j < CW; j++) acc[j] += (int64_t)dp[i][j] * w;
                    }
                }
                if (EPI == EPI_EXACT_I64) {
                    // acc < N < 2^52 before the chunk, so acc + chunk < 2^63: one Barrett step
#pragma unroll
                    for (int j = 0; j < CW; j++)
                        acc[j] = (int64_t)gffm_dev::barrett64((uint64_t)acc[j], (uint64_t)p.N, p.minv);
                } else if ((chunk & 63) == 63) {
#pragma unroll
                    for (int j = 0; j < CW; j++) acc[j] = reduce_signed(acc[j], p);
                }
            }
            if (!ok || abort_s) break;
            if (row < p.m) {
                if (SUB) {
                    int32_t *cbase = (int32_t *)p.C + row + col0 * p.ldc;
                    if (FAST) {
                        // x in (0, 2^32 N): t = (x + m N) / 2^32 < 2N, t = x 2^-32 mod N
                        const uint32_t n32 = (uint32_t)p.N;
#pragma unroll
                        for (int j = 0; j < CW; j++) {
                            const uint64_t x = (uint64_t)acc[j];
                            const uint32_t m = (uint32_t)x * p.ninv;
                            uint32_t r = (uint32_t)((x + (uint64_t)m * n32) >> 32);
                            r = r >= n32 ? r - n32 : r;
                            const int32_t v = cv[j] - (int32_t)r;
                            if (col0 + CW <= p.n || col0 + j < p.n) cbase[j * p.ldc] = v < 0 ? v + (int32_t)n32 : v;
                        }
                    } else {
#pragma unroll
                        for (int j = 0; j < CW; j++) {
                            if (col0 + j < p.n) {
                                const int64_t v = (int64_t)cv[j] - reduce_signed(acc[j], p);
                                cbase[j * p.ldc] = (int32_t)(v < 0 ? v + p.N : v);
                            }
                        }
                    }
                } else if (EPI == EPI_EXACT_I64) {
                    int64_t *cbase = (int64_t *)p.C + row + col0 * p.ldc;
#pragma unroll
                    for (int j = 0; j < CW; j++)
                        if (col0 + j < p.n) cbase[j * p.ldc] = acc[j];
                } else if (EPI == EPI_KSUB_F64) {
                    // C = (AB - X - Y) mod N: all subtrahend loads before any store
                    const int64_t base = row + col0 * p.ldc;
                    double xv[CW];
#pragma unroll
                    for (int j = 0; j < CW; j++)
                        xv[j] = (col0 + j < p.n) ? __ldcg(p.X + base + j * p.ldc) + __ldcg(p.Y + base + j * p.ldc) : 0.0;
#pragma unroll
                    for (int j = 0; j < CW; j++) {
                        if (col0 + j < p.n) {
                            int64_t v = reduce_signed(acc[j], p) - (int64_t)xv[j];   // X + Y < 2N, exact in double
                            v += (v < 0) ? p.N : 0;
                            v += (v < 0) ? p.N : 0;
                            ((double *)p.C)[base + j * p.ldc] = (double)v;
                        }
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < CW; j++) {
                        const int64_t col = col0 + j;
                        if (col < p.n) {
                            const int64_t r = reduce_signed(acc[j], p);
                            const int64_t off = row + col * p.ldc;
                            if (EPI == EPI_STORE_F64)
                                ((double *)p.C)[off] = (double)r;
                            else if (EPI == EPI_STORE_F32)
                                ((float *)p.C)[off] = (float)r;
                            else
                                ((int32_t *)p.C)[off] = (int32_t)r;
                        }
                    }
                }
            }
        }
    }

    gffm_dev::tc_fence_before();
    __syncthreads();
    gffm_dev::tc_fence_after();
    if (warp == 1) gffm_dev::tmem_dealloc(tmem, C_::TMEM_COLS);
}

// ---------------------------------------------------------------------------
// Digit split kernels
// ---------------------------------------------------------------------------
struct ModN {
    int64_t n;
    uint64_t minv;
};

// residue of an integer-valued element in [0, N)
template <typename T>
__device__ __forceinline__ int32_t residue(T v, const ModN &M) {
    int64_t x = (int64_t)v;
    int64_t r;
    if (x >= 0 && x < M.n) {
        r = x;
    } else if (x >= 0) {
        r = (int64_t)gffm_dev::barrett64((uint64_t)x, (uint64_t)M.n, M.minv);
    } else {
        uint64_t q = gffm_dev::barrett64((uint64_t)(-x), (uint64_t)M.n, M.minv);
        r = q ? M.n - (int64_t)q : 0;
    }
    return (int32_t)r;
}

// the value a split of mode MODE encodes for element v (and v2, SPLIT_SUM)
template <int MODE, typename T>
__device__ __forceinline__ int32_t split_value(T v, T v2, const ModN &M) {
    int32_t r = residue(v, M);
    if (MODE == SPLIT_RAW) return r;
    if (MODE == SPLIT_SUM) {
        r += residue(v2, M);
        if (r >= M.n) r -= (int32_t)M.n;
    }
    return (2 * (int64_t)r > M.n) ? r - (int32_t)M.n : r;
}

// L balanced base-2^bits digits of c (bits = 7: digits in [-64, 63]; bits = 8: [-128, 127])
template <int L>
__device__ __forceinline__ void digits(int32_t c, __half (&d)[L], int bits = 7) {
    const int32_t half = 1 << (bits - 1), mask = (1 << bits) - 1;
#pragma unroll
    for (int i = 0; i < L; i++) {
        int32_t di = ((c + half) & mask) - half;
        d[i] = __int2half_rn(di);
        c = (c - di) >> bits;
    }
}

// A (m x k, column-major, lda) -> digit planes D[l][r][kk] (K-major, Mpad x Kpad per plane)
template <typename T, int L, int MODE>
__global__ void __launch_bounds__(256) k_split_a(const T *__restrict__ A, const T *__restrict__ A2, int64_t lda, int m,
                                                 int k, __half *__restrict__ D, int Mpad, int Kpad, ModN M, int bits) {
    __shared__ int32_t tile[32][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int64_t r0 = (int64_t)blockIdx.y * 32, k0 = (int64_t)blockIdx.x * 32;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        int64_t kk = k0 + ty + 8 * i, r = r0 + tx;
        int32_t v = 0;
        if (r < m && kk < k) {
            const int64_t off = r + kk * lda;
            v = split_value<MODE>(A[off], MODE == SPLIT_SUM ? A2[off] : T(0), M);
        }
        tile[ty + 8 * i][tx] = v;
    }
    __syncthreads();
    const size_t plane = (size_t)Mpad * Kpad;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        int64_t r = r0 + ty + 8 * i, kk = k0 + tx;
        __half d[L];
        digits<L>(tile[tx][ty + 8 * i], d, bits);
#pragma unroll
        for (int l = 0; l < L; l++) D[l * plane + (size_t)r * Kpad + kk] = d[l];
    }
}

// B (k x n, column-major, ldb) -> digit planes D[l][c][kk] (K-major, Npad x Kpad per plane)
template <typename T, int L, int MODE>
__global__ void __launch_bounds__(256) k_split_b(const T *__restrict__ B, const T *__restrict__ B2, int64_t ldb, int k,
                                                 int n, __half *__restrict__ D, int Npad, int Kpad, ModN M, int bits) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;  // pair index
    const int64_t pairs_per_col = Kpad / 2;
    const int64_t total = pairs_per_col * Npad;
    if (idx >= total) return;
    const int64_t c = idx / pairs_per_col;
    const int64_t kk = (idx - c * pairs_per_col) * 2;
    const int64_t off = kk + c * ldb;
    int32_t v0 = (c < n && kk < k) ? split_value<MODE>(B[off], MODE == SPLIT_SUM ? B2[off] : T(0), M) : 0;
    int32_t v1 = (c < n && kk + 1 < k) ? split_value<MODE>(B[off + 1], MODE == SPLIT_SUM ? B2[off + 1] : T(0), M) : 0;
    __half d0[L], d1[L];
    digits<L>(v0, d0, bits);
    digits<L>(v1, d1, bits);
    const size_t plane = (size_t)Npad * Kpad;
#pragma unroll
    for (int l = 0; l < L; l++)
        *reinterpret_cast<__half2 *>(D + l * plane + (size_t)c * Kpad + kk) = __halves2half2(d0[l], d1[l]);
}

}  // namespace limb
