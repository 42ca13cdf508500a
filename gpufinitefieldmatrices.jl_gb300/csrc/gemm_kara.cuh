// gemm_kara.cuh -- exact modular GEMM for moduli of four 7-bit digits
// (2080639 < N < 2^26) with one level of Karatsuba over 13-bit halves:
// 12 fp16 digit products per modular multiply-add instead of the schoolbook's 16.
//
// Representation.  A residue x in [0, N) is centred to c in (-N/2, N/2],
// |c| < 2^25, and split into balanced halves and digits
//     c  = lo + 2^13 hi,          lo in [-4096, 4095], |hi| <= 4096
//     lo = a0 + 2^7 a1,           a0 in [-64, 63],     |a1| <= 32
//     hi = a2 + 2^7 a3,           a2 in [-64, 63],     |a3| <= 32
// plus the balanced digits of the Karatsuba sum S = lo + hi (|S| <= 8192):
//     S  = s0 + 2^7 s1,           s0 in [-64, 63],     |s1| <= 64
// (any digit split of S serves, since the middle product only has to equal
// (A_lo + A_hi)(B_lo + B_hi); this one keeps its per-k sums at half of what
// s0 = a0 + a2, s1 = a1 + a3 would give): six digit planes
// [a0, a1, a2, a3, s0, s1], every value exact in fp16.
//
// Products.  With X = 2^7 and Y = 2^13, for each pair of half-numbers
//     P0 = (a0 + X a1)(b0 + X b1)    planes 0, 1
//     P2 = (a2 + X a3)(b2 + X b3)    planes 2, 3
//     Pm = (s0 + X s1)(t0 + X t1)    planes 4, 5
// (each summed over k), A*B = P0 + Y (Pm - P0 - P2) + Y^2 P2.  Each P is a
// two-digit schoolbook product with three shift accumulators
// P = C_0 + X C_1 + X^2 C_2, so
//     A*B = sum_s X^s [ (1 - Y) C0_s + (Y^2 - Y) C2_s + Y Cm_s ]
// and the epilogue adds C_{p,s} * W[p][s] with the weights reduced mod N.
//
// Tensor-core mapping.  An output tile is 128 x 128.  The products run one
// after the other (product-outer loop): for product p a pipeline stage holds
// the two A digit tiles x0, x1 (128 x 64 each) and the two B digit tiles y0,
// y1 stacked into one 256-row operand B' = [y0; y1].  Per k-step of 16,
// tcgen05.mma x0 x B' (M = 128, N = 256) writes [x0 y0 | x0 y1] at TMEM
// columns 0..255 and x1 x B' writes [x1 y0 | x1 y1] at columns 128..383, so
// the shift-s accumulator C_s sits at columns 128 s.  N = 256 is the width
// at which an M = 128 mma runs at the full tensor rate on this GPU (measured:
// N = 128 and N = 64 mma's take about 95 cycles each, bound by a
// per-instruction floor, against 128 cycles for N = 256).
//
// Exactness.  Per k, |C_s| <= 4096 for P0 and P2 (|a0 b0| <= 4096,
// |a0 b1| + |a1 b0| <= 4096, |a1 b1| <= 1024) and <= 8192 for Pm
// (|s0 t0| <= 4096, |s0 t1| + |s1 t0| <= 8192, |s1 t1| <= 4096), so chunks of
// 4096 (P0, P2) and 2048 (Pm) values of k keep every fp32 partial sum within
// 2^24.  After each chunk the epilogue drains the three accumulators into
// int64 registers, exactly as the schoolbook kernel (gemm_limb.cuh) does.
//
// Accumulator slots.  TMEM's 512 columns are four 128-column slots; exact
// chunk g keeps its shifts 0, 1, 2 in slots (g & 1) + 0, 1, 2, so consecutive
// chunks share two slots and each has one of its own.  The epilogue drains the
// shared slots first and frees each slot on its own barrier, and the mma
// issuer waits for a slot only before its first write of the chunk: the next
// chunk's mma's start once two of the previous chunk's three accumulators are
// drained, and the third drain runs beside them.
//
// Warp roles (576 threads): warp 0 TMA producer, warp 1 TMEM allocator and
// single-thread mma issuer, warps 2..17 the epilogue (four per TMEM lane
// quadrant, 32 of the 128 columns each).  Every wait is bounded; on timeout
// the kernel records the failure in the library's error word, lets its own
// copies and mma's finish and frees TMEM before returning.
#pragma once

#include "gemm_limb.cuh"

namespace kara {

constexpr int BM = 128;                  // output rows per tile
constexpr int BN = 128;                  // output columns per tile
constexpr int BK = 64;                   // k per stage (one 128-byte swizzle row of fp16)
constexpr int PLANES = 6;                // a0 a1 a2 a3 s0 s1
constexpr int TILE = 128 * BK * 2;       // one 128-row digit tile: 16 KB
constexpr int STAGE_BYTES = 4 * TILE;    // x0, x1, y0, y1
constexpr int STAGES = 3;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024;
constexpr int EPI_WARPS = 16;
constexpr int THREADS = 64 + 32 * EPI_WARPS;
constexpr int TMEM_COLS = 512;           // four 128-column slots: a chunk's three shift accumulators at slot 0 or 1
static_assert(SMEM_BYTES <= 227 * 1024, "stages exceed shared memory");

struct Params {
    int m, n;                 // true output size
    int kblocks;              // padded K / BK
    int Mpad, Npad;           // rows per digit plane of the A / B digit arrays
    int mtiles, ntiles;
    int chunk_kb[3];          // k-blocks per exact chunk, per product (P0, P2, Pm)
    int64_t N;
    uint64_t minv;            // floor((2^64-1)/N)
    int64_t bias;             // multiple of N, >= 2^60
    int32_t W[3][3];          // [product][shift] weights mod N
    void *C;
    int64_t ldc;
    const double *X, *Y;      // EPI_KSUB_F64 subtrahends
    int *err;
};

__device__ __forceinline__ int64_t reduce_signed(int64_t acc, const Params &p) {
    return (int64_t)gffm_dev::barrett64((uint64_t)(acc + p.bias), (uint64_t)p.N, p.minv);
}

template <int EPI>
__global__ void __launch_bounds__(THREADS, 1)
    k_gemm_kara(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, Params p) {
    using limb::tile_coords;
    extern __shared__ uint8_t dsmem_raw[];
    __shared__ uint64_t full_bar[STAGES];
    __shared__ uint64_t empty_bar[STAGES];
    __shared__ uint64_t acc_full_bar, slot_free_bar[4], drain_bar;
    __shared__ uint32_t tmem_base_s;
    __shared__ int abort_sh;
    volatile int &abort_s = abort_sh;

    uint8_t *smem = (uint8_t *)(((uintptr_t)dsmem_raw + 1023) & ~(uintptr_t)1023);
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const int ntiles_total = p.mtiles * p.ntiles;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; s++) {
            gffm_dev::mbar_init(&full_bar[s], 1);
            gffm_dev::mbar_init(&empty_bar[s], 1);
        }
        gffm_dev::mbar_init(&acc_full_bar, 1);
        for (int q = 0; q < 4; q++) gffm_dev::mbar_init(&slot_free_bar[q], EPI_WARPS);
        gffm_dev::mbar_init(&drain_bar, 1);
        abort_s = 0;
        gffm_dev::fence_mbar_init();
        gffm_dev::prefetch_tmap(&tmA);
        gffm_dev::prefetch_tmap(&tmB);
    }
    if (warp == 1) gffm_dev::tmem_alloc(&tmem_base_s, TMEM_COLS);
    gffm_dev::tc_fence_before();
    __syncthreads();
    gffm_dev::tc_fence_after();
    const uint32_t tmem = tmem_base_s;

    if (warp == 0) {
        // ---------------- TMA producer: tile, product, k-block ----------------
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0;
            uint32_t issued_parity_mask = 0, issued_mask = 0;
            for (int t = blockIdx.x; t < ntiles_total && !abort_s; t += gridDim.x) {
                int tm, tn;
                tile_coords(t, p.mtiles, p.ntiles, tm, tn);
                for (int prod = 0; prod < 3 && !abort_s; prod++) {
                    for (int kb = 0; kb < p.kblocks; kb++) {
                        if (!gffm_dev::mbar_wait(&empty_bar[stage], phase ^ 1)) {
                            atomicOr(p.err, 1);
                            abort_s = 1;
                            break;
                        }
                        if (abort_s) break;
                        uint8_t *sa = smem + stage * STAGE_BYTES;
                        uint8_t *sb = sa + 2 * TILE;
                        gffm_dev::mbar_arrive_expect_tx(&full_bar[stage], STAGE_BYTES);
#pragma unroll
                        for (int l = 0; l < 2; l++)
                            gffm_dev::tma_load_2d(sa + l * TILE, &tmA, &full_bar[stage], kb * BK,
                                                  (2 * prod + l) * p.Mpad + tm * BM);
#pragma unroll
                        for (int l = 0; l < 2; l++)
                            gffm_dev::tma_load_2d(sb + l * TILE, &tmB, &full_bar[stage], kb * BK,
                                                  (2 * prod + l) * p.Npad + tn * BN);
                        issued_mask |= 1u << stage;
                        issued_parity_mask = (issued_parity_mask & ~(1u << stage)) | (phase << stage);
                        if (++stage == STAGES) {
                            stage = 0;
                            phase ^= 1;
                        }
                    }
                }
            }
            if (abort_s) {
                for (int s = 0; s < STAGES; s++)
                    if (issued_mask & (1u << s)) gffm_dev::mbar_wait(&full_bar[s], (issued_parity_mask >> s) & 1);
            }
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer ----------------
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0;
            bool issued_any = false;
            const uint32_t idesc_wide = gffm_dev::idesc_f16_f32(BM, 2 * BN);
            const uint32_t idesc_one = gffm_dev::idesc_f16_f32(BM, BN);
            // before chunk g's first write of slot q: the slot's previous chunk is drained.  Slots
            // 1 and 2 serve every chunk, slot 0 the even chunks, slot 3 the odd ones, so the
            // chunks before g that used slot q are g, g / 2 or (g - 1) / 2, and the slot's
            // barrier has completed one phase per drained use.
            auto claim = [&](int q, int g) {
                const int prior = (q == 1 || q == 2) ? g : (q == 0 ? g >> 1 : (g - 1) >> 1);
                if (prior > 0 && !gffm_dev::mbar_wait(&slot_free_bar[q], (uint32_t)(prior - 1) & 1)) {
                    atomicOr(p.err, 2);
                    abort_s = 1;
                    return false;
                }
                gffm_dev::tc_fence_after();
                return true;
            };
            int g = 0;   // chunk counter: the slot base alternates
            for (int t = blockIdx.x; t < ntiles_total && !abort_s; t += gridDim.x) {
                for (int prod = 0; prod < 3 && !abort_s; prod++) {
                    const int ckb = p.chunk_kb[prod];
                    for (int kb0 = 0; kb0 < p.kblocks && !abort_s; kb0 += ckb, g++) {
                        const int kb1 = kb0 + ckb < p.kblocks ? kb0 + ckb : p.kblocks;
                        const int sb = g & 1;   // slot of this chunk's shift 0
                        const uint32_t acc = tmem + (uint32_t)(BN * sb);
                        for (int kb = kb0; kb < kb1; kb++) {
                            if (!gffm_dev::mbar_wait(&full_bar[stage], phase)) {
                                atomicOr(p.err, 4);
                                abort_s = 1;
                                break;
                            }
                            gffm_dev::tc_fence_after();
                            const uint32_t sa = gffm_dev::smem_u32(smem + stage * STAGE_BYTES);
                            const uint32_t sbb = sa + 2 * TILE;
#pragma unroll
                            for (int kk = 0; kk < BK / 16; kk++) {
                                const uint64_t bdesc = gffm_dev::umma_desc_sw128(sbb + kk * 32);
                                const uint64_t a0 = gffm_dev::umma_desc_sw128(sa + kk * 32);
                                const uint64_t a1 = gffm_dev::umma_desc_sw128(sa + TILE + kk * 32);
                                if (kb == kb0 && kk == 0) {
                                    // first k-step of a chunk: initialise the three shift accumulators
                                    // once, each slot claimed just before its first write
                                    if (!claim(sb, g) || !claim(sb + 1, g)) break;
                                    gffm_dev::mma_f16(acc, a0, bdesc, idesc_wide, 0);
                                    gffm_dev::mma_f16(acc + BN, a1, bdesc, idesc_one, 1);
                                    if (!claim(sb + 2, g)) break;
                                    gffm_dev::mma_f16(acc + 2 * BN, a1, gffm_dev::umma_desc_sw128(sbb + TILE + kk * 32),
                                                      idesc_one, 0);
                                } else {
                                    gffm_dev::mma_f16(acc, a0, bdesc, idesc_wide, 1);
                                    gffm_dev::mma_f16(acc + BN, a1, bdesc, idesc_wide, 1);
                                }
                            }
                            if (abort_s) break;
                            issued_any = true;
                            gffm_dev::mma_commit(&empty_bar[stage]);
                            if (++stage == STAGES) {
                                stage = 0;
                                phase ^= 1;
                            }
                        }
                        if (abort_s) break;
                        gffm_dev::mma_commit(&acc_full_bar);
                    }
                }
            }
            if (abort_s && issued_any) {
                gffm_dev::mma_commit(&drain_bar);
                gffm_dev::mbar_wait(&drain_bar, 0);
            }
        }
    } else {
        // ---------------- epilogue ----------------
        constexpr int CW = BN / (EPI_WARPS / 4);   // 32 output columns per warp
        const int quad = warp & 3;                 // TMEM lane quadrant this warp may access
        const int part = (warp - 2) >> 2;          // which 32 of the tile's 128 columns
        const uint32_t lane_base = (uint32_t)(quad * 32) << 16;
        uint32_t acc_phase = 0;
        int g = 0;   // chunk counter, as the mma issuer's
        for (int t = blockIdx.x; t < ntiles_total; t += gridDim.x) {
            int tm, tn;
            tile_coords(t, p.mtiles, p.ntiles, tm, tn);
            const int64_t row = (int64_t)tm * BM + quad * 32 + lane;
            const int64_t col0 = (int64_t)tn * BN + CW * part;
            int64_t acc[CW];
#pragma unroll
            for (int j = 0; j < CW; j++) acc[j] = 0;
            bool ok = true;
            int chunk = 0;
            for (int prod = 0; prod < 3 && ok; prod++) {
                const int ckb = p.chunk_kb[prod];
                for (int kb0 = 0; kb0 < p.kblocks; kb0 += ckb, chunk++, g++) {
                    if (!gffm_dev::mbar_wait(&acc_full_bar, acc_phase)) {
                        atomicOr(p.err, 8);
                        abort_s = 1;
                        ok = false;
                        break;
                    }
                    acc_phase ^= 1;
                    gffm_dev::tc_fence_after();
                    // shift s of this chunk sits in slot `slot`; once drained the slot is freed
                    auto drain = [&](int s, int slot) {
                        const int w = p.W[prod][s];
#pragma unroll
                        for (int h = 0; h < CW / 8; h++) {
                            uint32_t v[8];
                            gffm_dev::tmem_ld_32x32b_x8(tmem + lane_base + BN * slot + CW * part + 8 * h, v);
                            gffm_dev::tmem_ld_wait();
#pragma unroll
                            for (int j = 0; j < 8; j++)
                                acc[8 * h + j] += (int64_t)__float2int_rz(__uint_as_float(v[j])) * w;
                        }
                        gffm_dev::tc_fence_before();
                        __syncwarp();
                        if (lane == 0) gffm_dev::mbar_arrive(&slot_free_bar[slot]);
                    };
                    // the slots the next chunk writes first are drained first: shifts 1, 2, 0 after a
                    // chunk at slot 0, shifts 0, 1, 2 after a chunk at slot 1
                    if ((g & 1) == 0) {
                        drain(1, 1);
                        drain(2, 2);
                        drain(0, 0);
                    } else {
                        drain(0, 1);
                        drain(1, 2);
                        drain(2, 3);
                    }
                    // each chunk adds less than 3 * 2^50 in magnitude: reduce every 64 chunks
                    if ((chunk & 63) == 63) {
#pragma unroll
                        for (int j = 0; j < CW; j++) acc[j] = reduce_signed(acc[j], p);
                    }
                }
            }
            if (!ok || abort_s) break;
            if (row < p.m) {
                if (EPI == limb::EPI_KSUB_F64) {
                    const int64_t base = row + col0 * p.ldc;
#pragma unroll
                    for (int h = 0; h < CW / 8; h++) {
                        double xv[8];
#pragma unroll
                        for (int j = 0; j < 8; j++) {
                            const int64_t col = col0 + 8 * h + j;
                            xv[j] = col < p.n ? __ldcg(p.X + base + (8 * h + j) * p.ldc) +
                                                    __ldcg(p.Y + base + (8 * h + j) * p.ldc)
                                              : 0.0;
                        }
#pragma unroll
                        for (int j = 0; j < 8; j++) {
                            if (col0 + 8 * h + j < p.n) {
                                int64_t v = reduce_signed(acc[8 * h + j], p) - (int64_t)xv[j];   // X + Y < 2N
                                v += (v < 0) ? p.N : 0;
                                v += (v < 0) ? p.N : 0;
                                ((double *)p.C)[base + (8 * h + j) * p.ldc] = (double)v;
                            }
                        }
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < CW; j++) {
                        const int64_t col = col0 + j;
                        if (col < p.n) {
                            const int64_t r = reduce_signed(acc[j], p);
                            const int64_t off = row + col * p.ldc;
                            if (EPI == limb::EPI_STORE_F64)
                                ((double *)p.C)[off] = (double)r;
                            else if (EPI == limb::EPI_STORE_F32)
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
    if (warp == 1) gffm_dev::tmem_dealloc(tmem, TMEM_COLS);
}

// ---------------------------------------------------------------------------
// Digit split: six planes per operand
// ---------------------------------------------------------------------------
__device__ __forceinline__ void digits6(int32_t c, __half (&d)[PLANES]) {
    const int32_t lo = ((c + 4096) & 8191) - 4096;
    const int32_t hi = (c - lo) >> 13;
    const int32_t a0 = ((lo + 64) & 127) - 64, a1 = (lo - a0) >> 7;
    const int32_t a2 = ((hi + 64) & 127) - 64, a3 = (hi - a2) >> 7;
    d[0] = __int2half_rn(a0);
    d[1] = __int2half_rn(a1);
    d[2] = __int2half_rn(a2);
    d[3] = __int2half_rn(a3);
    const int32_t S = lo + hi;                                  // |S| <= 8192
    const int32_t s0 = ((S + 64) & 127) - 64, s1 = (S - s0) >> 7;
    d[4] = __int2half_rn(s0);
    d[5] = __int2half_rn(s1);
}

// A (m x k, column-major, lda) -> planes D[pl][r][kk] (K-major, Mpad x Kpad per plane); MODE is
// limb::SPLIT_CENTRED, or limb::SPLIT_SUM for the centred (A + A2) mod N
template <typename T, int MODE>
__global__ void __launch_bounds__(256) k_split_a6(const T *__restrict__ A, const T *__restrict__ A2, int64_t lda, int m,
                                                  int k, __half *__restrict__ D, int Mpad, int Kpad, limb::ModN M) {
    __shared__ int32_t tile[32][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int64_t r0 = (int64_t)blockIdx.y * 32, k0 = (int64_t)blockIdx.x * 32;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int64_t kk = k0 + ty + 8 * i, r = r0 + tx;
        int32_t v = 0;
        if (r < m && kk < k) {
            const int64_t off = r + kk * lda;
            v = limb::split_value<MODE>(A[off], MODE == limb::SPLIT_SUM ? A2[off] : T(0), M);
        }
        tile[ty + 8 * i][tx] = v;
    }
    __syncthreads();
    const size_t plane = (size_t)Mpad * Kpad;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int64_t r = r0 + ty + 8 * i, kk = k0 + tx;
        __half d[PLANES];
        digits6(tile[tx][ty + 8 * i], d);
#pragma unroll
        for (int l = 0; l < PLANES; l++) D[l * plane + (size_t)r * Kpad + kk] = d[l];
    }
}

// B (k x n, column-major, ldb) -> planes D[pl][c][kk] (K-major, Npad x Kpad per plane); two k per thread
template <typename T, int MODE>
__global__ void __launch_bounds__(256) k_split_b6(const T *__restrict__ B, const T *__restrict__ B2, int64_t ldb, int k,
                                                  int n, __half *__restrict__ D, int Npad, int Kpad, limb::ModN M) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t pairs_per_col = Kpad / 2;
    if (idx >= pairs_per_col * Npad) return;
    const int64_t c = idx / pairs_per_col;
    const int64_t kk = (idx - c * pairs_per_col) * 2;
    const int64_t off = kk + c * ldb;
    const bool sum = MODE == limb::SPLIT_SUM;
    const int32_t v0 = (c < n && kk < k) ? limb::split_value<MODE>(B[off], sum ? B2[off] : T(0), M) : 0;
    const int32_t v1 = (c < n && kk + 1 < k) ? limb::split_value<MODE>(B[off + 1], sum ? B2[off + 1] : T(0), M) : 0;
    __half d0[PLANES], d1[PLANES];
    digits6(v0, d0);
    digits6(v1, d1);
    const size_t plane = (size_t)Npad * Kpad;
#pragma unroll
    for (int l = 0; l < PLANES; l++)
        *reinterpret_cast<__half2 *>(D + l * plane + (size_t)c * Kpad + kk) = __halves2half2(d0[l], d1[l]);
}

}  // namespace kara
