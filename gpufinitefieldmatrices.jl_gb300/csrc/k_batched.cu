// k_batched.cu -- batched uneven instances: many independent products and
// PLUQs, each with its own sizes and modulus, in three launches captured in
// one CUDA graph:
//   k_split_batched   digit planes of every product operand (one launch over all)
//   k_gemm_grouped    persistent tcgen05 GEMM over the output tiles of every product;
//                     the digit count L (1..4) of each instance is a runtime value
//                     and each instance has its own TMA descriptors in global memory
//   k_pluq_batched    persistent PLUQ, a CTA per instance (batched_pluq.cuh)
// The product path is the limb GEMM of gemm_limb.cuh with per-tile instance
// parameters; the PLUQ path follows pluq_gpu_kernel step for step.
#include "batched_pluq.cuh"
#include "gemm_limb.cuh"
#include "limb_host.h"

#include <algorithm>
#include <numeric>
#include <vector>

namespace batched {

using namespace limb;

struct MMInst {
    int m, n, L, kblocks, mtiles, ntiles, chunk_kb, Mpad, Npad, fast;
    int32_t W[MAX_SHIFTS];       // 2^(bits s) mod N
    int64_t N;
    uint64_t minv;
    int64_t bias;
    double *C;
    int64_t ldc;
    // fast epilogue (fast != 0: odd N, one exact chunk whose shift sums stay within 2^22):
    // the sums are read by adding 1.5 * 2^23 in fp32 (in pairs when fast == 2, the 7-bit
    // digits' case; limb::fast_pair) and reduced by one 32-bit Montgomery step
    uint32_t ninv;               // -N^-1 mod 2^32
    int32_t Wm[MAX_SHIFTS];      // 2^(bits s) * 2^32 mod N
    int64_t fbias;               // the initial value (limb::fast_consts)
};

struct WorkItem {
    int inst, tm, tn, pad_;
};

struct SplitJob {
    const double *src;
    int64_t ld;
    __half *dst;
    int rows, cols;              // operand extent: A is m x k, B is k x n
    int prow, kpad;              // digit rows per plane (Mpad or Npad) and padded K
    int L, is_b;
    int64_t N;
    uint64_t minv;
    int64_t blk0;                // first block of this job
    int bits, pad_;              // digit width (7 or 8)
};

constexpr int G_STAGES = 2;
constexpr int G_STAGE_BYTES = 4 * (A_TILE + B_TILE);
constexpr int G_SMEM_BYTES = G_STAGES * G_STAGE_BYTES + 1024;
constexpr int G_TMEM_COLS = 512;

// ---------------------------------------------------------------------------
// digit split of every product operand
// ---------------------------------------------------------------------------
// A block takes one chunk: up to SPLIT_CHUNK consecutive work units (32 x 32 tiles
// of A, or 256 runs of 8 K values of B) of one operand, found with a single table load.
constexpr int SPLIT_CHUNK = 8;
constexpr int SPLIT_B_RUN = 8;   // K values of B per thread and unit (one 16-byte store per plane)

struct SplitChunk {
    int job, local0, count, pad_;
};

// the L digit planes of n consecutive centred values, packed: one store per plane
template <int L, int NV>
__device__ __forceinline__ void store_digit_run(const int32_t (&c)[NV], __half *dst, size_t plane, int bits) {
    __half d[NV][L];
#pragma unroll
    for (int i = 0; i < NV; i++) digits<L>(c[i], d[i], bits);
#pragma unroll
    for (int l = 0; l < L; l++) {
        __half2 h[NV / 2];
#pragma unroll
        for (int i = 0; i < NV / 2; i++) h[i] = __halves2half2(d[2 * i][l], d[2 * i + 1][l]);
        if (NV == 8)
            *reinterpret_cast<int4 *>(dst + l * plane) = *reinterpret_cast<const int4 *>(h);
        else
            *reinterpret_cast<uint2 *>(dst + l * plane) = *reinterpret_cast<const uint2 *>(h);
    }
}

// A operand: 32 x 32 tiles transposed through shared memory.  The next unit's
// values are loaded before the current one is converted and stored, so a
// thread keeps loads in flight across the units of its chunk.  After the
// transpose a thread writes 4 consecutive K values of one row (8 bytes per plane).
template <int L>
__device__ __forceinline__ void split_a_chunk(const SplitJob &J, const SplitChunk &ch, int32_t (*tile)[33]) {
    const int kt = J.kpad / 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int wr = threadIdx.x >> 3, wk = 4 * (threadIdx.x & 7);   // the row and K run this thread writes
    const ModN M{J.N, J.minv};
    const size_t plane = (size_t)J.prow * J.kpad;
    double cur[4], nxt[4];
    bool okc[4], okn[4];
    auto load = [&](int64_t local, double (&v)[4], bool (&ok)[4]) {
        const int64_t r0 = (local / kt) * 32, k0 = (local % kt) * 32;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int64_t kk = k0 + ty + 8 * i, r = r0 + tx;
            ok[i] = r < J.rows && kk < J.cols;
            v[i] = ok[i] ? J.src[r + kk * J.ld] : 0.0;
        }
    };
    load(ch.local0, cur, okc);
    for (int u = 0; u < ch.count; u++) {
        const int64_t local = (int64_t)ch.local0 + u;
        if (u + 1 < ch.count) load(local + 1, nxt, okn);
        const int64_t r0 = (local / kt) * 32, k0 = (local % kt) * 32;
        // tile[kk][r]: the centred value of A[r0 + r][k0 + kk]
#pragma unroll
        for (int i = 0; i < 4; i++) tile[ty + 8 * i][tx] = okc[i] ? split_value<SPLIT_CENTRED>(cur[i], 0.0, M) : 0;
        __syncthreads();
        int32_t c[4];
#pragma unroll
        for (int j = 0; j < 4; j++) c[j] = tile[wk + j][wr];
        store_digit_run<L, 4>(c, J.dst + (size_t)(r0 + wr) * J.kpad + k0 + wk, plane, J.bits);
        __syncthreads();   // the tile is reused by the next unit
#pragma unroll
        for (int i = 0; i < 4; i++) {
            cur[i] = nxt[i];
            okc[i] = okn[i];
        }
    }
}

// B operand: a unit is 256 runs of SPLIT_B_RUN consecutive K values of one column (the
// operand is column-major: contiguous reads, one 16-byte store per plane); the next
// unit's run is loaded ahead.
template <int L>
__device__ __forceinline__ void split_b_chunk(const SplitJob &J, const SplitChunk &ch) {
    const int64_t rpc = J.kpad / SPLIT_B_RUN;   // runs per column
    const int64_t total = rpc * J.prow;
    const ModN M{J.N, J.minv};
    const int k = J.rows, n = J.cols;
    const size_t plane = (size_t)J.prow * J.kpad;
    double cv[SPLIT_B_RUN], nv[SPLIT_B_RUN];
    auto load = [&](int64_t local, double (&v)[SPLIT_B_RUN]) {
        const int64_t idx = local * 256 + threadIdx.x;
        const int64_t c = idx / rpc;
        const int64_t kk = (idx - c * rpc) * SPLIT_B_RUN;
        const bool colok = idx < total && c < n;
#pragma unroll
        for (int i = 0; i < SPLIT_B_RUN; i++) v[i] = (colok && kk + i < k) ? J.src[kk + i + c * J.ld] : 0.0;
    };
    load(ch.local0, cv);
    for (int u = 0; u < ch.count; u++) {
        const int64_t local = (int64_t)ch.local0 + u;
        const int64_t idx = local * 256 + threadIdx.x;
        if (idx >= total) return;
        if (u + 1 < ch.count) load(local + 1, nv);
        const int64_t c = idx / rpc;
        const int64_t kk = (idx - c * rpc) * SPLIT_B_RUN;
        int32_t v[SPLIT_B_RUN];
#pragma unroll
        for (int i = 0; i < SPLIT_B_RUN; i++)
            v[i] = (c < n && kk + i < k) ? split_value<SPLIT_CENTRED>(cv[i], 0.0, M) : 0;
        store_digit_run<L, SPLIT_B_RUN>(v, J.dst + (size_t)c * J.kpad + kk, plane, J.bits);
#pragma unroll
        for (int i = 0; i < SPLIT_B_RUN; i++) cv[i] = nv[i];
    }
}

__global__ void __launch_bounds__(256, 3) k_split_batched(const SplitJob *__restrict__ jobs,
                                                       const SplitChunk *__restrict__ chunks) {
    __shared__ int32_t tile[32][33];
    const SplitChunk ch = chunks[blockIdx.x];
    const SplitJob J = jobs[ch.job];
    if (J.is_b) {
        switch (J.L) {
            case 1: split_b_chunk<1>(J, ch); break;
            case 2: split_b_chunk<2>(J, ch); break;
            case 3: split_b_chunk<3>(J, ch); break;
            default: split_b_chunk<4>(J, ch); break;
        }
    } else {
        switch (J.L) {
            case 1: split_a_chunk<1>(J, ch, tile); break;
            case 2: split_a_chunk<2>(J, ch, tile); break;
            case 3: split_a_chunk<3>(J, ch, tile); break;
            default: split_a_chunk<4>(J, ch, tile); break;
        }
    }
}

// ---------------------------------------------------------------------------
// grouped limb GEMM over the output tiles of every product
// ---------------------------------------------------------------------------
__device__ __forceinline__ void tmap_acquire(const CUtensorMap *map) {
    asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(map) : "memory");
}

__device__ __forceinline__ int64_t reduce_inst(int64_t acc, const MMInst &I) {
    return (int64_t)gffm_dev::barrett64((uint64_t)(acc + I.bias), (uint64_t)I.N, I.minv);
}

// epilogue warps of the grouped GEMM: four per TMEM lane quadrant, 16 columns each
constexpr int G_EPI_WARPS = 16;
constexpr int G_THREADS = 64 + 32 * G_EPI_WARPS;

// one tile's drain and store by one epilogue warp (32 rows x 16 columns)
template <bool FAST>
__device__ __forceinline__ bool grouped_tile(const MMInst &I, const WorkItem &it, uint32_t tq, int quad, int part,
                                             int lane, uint64_t *acc_full_bar, uint64_t *acc_empty_bar,
                                             uint32_t &acc_phase, int *err, volatile int &abort_s) {
    const int nshift = 2 * I.L - 1;
    int64_t acc[16];
#pragma unroll
    for (int j = 0; j < 16; j++) acc[j] = FAST ? I.fbias : 0;
    int chunk = 0;
    for (int kb0 = 0; kb0 < I.kblocks; kb0 += I.chunk_kb, chunk++) {
        if (!gffm_dev::mbar_wait(acc_full_bar, acc_phase)) {
            atomicOr(err, 8);
            abort_s = 1;
            return false;
        }
        gffm_dev::tc_fence_after();
        if (FAST && I.fast == 2) {
            // the shifts in pairs, 8 columns of both at a time
            for (int s = 0; s < nshift; s += 2) {
                const int w = I.Wm[s];
                if (s + 1 < nshift) {
#pragma unroll
                    for (int h = 0; h < 16; h += 8) {
                        uint32_t v[8], u[8];
                        gffm_dev::tmem_ld_32x32b_x8(tq + 64 * s + h, v);
                        gffm_dev::tmem_ld_32x32b_x8(tq + 64 * (s + 1) + h, u);
                        gffm_dev::tmem_ld_wait();
#pragma unroll
                        for (int j = 0; j < 8; j++) acc[h + j] += (int64_t)fast_pair(v[j], u[j]) * w;
                    }
                } else {
                    uint32_t v[16];
                    gffm_dev::tmem_ld_32x32b_x16(tq + 64 * s, v);
                    gffm_dev::tmem_ld_wait();
#pragma unroll
                    for (int j = 0; j < 16; j++) acc[j] += (int64_t)(int32_t)fast_bits(v[j]) * w;
                }
            }
        }
        for (int s = 0; s < (FAST && I.fast == 2 ? 0 : nshift); s++) {
            uint32_t v[16];
            gffm_dev::tmem_ld_32x32b_x16(tq + 64 * s, v);
            gffm_dev::tmem_ld_wait();
            if (FAST) {
                const int w = I.Wm[s];
#pragma unroll
                for (int j = 0; j < 16; j++) acc[j] += (int64_t)(int32_t)fast_bits(v[j]) * w;
            } else {
                const int w = I.W[s];
#pragma unroll
                for (int j = 0; j < 16; j++) acc[j] += (int64_t)__float2int_rz(__uint_as_float(v[j])) * w;
            }
        }
        gffm_dev::tc_fence_before();
        __syncwarp();
        if (lane == 0) gffm_dev::mbar_arrive(acc_empty_bar);
        acc_phase ^= 1;
        if (!FAST && (chunk & 63) == 63) {
#pragma unroll
            for (int j = 0; j < 16; j++) acc[j] = reduce_inst(acc[j], I);
        }
    }
    const int64_t row = (int64_t)it.tm * BM + quad * 32 + lane;
    const int64_t col0 = (int64_t)it.tn * BN + part * 16;
    if (row < I.m) {
        double *cb = I.C + row + col0 * I.ldc;
        const uint32_t n32 = (uint32_t)I.N;
#pragma unroll
        for (int j = 0; j < 16; j++) {
            if (col0 + j < I.n) {
                if (FAST) {
                    // x in (0, 2^32 N): t = (x + m N) / 2^32 < 2N, t = x 2^-32 mod N
                    const uint64_t x = (uint64_t)acc[j];
                    const uint32_t mq = (uint32_t)x * I.ninv;
                    uint32_t r = (uint32_t)((x + (uint64_t)mq * n32) >> 32);
                    cb[j * I.ldc] = (double)(r >= n32 ? r - n32 : r);
                } else {
                    cb[j * I.ldc] = (double)reduce_inst(acc[j], I);
                }
            }
        }
    }
    return true;
}

__global__ void __launch_bounds__(G_THREADS, 1)
    k_gemm_grouped(const MMInst *__restrict__ insts, const WorkItem *__restrict__ items, int nitems,
                   const CUtensorMap *__restrict__ tmaps, int *err) {
    extern __shared__ uint8_t dsmem_raw[];
    __shared__ uint64_t full_bar[G_STAGES];
    __shared__ uint64_t empty_bar[G_STAGES];
    __shared__ uint64_t acc_full_bar, acc_empty_bar, drain_bar;
    __shared__ uint32_t tmem_base_s;
    __shared__ int abort_sh;
    volatile int &abort_s = abort_sh;

    uint8_t *smem = (uint8_t *)(((uintptr_t)dsmem_raw + 1023) & ~(uintptr_t)1023);
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;

    if (threadIdx.x == 0) {
        for (int s = 0; s < G_STAGES; s++) {
            gffm_dev::mbar_init(&full_bar[s], 1);
            gffm_dev::mbar_init(&empty_bar[s], 1);
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
            int last_inst = -1;
            for (int t = blockIdx.x; t < nitems && !abort_s; t += gridDim.x) {
                const WorkItem it = items[t];
                const MMInst &I = insts[it.inst];
                const int L = I.L;
                const CUtensorMap *tmA = tmaps + 2 * it.inst;
                const CUtensorMap *tmB = tmA + 1;
                if (it.inst != last_inst) {
                    tmap_acquire(tmA);
                    tmap_acquire(tmB);
                    last_inst = it.inst;
                }
                const uint32_t bytes = (uint32_t)L * (A_TILE + B_TILE);
                for (int kb = 0; kb < I.kblocks; kb++) {
                    if (!gffm_dev::mbar_wait(&empty_bar[stage], phase ^ 1)) {
                        atomicOr(err, 1);
                        abort_s = 1;
                        break;
                    }
                    if (abort_s) break;
                    uint8_t *sa = smem + stage * G_STAGE_BYTES;
                    uint8_t *sb = sa + 4 * A_TILE;
                    gffm_dev::mbar_arrive_expect_tx(&full_bar[stage], bytes);
                    for (int l = 0; l < L; l++)
                        gffm_dev::tma_load_2d(sa + l * A_TILE, tmA, &full_bar[stage], kb * BK, l * I.Mpad + it.tm * BM);
                    for (int l = 0; l < L; l++)
                        gffm_dev::tma_load_2d(sb + l * B_TILE, tmB, &full_bar[stage], kb * BK, l * I.Npad + it.tn * BN);
                    issued_mask |= 1u << stage;
                    issued_parity_mask = (issued_parity_mask & ~(1u << stage)) | (phase << stage);
                    if (++stage == G_STAGES) {
                        stage = 0;
                        phase ^= 1;
                    }
                }
            }
            if (abort_s) {
                for (int s = 0; s < G_STAGES; s++)
                    if (issued_mask & (1u << s)) gffm_dev::mbar_wait(&full_bar[s], (issued_parity_mask >> s) & 1);
            }
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer ----------------
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0, acc_phase = 0;
            bool issued_any = false;
            for (int t = blockIdx.x; t < nitems && !abort_s; t += gridDim.x) {
                const WorkItem it = items[t];
                const MMInst &I = insts[it.inst];
                const int L = I.L;
                const uint32_t idesc_full = gffm_dev::idesc_f16_f32(BM, BN * L);
                const uint32_t idesc_lo = gffm_dev::idesc_f16_f32(BM, BN * (L > 1 ? L - 1 : 1));
                const uint32_t idesc_one = gffm_dev::idesc_f16_f32(BM, BN);
                for (int kb0 = 0; kb0 < I.kblocks && !abort_s; kb0 += I.chunk_kb) {
                    const int kb1 = min(kb0 + I.chunk_kb, I.kblocks);
                    if (!gffm_dev::mbar_wait(&acc_empty_bar, acc_phase ^ 1)) {
                        atomicOr(err, 2);
                        abort_s = 1;
                        break;
                    }
                    gffm_dev::tc_fence_after();
                    for (int kb = kb0; kb < kb1; kb++) {
                        if (!gffm_dev::mbar_wait(&full_bar[stage], phase)) {
                            atomicOr(err, 4);
                            abort_s = 1;
                            break;
                        }
                        gffm_dev::tc_fence_after();
                        const uint32_t sa = gffm_dev::smem_u32(smem + stage * G_STAGE_BYTES);
                        const uint32_t sb = sa + 4 * A_TILE;
#pragma unroll
                        for (int kk = 0; kk < BK / 16; kk++) {
                            const uint64_t bdesc = gffm_dev::umma_desc_sw128(sb + kk * 32);
                            if (kb == kb0 && kk == 0) {
                                gffm_dev::mma_f16(tmem, gffm_dev::umma_desc_sw128(sa + kk * 32), bdesc, idesc_full, 0);
                                for (int i = 1; i < L; i++) {
                                    const uint64_t adesc = gffm_dev::umma_desc_sw128(sa + i * A_TILE + kk * 32);
                                    gffm_dev::mma_f16(tmem + 64 * i, adesc, bdesc, idesc_lo, 1);
                                    gffm_dev::mma_f16(tmem + 64 * (i + L - 1), adesc,
                                                      gffm_dev::umma_desc_sw128(sb + (L - 1) * B_TILE + kk * 32),
                                                      idesc_one, 0);
                                }
                            } else {
                                for (int i = 0; i < L; i++)
                                    gffm_dev::mma_f16(tmem + 64 * i, gffm_dev::umma_desc_sw128(sa + i * A_TILE + kk * 32),
                                                      bdesc, idesc_full, 1);
                            }
                        }
                        issued_any = true;
                        gffm_dev::mma_commit(&empty_bar[stage]);
                        if (++stage == G_STAGES) {
                            stage = 0;
                            phase ^= 1;
                        }
                    }
                    if (abort_s) break;
                    gffm_dev::mma_commit(&acc_full_bar);
                    acc_phase ^= 1;
                }
            }
            if (abort_s && issued_any) {
                gffm_dev::mma_commit(&drain_bar);
                gffm_dev::mbar_wait(&drain_bar, 0);
            }
        }
    } else {
        // ---------------- epilogue ----------------
        const int quad = warp & 3;
        const int part = (warp - 2) >> 2;   // which 16 of the tile's 64 columns
        const uint32_t tq = tmem + ((uint32_t)(quad * 32) << 16) + 16 * part;
        uint32_t acc_phase = 0;
        for (int t = blockIdx.x; t < nitems; t += gridDim.x) {
            const WorkItem it = items[t];
            const MMInst I = insts[it.inst];
            const bool ok = I.fast ? grouped_tile<true>(I, it, tq, quad, part, lane, &acc_full_bar, &acc_empty_bar,
                                                        acc_phase, err, abort_s)
                                   : grouped_tile<false>(I, it, tq, quad, part, lane, &acc_full_bar, &acc_empty_bar,
                                                         acc_phase, err, abort_s);
            if (!ok || abort_s) break;
        }
    }

    gffm_dev::tc_fence_before();
    __syncthreads();
    gffm_dev::tc_fence_after();
    if (warp == 1) gffm_dev::tmem_dealloc(tmem, G_TMEM_COLS);
}

}  // namespace batched

#include "batched_steps.cuh"

// ---------------------------------------------------------------------------
// host: plans
// ---------------------------------------------------------------------------
struct gffm_batch_plan_s {
    int device = 0;
    void *mem = nullptr;
    size_t mem_bytes = 0;
    int n_mm = 0, n_pq = 0, nitems = 0, njobs = 0;
    int64_t split_blocks = 0;
    int gemm_grid = 0, pq_grid = 0, pq_nb = 0, pq_rcap = 0;
    size_t pq_smem = 0;
    batched::MMInst *d_mm = nullptr;
    batched::WorkItem *d_items = nullptr;
    CUtensorMap *d_tmaps = nullptr;
    batched::SplitJob *d_jobs = nullptr;
    batched::SplitChunk *d_chunks = nullptr;
    int64_t nchunks = 0;
    batched::PQInst *d_pq = nullptr;
    int *d_order = nullptr, *d_next = nullptr;
    int32_t *d_tmp = nullptr;
    int tmp_ldw = 4;
    // the panel-step route (batched_steps.cuh)
    int n_step = 0, step_grid = 0, step_misc_grid = 0, trail_grid = 0;
    batched::StepArgs step{};
    // the step-route instances in groups, each factored by its own chain of step launches on
    // its own graph branch, so that one group's launches fill the other's step tails
    struct StepGroup {
        batched::StepArgs args;                 // order, live and counters of the group
        int n_steps = 0, members = 0;
        std::vector<int> live;                  // per step: running instances of the group
        std::vector<int> rcap, smem, grid3;     // per step: panel height, shared memory, CTAs (0: 2 per SM)
        std::vector<int> per_sm;                // per step: panel CTAs per SM (2, 3 or 4)
        std::vector<int> items0;                // per step: first work item (n_steps + 1 entries)
    };
    std::vector<StepGroup> groups;
    batched::WorkItem *d_step_items = nullptr;
    int *d_counters = nullptr;                  // the PLUQ kernels' scheduling counters
    int n_counters = 0;
    cudaGraphExec_t exec = nullptr;
    struct ZeroK {
        double *C;
        int64_t ldc, m, n;
    };
    std::vector<ZeroK> zero_k;   // products with an empty inner dimension: C = 0
    // PLUQ instances taller than the persistent kernel takes: factored after the graph by
    // the single-matrix elimination, their swap stacks staged through these host buffers
    std::vector<gffm_batch_desc> tall;
    std::vector<int64_t> h_rows, h_cols;
};

namespace {

using gffm::set_error;

#define PLAN_CUDA(call)                                 \
    do {                                                \
        cudaError_t e__ = (call);                       \
        if (e__ != cudaSuccess) {                       \
            free_plan(p);                               \
            return gffm::cuda_error(e__, #call);        \
        }                                               \
    } while (0)

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// PLUQ instances with more rows run after the graph on the single-matrix elimination
constexpr int64_t kGraphPluqMaxRows = 1024;
// the step route's panel kernel at four CTAs per SM where shared memory allows (64 registers)
constexpr bool kStepFourPerSM = true;

int check_desc(const gffm_batch_desc &d, int64_t i) {
    if (d.op != GFFM_BATCH_MATMUL && d.op != GFFM_BATCH_PLUQ)
        return set_error(GFFM_ERR_ARG, "instance %lld: unknown op %lld", (long long)i, (long long)d.op);
    if (d.N < 2 || d.N >= (int64_t(1) << 26))
        return set_error(GFFM_ERR_MODULUS, "instance %lld: the batched path needs 2 <= N < 2^26 (got %lld)",
                         (long long)i, (long long)d.N);
    if (d.m < 0 || d.n < 0 || d.k < 0) return set_error(GFFM_ERR_ARG, "instance %lld: negative size", (long long)i);
    if (d.op == GFFM_BATCH_MATMUL) {
        int st = limb::check_args(d.m, d.n, d.k, d.lda, d.ldb, d.ldc, d.N);
        if (st) return st;
        if (d.m > 0 && d.n > 0 && (!d.C || (d.k > 0 && (!d.A || !d.B))))
            return set_error(GFFM_ERR_ARG, "instance %lld: null data pointer", (long long)i);
    } else {
        if (d.n > (int64_t(1) << 20)) return set_error(GFFM_ERR_ARG, "instance %lld: n above 2^20", (long long)i);
        if (d.lda < std::max<int64_t>(d.m, 1) || d.ldc < std::max<int64_t>(d.m, 1) || d.ldl < std::max<int64_t>(d.m, 1))
            return set_error(GFFM_ERR_ARG, "instance %lld: leading dimension smaller than m", (long long)i);
        if (d.l_cols < 1 || d.l_cols > (int64_t(1) << 20))
            return set_error(GFFM_ERR_ARG, "instance %lld: l_cols out of range", (long long)i);
        if (!d.info || (d.m > 0 && d.n > 0 && (!d.A || !d.C || !d.L || !d.row_swaps || !d.col_swaps)))
            return set_error(GFFM_ERR_ARG, "instance %lld: null pointer", (long long)i);
    }
    return GFFM_OK;
}

struct Carve {
    size_t off = 0;
    size_t take(size_t bytes, size_t align = 256) {
        off = align_up(off, align);
        size_t o = off;
        off += bytes;
        return o;
    }
};

int build_graph(gffm_batch_plan p, bool overlap) {
    using namespace batched;
    cudaStream_t s0, s1 = nullptr;
    GFFM_CUDA(cudaStreamCreateWithFlags(&s0, cudaStreamNonBlocking));
    cudaGraph_t graph = nullptr;
    int st = GFFM_OK;
    cudaEvent_t fork = nullptr, join = nullptr;
    // the step-route groups' branches
    cudaEvent_t gfork = nullptr;
    cudaEvent_t gjoin[batched::ST_MAX_GROUPS] = {};
    cudaStream_t gstreams[batched::ST_MAX_GROUPS] = {};
    auto fail = [&](cudaError_t e, const char *what) {
        if (st == GFFM_OK && e != cudaSuccess) st = gffm::cuda_error(e, what);
    };
    fail(cudaStreamBeginCapture(s0, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
    if (!st) {
        cudaStream_t pq_stream = s0;
        if (overlap && p->n_mm > 0 && p->n_pq > 0) {
            fail(cudaStreamCreateWithFlags(&s1, cudaStreamNonBlocking), "cudaStreamCreate");
            fail(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming), "cudaEventCreate");
            fail(cudaEventCreateWithFlags(&join, cudaEventDisableTiming), "cudaEventCreate");
            fail(cudaEventRecord(fork, s0), "cudaEventRecord");
            fail(cudaStreamWaitEvent(s1, fork, 0), "cudaStreamWaitEvent");
            pq_stream = s1;
        }
        if (p->n_pq > 0) {
            fail(cudaMemsetAsync(p->d_counters, 0, sizeof(int) * p->n_counters, pq_stream), "cudaMemsetAsync");
            if (p->n_step > 0) {
                const size_t conv_smem = (size_t)8 * 32 * 33 * 4;
                const int G = (int)p->groups.size();
                if (G > 1) {
                    fail(cudaEventCreateWithFlags(&gfork, cudaEventDisableTiming), "cudaEventCreate");
                    fail(cudaEventRecord(gfork, pq_stream), "cudaEventRecord");
                }
                for (int gi = 0; gi < G; gi++) {
                    const auto &grp = p->groups[gi];
                    cudaStream_t gs = pq_stream;
                    if (gi > 0) {
                        fail(cudaStreamCreateWithFlags(&gstreams[gi], cudaStreamNonBlocking), "cudaStreamCreate");
                        fail(cudaStreamWaitEvent(gstreams[gi], gfork, 0), "cudaStreamWaitEvent");
                        gs = gstreams[gi];
                    }
                    // the group's working copies, its steps, then its outputs
                    const int gcount = (int)grp.members;
                    k_pq_prologue<<<std::max(1, std::min(gcount, p->step_misc_grid)), PQ_THREADS, conv_smem, gs>>>(
                        grp.args, gcount);
                    fail(cudaGetLastError(), "k_pq_prologue");
                    for (int s = 0; s < grp.n_steps; s++) {
                        StepArgs sa = grp.args;
                        sa.rcap = grp.rcap[s];
                        if (grp.per_sm[s] == 4) {
                            k_pq_panel<4><<<std::max(1, std::min(grp.live[s], grp.grid3[s])), PQ_THREADS, grp.smem[s],
                                            gs>>>(sa, s);
                        } else if (grp.grid3[s]) {
                            k_pq_panel<3><<<std::max(1, std::min(grp.live[s], grp.grid3[s])), PQ_THREADS, grp.smem[s],
                                            gs>>>(sa, s);
                        } else {
                            k_pq_panel<2><<<std::max(1, std::min(grp.live[s], p->step_grid)), PQ_THREADS, grp.smem[s],
                                            gs>>>(sa, s);
                        }
                        fail(cudaGetLastError(), "k_pq_panel");
                        const int i0 = grp.items0[s], ni = grp.items0[s + 1] - i0;
                        if (ni > 0) {
                            k_gemm_trail<<<std::min(ni, p->trail_grid), G_THREADS, ST_SMEM_BYTES, gs>>>(
                                sa, s, p->d_step_items + i0, ni, gffm::device_error_flag());
                            fail(cudaGetLastError(), "k_gemm_trail");
                        }
                    }
                    k_pq_finish<<<std::max(1, std::min(gcount, p->step_misc_grid)), PQ_THREADS,
                                  conv_smem + sizeof(int) * p->pq_rcap, gs>>>(grp.args, gcount);
                    fail(cudaGetLastError(), "k_pq_finish");
                    if (gi > 0) {
                        fail(cudaEventCreateWithFlags(&gjoin[gi], cudaEventDisableTiming), "cudaEventCreate");
                        fail(cudaEventRecord(gjoin[gi], gs), "cudaEventRecord");
                        fail(cudaStreamWaitEvent(pq_stream, gjoin[gi], 0), "cudaStreamWaitEvent");
                    }
                }
            }
            PQArgs a;
            a.inst = p->d_pq;
            a.order = p->d_order;
            a.count = p->n_pq;
            a.nb = p->pq_nb;
            a.rcap = p->pq_rcap;
            a.next = p->d_next;
            a.tmp = p->d_tmp;
            a.tmp_ldw = p->tmp_ldw;
            a.flags = p->step.flags;
            k_pluq_batched<<<p->pq_grid, PQ_THREADS, p->pq_smem, pq_stream>>>(a);
            fail(cudaGetLastError(), "k_pluq_batched");
        }
        for (const auto &z : p->zero_k)
            fail(cudaMemset2DAsync(z.C, (size_t)z.ldc * 8, 0, (size_t)z.m * 8, (size_t)z.n, s0), "cudaMemset2DAsync");
        if (p->n_mm > 0 && p->nitems > 0) {
            k_split_batched<<<(unsigned)p->nchunks, 256, 0, s0>>>(p->d_jobs, p->d_chunks);
            fail(cudaGetLastError(), "k_split_batched");
            k_gemm_grouped<<<p->gemm_grid, G_THREADS, G_SMEM_BYTES, s0>>>(p->d_mm, p->d_items, p->nitems, p->d_tmaps,
                                                                          gffm::device_error_flag());
            fail(cudaGetLastError(), "k_gemm_grouped");
        }
        if (s1) {
            fail(cudaEventRecord(join, s1), "cudaEventRecord");
            fail(cudaStreamWaitEvent(s0, join, 0), "cudaStreamWaitEvent");
        }
        cudaError_t e = cudaStreamEndCapture(s0, &graph);
        fail(e, "cudaStreamEndCapture");
    }
    if (!st) fail(cudaGraphInstantiate(&p->exec, graph, 0), "cudaGraphInstantiate");
    if (graph) cudaGraphDestroy(graph);
    if (fork) cudaEventDestroy(fork);
    if (join) cudaEventDestroy(join);
    if (gfork) cudaEventDestroy(gfork);
    for (int gi = 0; gi < batched::ST_MAX_GROUPS; gi++) {
        if (gjoin[gi]) cudaEventDestroy(gjoin[gi]);
        if (gstreams[gi]) cudaStreamDestroy(gstreams[gi]);
    }
    if (s1) cudaStreamDestroy(s1);
    cudaStreamDestroy(s0);
    return st;
}

void free_plan(gffm_batch_plan p) {
    if (!p) return;
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->mem) cudaFree(p->mem);
    delete p;
}

int create(const gffm_batch_desc *descs, int64_t count, const gffm_batch_tuning *tuning, gffm_batch_plan *out) {
    using namespace batched;
    if (!out) return set_error(GFFM_ERR_ARG, "plan is NULL");
    *out = nullptr;
    if (count < 0 || (count > 0 && !descs)) return set_error(GFFM_ERR_ARG, "bad descriptor array");
    if (count > (int64_t(1) << 24)) return set_error(GFFM_ERR_ARG, "too many instances");
    for (int64_t i = 0; i < count; i++) {
        int st = check_desc(descs[i], i);
        if (st) return st;
    }
    int st = gffm::check_device();
    if (st) return st;
    gffm_batch_tuning tu{};
    if (tuning) tu = *tuning;
    if (tu.pluq_panel != 0 && tu.pluq_panel != 8 && tu.pluq_panel != 16 && tu.pluq_panel != 32)
        return set_error(GFFM_ERR_ARG, "pluq_panel must be 0, 8, 16 or 32");
    if (tu.gemm_ctas < 0 || tu.pluq_ctas < 0) return set_error(GFFM_ERR_ARG, "negative grid size");
    if (tu.digit_bits != 0 && tu.digit_bits != 7 && tu.digit_bits != 8)
        return set_error(GFFM_ERR_ARG, "digit_bits must be 0, 7 or 8");

    auto *p = new gffm_batch_plan_s();
    PLAN_CUDA(cudaGetDevice(&p->device));
    const int sms = gffm::sm_count();

    std::vector<int64_t> mm_ids, pq_ids;
    for (int64_t i = 0; i < count; i++) {
        const gffm_batch_desc &d = descs[i];
        if (d.op == GFFM_BATCH_PLUQ && d.m > kGraphPluqMaxRows && d.n > 0) {
            p->tall.push_back(d);
            continue;
        }
        if (d.m == 0 || d.n == 0) {
            if (d.op == GFFM_BATCH_PLUQ) pq_ids.push_back(i);   // still reports its info
            continue;
        }
        (d.op == GFFM_BATCH_MATMUL ? mm_ids : pq_ids).push_back(i);
    }
    p->n_mm = (int)mm_ids.size();
    p->n_pq = (int)pq_ids.size();

    // ---- layout of the one device allocation ----
    Carve cv;
    const size_t o_mm = cv.take(sizeof(MMInst) * std::max(1, p->n_mm));
    const size_t o_tm = cv.take(sizeof(CUtensorMap) * 2 * std::max(1, p->n_mm), 128);
    std::vector<MMInst> mm(p->n_mm);
    std::vector<WorkItem> items;
    std::vector<SplitJob> jobs;
    std::vector<size_t> o_da(p->n_mm), o_db(p->n_mm);
    std::vector<limb::Layout> lay(p->n_mm);
    int64_t blk = 0;
    for (int q = 0; q < p->n_mm; q++) {
        const gffm_batch_desc &d = descs[mm_ids[q]];
        MMInst &I = mm[q];
        // digit width: the tuning's, else whichever needs fewer digits (7 on a tie)
        const int bits = tu.digit_bits ? tu.digit_bits
                                       : (limb::limbs_for_bits(d.N, 8) < limb::limbs_for(d.N) ? 8 : 7);
        lay[q] = limb::layout_bits(d.m, d.n, d.k, d.N, bits);
        const limb::Layout &g = lay[q];
        I.m = (int)d.m;
        I.n = (int)d.n;
        I.L = g.L;
        I.kblocks = (int)(d.k > 0 ? g.Kpad / BK : 0);
        I.mtiles = (int)((d.m + BM - 1) / BM);
        I.ntiles = (int)((d.n + BN - 1) / BN);
        I.chunk_kb = limb::chunk_kblocks(g);
        I.Mpad = (int)g.Mpad;
        I.Npad = (int)g.Npad;
        I.N = d.N;
        I.minv = ~uint64_t(0) / (uint64_t)d.N;
        I.bias = d.N * (((int64_t(1) << 60) + d.N - 1) / d.N);
        int64_t w = 1 % d.N;
        for (int sft = 0; sft < MAX_SHIFTS; sft++) {
            I.W[sft] = (int32_t)w;
            w = (w * (g.bits == 8 ? 256 : 128)) % d.N;
        }
        // the fast epilogue: odd N, one exact chunk, shift sums within 2^22
        I.fast = 0;
        I.ninv = 0;
        I.fbias = 0;
        if ((d.N & 1) && I.kblocks <= I.chunk_kb &&
            (int64_t)I.kblocks * BK * g.L * (int64_t(1) << (2 * g.bits - 2)) <= (int64_t(1) << 22)) {
            limb::fast_consts(d.N, g.L, g.bits, g.bits == 7, &I.ninv, I.Wm, &I.fbias);
            I.fast = g.bits == 7 ? 2 : 1;   // 2: the drain reads the shifts in pairs
        } else {
            for (int sft = 0; sft < MAX_SHIFTS; sft++) I.Wm[sft] = 0;
        }
        I.C = d.C;
        I.ldc = d.ldc;
        if (d.k == 0) p->zero_k.push_back({d.C, d.ldc, d.m, d.n});
        o_da[q] = cv.take(g.a_bytes, 1024);
        o_db[q] = cv.take(g.b_bytes, 1024);
    }
    const size_t o_pq = cv.take(sizeof(PQInst) * std::max(1, p->n_pq));
    const size_t o_order = cv.take(sizeof(int) * std::max(1, p->n_pq));
    std::vector<PQInst> pq(p->n_pq);
    std::vector<size_t> o_w(p->n_pq), o_lw(p->n_pq);
    int rcap = 4;
    for (int q = 0; q < p->n_pq; q++) {
        const gffm_batch_desc &d = descs[pq_ids[q]];
        PQInst &I = pq[q];
        I.m = (int)d.m;
        I.n = (int)d.n;
        I.l_cols = (int)d.l_cols;
        I.lsw = (int)std::min<int64_t>((d.m + 31) / 32 * 32, d.l_cols);
        I.M.n = (uint32_t)d.N;
        I.M.minv = ~uint64_t(0) / (uint64_t)d.N;
        I.A = d.A;
        I.lda = d.lda;
        I.U = d.C;
        I.ldu = d.ldc;
        I.L = d.L;
        I.ldl = d.ldl;
        I.ldw = (int)align_up((size_t)std::max<int64_t>(d.n, 1), 4);
        I.lwc = (int)std::min<int64_t>(d.l_cols, d.n);
        I.ldlw = (int)align_up((size_t)std::max(I.lwc, 1), 4);
        I.pad_ = 0;
        I.row_swaps = d.row_swaps;
        I.col_swaps = d.col_swaps;
        I.info = d.info;
        o_w[q] = cv.take((size_t)std::max<int64_t>(d.m, 1) * I.ldw * 4);
        o_lw[q] = cv.take((size_t)std::max<int64_t>(d.m, 1) * I.ldlw * 4);
        rcap = std::max(rcap, (int)align_up((size_t)d.m, 4));
        p->tmp_ldw = std::max(p->tmp_ldw, I.ldw);
    }
    // ---- the panel-step route (batched_steps.cuh): square PLUQs of n = 32 k >= 64 rows, an odd
    // prime, L at least n columns wide; under the default panel tuning only ----
    std::vector<int> st_q;   // PLUQ instance indices, largest first
    if (tu.pluq_panel == 0)
        for (int q = 0; q < p->n_pq; q++) {
            const gffm_batch_desc &d = descs[pq_ids[q]];
            if (d.m == d.n && d.n >= 64 && d.n % ST_NB == 0 && (d.N & 1) && d.l_cols >= d.n) st_q.push_back(q);
        }
    std::stable_sort(st_q.begin(), st_q.end(), [&](int x, int y) { return pq[x].n > pq[y].n; });
    p->n_step = (int)st_q.size();
    std::vector<StepInst> stv(p->n_step);
    std::vector<size_t> o_src(p->n_step), o_id(p->n_step), o_u12(p->n_step), o_nr(p->n_step), o_ad(p->n_step),
        o_bd(p->n_step);
    for (int j = 0; j < p->n_step; j++) {
        const int q = st_q[j];
        const gffm_batch_desc &d = descs[pq_ids[q]];
        StepInst &J = stv[j];
        J.pq = q;
        J.n = (int)d.n;
        J.L = limb::limbs_for(d.N);
        J.Mpad = (int)align_up((size_t)d.n - ST_NB, ST_BM);
        J.Npad = (int)align_up((size_t)d.n - ST_NB, ST_BN);
        limb::fast_consts(d.N, J.L, 7, true, &J.ninv, J.Wm, &J.fbias);
        o_src[j] = cv.take(sizeof(int) * d.n);
        o_id[j] = cv.take(sizeof(int) * d.n);
        o_u12[j] = cv.take(sizeof(int32_t) * ST_NB * d.n);
        o_nr[j] = cv.take(sizeof(int));
    }
    const size_t o_planes = align_up(cv.off, 1024);
    for (int j = 0; j < p->n_step; j++) {
        o_ad[j] = cv.take((size_t)stv[j].L * stv[j].Mpad * ST_KPAD * 2, 1024);
        o_bd[j] = cv.take((size_t)stv[j].L * stv[j].Npad * ST_KPAD * 2, 1024);
    }
    const size_t planes_bytes = cv.off > o_planes ? cv.off - o_planes : 0;
    const size_t o_steps = cv.take(sizeof(StepInst) * std::max(1, p->n_step));
    // groups: the instances dealt round-robin in size order (similar mixes of sizes)
    const int n_groups = p->n_step >= ST_GROUP_MIN ? ST_MAX_GROUPS : 1;
    std::vector<std::vector<int>> gmembers(n_groups);
    for (int j = 0; j < p->n_step; j++) gmembers[j % n_groups].push_back(j);
    p->groups.resize(p->n_step > 0 ? n_groups : 0);
    int total_steps = 0;
    for (size_t gi = 0; gi < p->groups.size(); gi++) {
        p->groups[gi].n_steps = gmembers[gi].empty() ? 0 : stv[gmembers[gi][0]].n / ST_NB;
        p->groups[gi].members = (int)gmembers[gi].size();
        total_steps += p->groups[gi].n_steps;
    }
    const size_t o_st_order = cv.take(sizeof(int) * std::max(1, p->n_step));
    const size_t o_live = cv.take(sizeof(int) * std::max(1, total_steps));
    const size_t o_stmaps = cv.take(sizeof(CUtensorMap) * 2 * std::max(1, p->n_step), 128);
    const size_t o_flags = cv.take(sizeof(int) * std::max(1, p->n_pq));
    p->n_counters = 1 + total_steps;   // the per-instance kernel's, then one per group and step
    const size_t o_counters = cv.take(sizeof(int) * p->n_counters);
    std::vector<WorkItem> st_items;
    for (size_t gi = 0; gi < p->groups.size(); gi++) {
        auto &grp = p->groups[gi];
        const auto &mem = gmembers[gi];
        for (int s = 0; s < grp.n_steps; s++) {
            int live = 0;
            while (live < (int)mem.size() && stv[mem[live]].n > ST_NB * s) live++;
            grp.live.push_back(live);
            grp.items0.push_back((int)st_items.size());
            for (int q = 0; q < live; q++) {
                const int j = mem[q];
                const int rt = stv[j].n - ST_NB * s - ST_NB;   // rows = columns of the trailing block
                for (int tm = 0; tm < (rt + ST_BM - 1) / ST_BM; tm++)
                    for (int tn = 0; tn < (rt + ST_BN - 1) / ST_BN; tn++) st_items.push_back(WorkItem{j, tm, tn, 0});
            }
        }
        grp.items0.push_back((int)st_items.size());
    }
    const size_t o_st_items = cv.take(sizeof(WorkItem) * std::max<size_t>(1, st_items.size()));
    // PLUQ grid (it sizes the per-CTA row-move buffers)
    p->pq_nb = tu.pluq_panel ? tu.pluq_panel : 32;
    p->pq_rcap = rcap;
    p->pq_smem = pq_smem_words(rcap) * 4;
    int per_sm = 1;
    if (p->n_pq > 0) {
        PLAN_CUDA(cudaFuncSetAttribute(k_pluq_batched, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p->pq_smem));
        PLAN_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pluq_batched, PQ_THREADS, p->pq_smem));
        if (per_sm < 1) {
            free_plan(p);
            return set_error(GFFM_ERR_UNSUPPORTED, "batched PLUQ panel does not fit in shared memory");
        }
    }
    p->pq_grid = std::max(1, std::min(p->n_pq, tu.pluq_ctas ? tu.pluq_ctas : per_sm * sms));
    if (p->n_step > 0) {
        int per_sm_step = 1;
        PLAN_CUDA(cudaFuncSetAttribute(k_pq_panel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p->pq_smem));
        PLAN_CUDA(cudaFuncSetAttribute(k_pq_panel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p->pq_smem));
        PLAN_CUDA(cudaFuncSetAttribute(k_pq_panel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p->pq_smem));
        PLAN_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_step, k_pq_panel<2>, PQ_THREADS, p->pq_smem));
        p->step_grid = std::max(1, per_sm_step) * sms;
        if (tu.pluq_ctas) p->step_grid = tu.pluq_ctas;
        // per group and step: the panel height of its tallest running instance (the first in
        // the group's order), the shared memory it needs, and three CTAs per SM where they fit
        for (size_t gi = 0; gi < p->groups.size(); gi++) {
            auto &grp = p->groups[gi];
            for (int s = 0; s < grp.n_steps; s++) {
                const int rc = (int)align_up((size_t)stv[gmembers[gi][0]].n - ST_NB * s, 4);
                const size_t sm = st_smem_words(rc) * 4;
                int per3 = 0, per4 = 0;
                PLAN_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per3, k_pq_panel<3>, PQ_THREADS, sm));
                PLAN_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per4, k_pq_panel<4>, PQ_THREADS, sm));
                const int k = tu.pluq_ctas ? 2 : (per4 >= 4 && kStepFourPerSM ? 4 : (per3 >= 3 ? 3 : 2));
                grp.rcap.push_back(rc);
                grp.smem.push_back((int)sm);
                grp.per_sm.push_back(k);
                grp.grid3.push_back(k >= 3 ? k * sms : 0);
                if (sm > p->pq_smem) {   // never for these layouts; kept in step with the attribute
                    PLAN_CUDA(cudaFuncSetAttribute(k_pq_panel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
                    PLAN_CUDA(cudaFuncSetAttribute(k_pq_panel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
                }
            }
        }
        p->step_misc_grid = std::max(1, std::min(p->n_step, 4 * sms));
        p->trail_grid = sms;
        PLAN_CUDA(cudaFuncSetAttribute(k_gemm_trail, cudaFuncAttributeMaxDynamicSharedMemorySize, ST_SMEM_BYTES));
    }
    const size_t o_tmp = cv.take((size_t)p->pq_grid * PQ_MAX_MOVES * p->tmp_ldw * 4);
    // work items (output tiles), largest instances first
    std::vector<int> mm_order(p->n_mm);
    std::iota(mm_order.begin(), mm_order.end(), 0);
    std::stable_sort(mm_order.begin(), mm_order.end(), [&](int a, int b) {
        return (int64_t)mm[a].L * mm[a].L * mm[a].kblocks > (int64_t)mm[b].L * mm[b].L * mm[b].kblocks;
    });
    for (int q : mm_order)
        for (int tm = 0; tm < mm[q].mtiles; tm++)
            for (int tn = 0; tn < mm[q].ntiles; tn++)
                if (mm[q].kblocks > 0) items.push_back(WorkItem{q, tm, tn, 0});
    p->nitems = (int)items.size();
    const size_t o_items = cv.take(sizeof(WorkItem) * std::max<size_t>(1, items.size()));
    const size_t o_jobs = cv.take(sizeof(SplitJob) * std::max(1, 2 * p->n_mm));
    // split work units per job: 32 x 32 tiles of A, 256 digit pairs of B
    int64_t nchunks = 0;
    for (int q = 0; q < p->n_mm; q++) {
        if (mm[q].kblocks == 0) continue;
        const limb::Layout &g = lay[q];
        const int64_t ua = (g.Kpad / 32) * (g.Mpad / 32), ub = ((g.Kpad / SPLIT_B_RUN) * g.Npad + 255) / 256;
        nchunks += (ua + SPLIT_CHUNK - 1) / SPLIT_CHUNK + (ub + SPLIT_CHUNK - 1) / SPLIT_CHUNK;
    }
    const size_t o_chunks = cv.take(sizeof(SplitChunk) * std::max<int64_t>(1, nchunks));
    p->mem_bytes = cv.off;
    cudaError_t e = cudaMalloc(&p->mem, p->mem_bytes);
    if (e != cudaSuccess) {
        free_plan(p);
        return gffm::cuda_error(e, "cudaMalloc (batched plan)");
    }
    uint8_t *base = static_cast<uint8_t *>(p->mem);
    p->d_mm = reinterpret_cast<MMInst *>(base + o_mm);
    p->d_tmaps = reinterpret_cast<CUtensorMap *>(base + o_tm);
    p->d_pq = reinterpret_cast<PQInst *>(base + o_pq);
    p->d_order = reinterpret_cast<int *>(base + o_order);
    p->d_counters = reinterpret_cast<int *>(base + o_counters);
    p->d_next = p->d_counters;
    p->d_items = reinterpret_cast<WorkItem *>(base + o_items);
    p->d_jobs = reinterpret_cast<SplitJob *>(base + o_jobs);
    p->d_chunks = reinterpret_cast<SplitChunk *>(base + o_chunks);
    p->d_tmp = reinterpret_cast<int32_t *>(base + o_tmp);

    // split jobs and TMA descriptors
    std::vector<CUtensorMap> tmaps(2 * std::max(1, p->n_mm));
    for (int q = 0; q < p->n_mm; q++) {
        const gffm_batch_desc &d = descs[mm_ids[q]];
        const limb::Layout &g = lay[q];
        __half *da = reinterpret_cast<__half *>(base + o_da[q]);
        __half *db = reinterpret_cast<__half *>(base + o_db[q]);
        if (mm[q].kblocks > 0) {
            SplitJob ja{d.A, d.lda, da, (int)d.m, (int)d.k, (int)g.Mpad, (int)g.Kpad, g.L, 0, d.N, mm[q].minv, blk,
                        g.bits, 0};
            blk += (g.Kpad / 32) * (g.Mpad / 32);
            jobs.push_back(ja);
            SplitJob jb{d.B, d.ldb, db, (int)d.k, (int)d.n, (int)g.Npad, (int)g.Kpad, g.L, 1, d.N, mm[q].minv, blk,
                        g.bits, 0};
            blk += ((g.Kpad / SPLIT_B_RUN) * g.Npad + 255) / 256;
            jobs.push_back(jb);
        }
        st = limb::encode_digit_map(&tmaps[2 * q], da, g.Kpad, (int64_t)g.L * g.Mpad, BM);
        if (!st) st = limb::encode_digit_map(&tmaps[2 * q + 1], db, g.Kpad, (int64_t)g.L * g.Npad, BN);
        if (st) {
            free_plan(p);
            return st;
        }
    }
    p->njobs = (int)jobs.size();
    p->split_blocks = blk;
    std::vector<SplitChunk> chunks;
    chunks.reserve((size_t)nchunks);
    for (size_t j = 0; j < jobs.size(); j++) {
        const int64_t units = (j + 1 < jobs.size() ? jobs[j + 1].blk0 : blk) - jobs[j].blk0;
        for (int64_t u = 0; u < units; u += SPLIT_CHUNK)
            chunks.push_back(SplitChunk{(int)j, (int)u, (int)std::min<int64_t>(SPLIT_CHUNK, units - u), 0});
    }
    p->nchunks = (int64_t)chunks.size();
    // PLUQ workspace pointers and order (largest work first)
    std::vector<int> order(p->n_pq);
    for (int q = 0; q < p->n_pq; q++) {
        pq[q].W = reinterpret_cast<int32_t *>(base + o_w[q]);
        pq[q].LW = reinterpret_cast<int32_t *>(base + o_lw[q]);
    }
    for (int j = 0; j < p->n_step; j++) {
        StepInst &J = stv[j];
        J.srcmap = reinterpret_cast<int *>(base + o_src[j]);
        J.ident = reinterpret_cast<int *>(base + o_id[j]);
        J.U12 = reinterpret_cast<int32_t *>(base + o_u12[j]);
        J.nr = reinterpret_cast<int *>(base + o_nr[j]);
        J.Ad = reinterpret_cast<__half *>(base + o_ad[j]);
        J.Bd = reinterpret_cast<__half *>(base + o_bd[j]);
    }
    std::vector<CUtensorMap> stmaps(2 * std::max(1, p->n_step));
    for (int j = 0; j < p->n_step; j++) {
        const StepInst &J = stv[j];
        st = limb::encode_digit_map_k32(&stmaps[2 * j], J.Ad, (int64_t)J.L * J.Mpad, ST_BM);
        if (!st) st = limb::encode_digit_map_k32(&stmaps[2 * j + 1], J.Bd, (int64_t)J.L * J.Npad, ST_BN);
        if (st) {
            free_plan(p);
            return st;
        }
    }
    p->step.inst = p->d_pq;
    p->step.steps = reinterpret_cast<StepInst *>(base + o_steps);
    p->step.order = reinterpret_cast<int *>(base + o_st_order);
    p->step.live = reinterpret_cast<int *>(base + o_live);
    p->step.next = p->d_counters + 1;
    p->step.flags = reinterpret_cast<int *>(base + o_flags);
    p->step.tmaps = reinterpret_cast<CUtensorMap *>(base + o_stmaps);
    p->step.rcap = p->pq_rcap;
    p->d_step_items = reinterpret_cast<WorkItem *>(base + o_st_items);
    {
        // each group's arguments: the shared ones (set above), with its own slices of the
        // order, live counts and counters
        int order_off = 0, step_off = 0;
        for (size_t gi = 0; gi < p->groups.size(); gi++) {
            auto &grp = p->groups[gi];
            grp.args = p->step;
            grp.args.order = p->step.order + order_off;
            grp.args.live = p->step.live + step_off;
            grp.args.next = p->step.next + step_off;
            order_off += (int)gmembers[gi].size();
            step_off += grp.n_steps;
        }
    }
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        const int64_t wa = (int64_t)pq[a].m * pq[a].n * std::min(pq[a].m, pq[a].n);
        const int64_t wb = (int64_t)pq[b].m * pq[b].n * std::min(pq[b].m, pq[b].n);
        return wa > wb;
    });

    p->gemm_grid = std::max(1, std::min(p->nitems, tu.gemm_ctas ? tu.gemm_ctas : sms));
    if (p->n_mm > 0) {
        PLAN_CUDA(cudaFuncSetAttribute(k_gemm_grouped, cudaFuncAttributeMaxDynamicSharedMemorySize, G_SMEM_BYTES));
    }

    // upload the metadata
    PLAN_CUDA(cudaMemcpy(p->d_mm, mm.data(), sizeof(MMInst) * mm.size(), cudaMemcpyHostToDevice));
    PLAN_CUDA(cudaMemcpy(p->d_tmaps, tmaps.data(), sizeof(CUtensorMap) * 2 * p->n_mm, cudaMemcpyHostToDevice));
    PLAN_CUDA(cudaMemcpy(p->d_items, items.data(), sizeof(WorkItem) * items.size(), cudaMemcpyHostToDevice));
    PLAN_CUDA(cudaMemcpy(p->d_jobs, jobs.data(), sizeof(SplitJob) * jobs.size(), cudaMemcpyHostToDevice));
    PLAN_CUDA(cudaMemcpy(p->d_chunks, chunks.data(), sizeof(SplitChunk) * chunks.size(), cudaMemcpyHostToDevice));
    PLAN_CUDA(cudaMemcpy(p->d_pq, pq.data(), sizeof(PQInst) * pq.size(), cudaMemcpyHostToDevice));
    PLAN_CUDA(cudaMemcpy(p->d_order, order.data(), sizeof(int) * order.size(), cudaMemcpyHostToDevice));
    {
        // every PLUQ starts on the per-instance kernel; the prologue hands the step route's back
        std::vector<int> ones(std::max(1, p->n_pq), 1), st_order, st_live;
        for (size_t gi = 0; gi < p->groups.size(); gi++) {
            st_order.insert(st_order.end(), gmembers[gi].begin(), gmembers[gi].end());
            st_live.insert(st_live.end(), p->groups[gi].live.begin(), p->groups[gi].live.end());
        }
        PLAN_CUDA(cudaMemcpy(p->step.flags, ones.data(), sizeof(int) * ones.size(), cudaMemcpyHostToDevice));
        if (p->n_step > 0) {
            PLAN_CUDA(cudaMemcpy(const_cast<StepInst *>(p->step.steps), stv.data(), sizeof(StepInst) * stv.size(),
                                 cudaMemcpyHostToDevice));
            PLAN_CUDA(cudaMemcpy(const_cast<int *>(p->step.order), st_order.data(), sizeof(int) * p->n_step,
                                 cudaMemcpyHostToDevice));
            PLAN_CUDA(cudaMemcpy(const_cast<int *>(p->step.live), st_live.data(), sizeof(int) * st_live.size(),
                                 cudaMemcpyHostToDevice));
            PLAN_CUDA(cudaMemcpy(const_cast<CUtensorMap *>(p->step.tmaps), stmaps.data(),
                                 sizeof(CUtensorMap) * 2 * p->n_step, cudaMemcpyHostToDevice));
            if (!st_items.empty())
                PLAN_CUDA(cudaMemcpy(p->d_step_items, st_items.data(), sizeof(WorkItem) * st_items.size(),
                                     cudaMemcpyHostToDevice));
            // rows past an instance's running block are read by the GEMM (their results dropped)
            PLAN_CUDA(cudaMemset(base + o_planes, 0, planes_bytes));
        }
    }

    st = build_graph(p, tu.overlap != 0);
    if (st) {
        free_plan(p);
        return st;
    }
    *out = p;
    return GFFM_OK;
}

}  // namespace

extern "C" {

int gffm_batched_plan_create(const gffm_batch_desc *descs, int64_t count, const gffm_batch_tuning *tuning,
                             gffm_batch_plan *plan) {
    return create(descs, count, tuning, plan);
}

int gffm_batched_plan_info(gffm_batch_plan plan, int64_t *info) {
    if (!plan || !info) return set_error(GFFM_ERR_ARG, "null argument");
    info[0] = (int64_t)plan->mem_bytes;
    info[1] = plan->n_mm;
    info[2] = plan->n_pq + (int64_t)plan->tall.size();
    info[3] = plan->nitems;
    info[4] = plan->gemm_grid;
    info[5] = plan->pq_grid;
    return GFFM_OK;
}

int gffm_batched_run(gffm_batch_plan plan, gffm_stream_t stream) {
    if (!plan) return set_error(GFFM_ERR_ARG, "plan is NULL");
    if (!plan->exec && plan->tall.empty()) return GFFM_OK;
    int dev = 0;
    GFFM_CUDA(cudaGetDevice(&dev));
    if (dev != plan->device) return set_error(GFFM_ERR_ARG, "the plan belongs to device %d", plan->device);
    const cudaStream_t s = gffm::as_stream(stream);
    if (plan->exec) GFFM_CUDA(cudaGraphLaunch(plan->exec, s));
    // the tall PLUQs, one after another on the same stream (each call synchronizes it)
    for (const gffm_batch_desc &d : plan->tall) {
        plan->h_rows.assign(2 * d.m, 0);
        plan->h_cols.assign(2 * d.n, 0);
        int64_t nr = 0, nc = 0, rank = 0;
        int st = gffm_pluq_f64(d.m, d.n, d.A, d.lda, d.C, d.ldc, d.L, d.ldl, d.l_cols, d.N, plan->h_rows.data(), &nr,
                               plan->h_cols.data(), &nc, &rank, nullptr, 0, stream);
        int64_t info[4] = {nr, nc, rank, 0};
        if (st == GFFM_ERR_BOUNDS) {
            info[0] = info[1] = info[2] = 0;     // the reference's BoundsError for this instance
            info[3] = GFFM_ERR_BOUNDS;
        } else if (st) {
            return st;
        }
        if (info[0]) GFFM_CUDA(cudaMemcpyAsync(d.row_swaps, plan->h_rows.data(), 2 * info[0] * 8, cudaMemcpyHostToDevice, s));
        if (info[1]) GFFM_CUDA(cudaMemcpyAsync(d.col_swaps, plan->h_cols.data(), 2 * info[1] * 8, cudaMemcpyHostToDevice, s));
        GFFM_CUDA(cudaMemcpyAsync(d.info, info, sizeof(info), cudaMemcpyHostToDevice, s));
        GFFM_CUDA(cudaStreamSynchronize(s));   // the host staging is reused by the next instance
    }
    return GFFM_OK;
}

int gffm_batched_plan_destroy(gffm_batch_plan plan) {
    free_plan(plan);
    return GFFM_OK;
}

}  // extern "C"
