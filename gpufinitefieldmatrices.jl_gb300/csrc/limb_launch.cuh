// limb_launch.cuh -- launching the limb GEMM kernel (gemm_limb.cuh) with a given
// digit count, epilogue and tile width; shared by the translation units that
// instantiate its variants.
#pragma once

#include "gemm_limb.cuh"

namespace limb {

template <int L, int EPI, int BNV>
static int launch_gemm_L(const CUtensorMap &ta, const CUtensorMap &tb, const Params &p, int grid, cudaStream_t s) {
    auto kern = k_gemm_limb<L, EPI, BNV>;
    constexpr int smem = Cfg<L, BNV>::SMEM_BYTES;
    GFFM_CUDA((gffm::ensure_dynamic_smem<k_gemm_limb<L, EPI, BNV>>(smem)));
    gffm::profile_hook().before(s);
    kern<<<grid, gemm_threads(EPI), smem, s>>>(ta, tb, p);
    gffm::profile_hook().after(s);
    GFFM_LAUNCH_CHECK("k_gemm_limb");
    return GFFM_OK;
}

// the 32-column, double-buffered variant for short K (k_gemm_limb_short.cu)
int launch_gemm_short(int epi, int L, const CUtensorMap &ta, const CUtensorMap &tb, const Params &p, int grid,
                      cudaStream_t s);

}  // namespace limb
