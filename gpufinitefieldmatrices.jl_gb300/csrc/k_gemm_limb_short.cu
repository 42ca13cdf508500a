// k_gemm_limb_short.cu -- the limb GEMM's 32-column tile variant with two TMEM
// accumulator sets (gemm_limb.cuh, BNV = 32), used when every output tile is at
// most a couple of exact chunks long: the elimination's trailing updates
// (K = 128), back substitution and short products.  Kept in its own
// translation unit so the variants compile in parallel.
#include "limb_launch.cuh"

namespace limb {

template <int EPI>
static int launch_short_L(int L, const CUtensorMap &ta, const CUtensorMap &tb, const Params &p, int grid,
                          cudaStream_t s) {
    switch (L) {
        case 1: return launch_gemm_L<1, EPI, 32>(ta, tb, p, grid, s);
        case 2: return launch_gemm_L<2, EPI, 32>(ta, tb, p, grid, s);
        case 3: return launch_gemm_L<3, EPI, 32>(ta, tb, p, grid, s);
        default: return launch_gemm_L<4, EPI, 32>(ta, tb, p, grid, s);
    }
}

int launch_gemm_short(int epi, int L, const CUtensorMap &ta, const CUtensorMap &tb, const Params &p, int grid,
                      cudaStream_t s) {
    switch (epi) {
        case EPI_STORE_F64: return launch_short_L<EPI_STORE_F64>(L, ta, tb, p, grid, s);
        case EPI_STORE_F32: return launch_short_L<EPI_STORE_F32>(L, ta, tb, p, grid, s);
        case EPI_STORE_I32: return launch_short_L<EPI_STORE_I32>(L, ta, tb, p, grid, s);
        case EPI_EXACT_I64: return launch_short_L<EPI_EXACT_I64>(L, ta, tb, p, grid, s);
        case EPI_KSUB_F64: return launch_short_L<EPI_KSUB_F64>(L, ta, tb, p, grid, s);
        case EPI_SUB_I32M: return launch_short_L<EPI_SUB_I32M>(L, ta, tb, p, grid, s);
        default: return launch_short_L<EPI_SUB_I32>(L, ta, tb, p, grid, s);
    }
}

}  // namespace limb
