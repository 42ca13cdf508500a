// limb_host.h -- host interface of the limb tensor-core GEMM, shared by the
// GEMM entry points, the elimination (trailing updates) and Karatsuba.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>

namespace limb {

// epilogue of the GEMM: store Float64 / Float32 / int32 residues, or C = (C - AB) mod N on int32
enum Epi { EPI_STORE_F64 = 0, EPI_STORE_F32 = 1, EPI_SUB_I32 = 2, EPI_STORE_I32 = 3 };

struct Layout {
    int L;                 // digits per residue
    int64_t Mpad, Npad, Kpad;
    size_t a_bytes, b_bytes;
};

int limbs_for(int64_t N);
Layout layout(int64_t m, int64_t n, int64_t k, int64_t N);
int check_args(int64_t m, int64_t n, int64_t k, int64_t lda, int64_t ldb, int64_t ldc, int64_t N);

// digit planes of A (m x k) / B (k x n), column-major inputs of type T
template <typename T>
int split_a(const T *A, int64_t lda, int64_t m, int64_t k, __half *D, const Layout &g, int64_t N, cudaStream_t s);
template <typename T>
int split_b(const T *B, int64_t ldb, int64_t k, int64_t n, __half *D, const Layout &g, int64_t N, cudaStream_t s);

// C (m x n, ldc) <- epilogue(A*B mod N) from digit planes; epi is a limb::Epi
int gemm_digits(const Layout &g, const __half *Ad, const __half *Bd, int64_t m, int64_t n, int64_t k, int64_t N,
                void *C, int64_t ldc, int epi, int max_ctas, cudaStream_t s);

}  // namespace limb
