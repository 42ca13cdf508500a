// kara_host.h -- host interface of the 12-product Karatsuba limb GEMM
// (gemm_kara.cuh): moduli 2080639 < N < 2^26, store and Karatsuba-middle-term
// epilogues.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>

namespace kara {

struct Layout {
    int64_t Mpad, Npad, Kpad;   // rows of the A / B digit planes (multiples of 128), padded K (multiple of 64)
    size_t a_bytes, b_bytes;    // six fp16 planes each
};

// true when the Karatsuba form covers modulus N (four 7-bit digits: 2080639 < N < 2^26)
bool applies(int64_t N);
Layout layout(int64_t m, int64_t n, int64_t k);

// six digit planes of A (m x k) / B (k x n), column-major inputs of type T: the centred residues, or
// with A2 / B2 (Float64 only) the centred (A + A2) mod N, the Karatsuba sum of two operands
template <typename T>
int split_a(const T *A, int64_t lda, int64_t m, int64_t k, __half *D, const Layout &g, int64_t N, cudaStream_t s,
            const T *A2 = nullptr);
template <typename T>
int split_b(const T *B, int64_t ldb, int64_t k, int64_t n, __half *D, const Layout &g, int64_t N, cudaStream_t s,
            const T *B2 = nullptr);

// C (m x n, ldc) <- epilogue(A*B mod N) from the six-plane digit arrays; epi is limb::EPI_STORE_F64 /
// EPI_STORE_F32 / EPI_STORE_I32 / EPI_KSUB_F64 (X, Y: the subtrahends of the last one).
int gemm_digits(const Layout &g, const __half *Ad, const __half *Bd, int64_t m, int64_t n, int64_t k, int64_t N,
                void *C, int64_t ldc, int epi, int max_ctas, cudaStream_t s, const double *X = nullptr,
                const double *Y = nullptr);

}  // namespace kara
