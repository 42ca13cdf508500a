// limb_host.h -- host interface of the limb tensor-core GEMM, shared by the
// GEMM entry points, the elimination (trailing updates) and Karatsuba.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>

namespace limb {

// epilogue of the GEMM:
//   EPI_STORE_F64 / F32 / I32  C = AB mod N stored as Float64 / Float32 / int32
//   EPI_SUB_I32                C = (C - AB) mod N on int32
//   EPI_EXACT_I64              C = AB mod N on int64 for 2 <= N < 2^52, from NON-centred digits
//                              (SPLIT_RAW): every exact chunk value is folded in modulo N
//   EPI_KSUB_F64               C = (AB - X - Y) mod N on Float64, X and Y Float64 residues with C's ldc
//   EPI_SUB_I32M               EPI_SUB_I32 with odd N and one exact chunk (selected inside gemm_digits)
enum Epi { EPI_STORE_F64 = 0, EPI_STORE_F32 = 1, EPI_SUB_I32 = 2, EPI_STORE_I32 = 3, EPI_EXACT_I64 = 4, EPI_KSUB_F64 = 5,
           EPI_SUB_I32M = 6 };

// digit split of an operand:
//   SPLIT_CENTRED  x mod N centred into (-N/2, N/2]
//   SPLIT_RAW      x mod N in [0, N)            (needs raw_limbs_for(N) digits)
//   SPLIT_SUM      (x + y) mod N centred, y from a second array with the same leading dimension
enum Split { SPLIT_CENTRED = 0, SPLIT_RAW = 1, SPLIT_SUM = 2 };

struct Layout {
    int L;                 // digits per residue
    int bits = 7;          // digit width: balanced base-2^bits digits (7 or 8)
    int bn = 64;           // output tile width: 64, or 32 with two accumulator sets
    int64_t Mpad, Npad, Kpad;
    size_t a_bytes, b_bytes;
};

int limbs_for(int64_t N);
int limbs_for_bits(int64_t N, int bits);   // centred digits of width `bits` (7 or 8)
int raw_limbs_for(int64_t N);
Layout layout(int64_t m, int64_t n, int64_t k, int64_t N);
Layout layout_bits(int64_t m, int64_t n, int64_t k, int64_t N, int bits);
int chunk_kblocks(const Layout &g);        // k-blocks of 64 per exact accumulation chunk
// The fast drain's constants (odd N, one exact chunk, shift sums within 2^22): ninv =
// -N^-1 mod 2^32, Wm[s] = 2^(bits s) 2^32 mod N for s < MAX_SHIFTS, and the initial
// value that takes out the magic-number bits and keeps the sum in (0, 2^32 N), for a
// drain that reads the shifts in pairs (`paired`, 7-bit digits only; see fast_pair) or
// one at a time.
void fast_consts(int64_t N, int L, int bits, bool paired, uint32_t *ninv, int32_t *Wm, int64_t *fbias);
// how the digit products of a limb GEMM are formed (gffm_limb_tuning.form)
enum Form { FORM_DEFAULT = 0, FORM_SCHOOLBOOK = 1, FORM_KARATSUBA = 2 };
// the default form is Karatsuba (kara_host.h) for four 7-bit digits from this inner dimension on
constexpr int64_t KARA_MIN_K = 1024;
// the process-wide tune table's choice for a product (digit width, grid, tile width, form);
// defaults 7 / 0 / 64 / FORM_DEFAULT
void tuned_for(int64_t m, int64_t n, int64_t k, int64_t N, int *bits, int *max_ctas, int *tile_n, int *form);
// FORM_SCHOOLBOOK or FORM_KARATSUBA for a tuned form, digit width, tile width, modulus and inner dimension
int resolve_form(int form, int bits, int tile_n, int64_t N, int64_t k);
Layout layout_L(int64_t m, int64_t n, int64_t k, int L);
int check_args(int64_t m, int64_t n, int64_t k, int64_t lda, int64_t ldb, int64_t ldc, int64_t N);

// digit planes of A (m x k) / B (k x n), column-major inputs of type T; A2 / B2 only for SPLIT_SUM
template <typename T>
int split_a(const T *A, int64_t lda, int64_t m, int64_t k, __half *D, const Layout &g, int64_t N, cudaStream_t s,
            int mode = SPLIT_CENTRED, const T *A2 = nullptr);
template <typename T>
int split_b(const T *B, int64_t ldb, int64_t k, int64_t n, __half *D, const Layout &g, int64_t N, cudaStream_t s,
            int mode = SPLIT_CENTRED, const T *B2 = nullptr);

// Encode the TMA descriptor (a 128-byte CUtensorMap at `map`) of a digit array:
// `rows` rows of `kpad` fp16, box 64 x box_rows, 128-byte swizzle.
int encode_digit_map(void *map, const void *base, int64_t kpad, int64_t rows, int box_rows);
// the same over planes of K = 32 (64-byte rows): box 32 x box_rows, 64-byte swizzle
int encode_digit_map_k32(void *map, const void *base, int64_t rows, int box_rows);

// C (m x n, ldc) <- epilogue(A*B mod N) from digit planes; epi is a limb::Epi.  X, Y: EPI_KSUB_F64 only.
// tile_counter: nullptr for the static tile schedule, else a device int (zero before the first of
// them) from which every launch of this same product draws its tiles, so that a launch made later
// on SMs that became free shares the remaining tiles.
int gemm_digits(const Layout &g, const __half *Ad, const __half *Bd, int64_t m, int64_t n, int64_t k, int64_t N,
                void *C, int64_t ldc, int epi, int max_ctas, cudaStream_t s, const double *X = nullptr,
                const double *Y = nullptr, int *tile_counter = nullptr);

}  // namespace limb
