/*
 * gffm.h -- C ABI of libgffm, the GB300 (sm_103a) implementation of the hot
 * path of GPUFiniteFieldMatrices.jl: exact modular matrix multiply for moduli
 * N < 2^26, PLUQ / LU / RREF over prime fields, and the two-digit Karatsuba
 * matrix type.
 *
 * Conventions (they mirror the reference's CuModArray, src/CuModMatrix/
 * CuModMatrix.jl:42-122):
 *   - matrices are column-major device buffers with an explicit leading
 *     dimension (the reference pads every dimension by 32, so a CuModMatrix of
 *     size (m, n) has ld = m + 32; any ld >= m is accepted);
 *   - elements are residues stored as double (Float64) or float (Float32);
 *   - sizes are the true (unpadded) sizes;
 *   - every call is asynchronous on `stream` (a cudaStream_t, NULL = legacy
 *     default stream) unless its comment says it synchronizes;
 *   - every call returns a gffm_status; the message of the last failure on the
 *     calling thread is available from gffm_last_error_string();
 *   - argument and overflow checks happen on the host before any launch and
 *     raise the errors the reference throws (size / modulus mismatch, "cannot
 *     perform a single multiplication" ...).
 * The library never frees caller memory.  Calls that take a workspace accept
 * NULL, in which case they allocate stream-ordered scratch (cudaMallocAsync)
 * and release it on the same stream.
 */
#ifndef GFFM_H
#define GFFM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define GFFM_API __attribute__((visibility("default")))
#else
#define GFFM_API
#endif

typedef void *gffm_stream_t; /* cudaStream_t */

enum gffm_status {
    GFFM_OK = 0,
    GFFM_ERR_ARG = 1,         /* null pointer, negative size, ld too small */
    GFFM_ERR_SIZE = 2,        /* CuModArraySizeMismatchException / DimensionMismatch */
    GFFM_ERR_MODULUS = 3,     /* modulus out of the supported range */
    GFFM_ERR_STRIPE = 4,      /* "cannot perform a single multiplication" (stripe_mul.jl:200-202) */
    GFFM_ERR_WORKSPACE = 5,   /* caller workspace too small */
    GFFM_ERR_CUDA = 6,        /* a CUDA runtime / driver call failed */
    GFFM_ERR_TIMEOUT = 7,     /* a device-side wait gave up (kernel returned early) */
    GFFM_ERR_BOUNDS = 8,      /* the reference would index out of bounds */
    GFFM_ERR_NOT_PRIME = 9,   /* CuModMatrixModulusNotPrimeException */
    GFFM_ERR_UNSUPPORTED = 10 /* no sm_103 device, or an unsupported configuration */
};

/* ---- library ---------------------------------------------------------- */

/* Version string of the library (no reference counterpart). */
GFFM_API const char *gffm_version(void);

/* Message of the last failed call on this thread (no reference counterpart;
 * replaces the text of the Julia exceptions, CuModMatrix.jl:5-31). */
GFFM_API const char *gffm_last_error_string(void);

/* Synchronizes `stream` and reports (then clears) a device-side failure
 * recorded by any kernel of the library since the last call: GFFM_OK or
 * GFFM_ERR_TIMEOUT.  (No reference counterpart.) */
GFFM_API int gffm_device_status(gffm_stream_t stream);

/* Kernel timing hook (no reference counterpart): the next call on this thread
 * that launches the library's main tensor-core kernel (the limb GEMM, or a
 * trailing update of the elimination) records `start_event` just before and
 * `stop_event` just after that kernel, on the call's stream.  The events are
 * cudaEvent_t handles created by the caller; the hook is then cleared. */
GFFM_API int gffm_profile_next_kernel(void *start_event, void *stop_event);

/* find_max_stripe_ops(type, N) (src/CuModMatrix/kernel_mul/stripe_mul.jl:13-27):
 * the number of products that can be summed exactly in the element type
 * before a reduction.  bits = 53 (Float64), 24 (Float32), 11 (Float16). */
GFFM_API int gffm_find_max_stripe_ops(int bits, int64_t N, int64_t *out);

/* ---- elementwise modular kernels (the .jl files of src/CuModMatrix/kernel_ops) ----
 * All act on `len` contiguous elements -- the whole padded data array, as the
 * reference's grid-stride kernels do -- with Julia mod semantics (result in
 * [0, N)).  In-place use (C == A or C == B) is allowed. */

/* add!(C, A, B; mod_N) -> k_add_matrix! (add_ops.jl:3-11,23-30) */
GFFM_API int gffm_add_f64(double *C, const double *A, const double *B, int64_t len, int64_t N, gffm_stream_t stream);
GFFM_API int gffm_add_f32(float *C, const float *A, const float *B, int64_t len, int64_t N, gffm_stream_t stream);
/* sub!(C, A, B; mod_N) -> k_sub_matrix! (sub_ops.jl:3-11,33-40) */
GFFM_API int gffm_sub_f64(double *C, const double *A, const double *B, int64_t len, int64_t N, gffm_stream_t stream);
GFFM_API int gffm_sub_f32(float *C, const float *A, const float *B, int64_t len, int64_t N, gffm_stream_t stream);
/* elementwise_multiply!(C, A, B, mod_N) -> k_mul_matrix! (mul_ops.jl:13-21,23-30) */
GFFM_API int gffm_mul_elementwise_f64(double *C, const double *A, const double *B, int64_t len, int64_t N, gffm_stream_t stream);
GFFM_API int gffm_mul_elementwise_f32(float *C, const float *A, const float *B, int64_t len, int64_t N, gffm_stream_t stream);
/* scalar_add!(C, A, s, mod_N) -> k_add_scalar! (add_ops.jl:13-21,32-40) */
GFFM_API int gffm_scalar_add_f64(double *C, const double *A, double s, int64_t len, int64_t N, gffm_stream_t stream);
GFFM_API int gffm_scalar_add_f32(float *C, const float *A, float s, int64_t len, int64_t N, gffm_stream_t stream);
/* scalar_sub!(C, A, s, mod_N) -> k_sub_scalar! (sub_ops.jl:13-21,42-50) */
GFFM_API int gffm_scalar_sub_f64(double *C, const double *A, double s, int64_t len, int64_t N, gffm_stream_t stream);
GFFM_API int gffm_scalar_sub_f32(float *C, const float *A, float s, int64_t len, int64_t N, gffm_stream_t stream);
/* rscalar_sub!(C, A, s, mod_N), negate! = rscalar_sub!(B, A, 0) -> k_rsub_scalar! (sub_ops.jl:23-31,52-60) */
GFFM_API int gffm_rscalar_sub_f64(double *C, const double *A, double s, int64_t len, int64_t N, gffm_stream_t stream);
GFFM_API int gffm_rscalar_sub_f32(float *C, const float *A, float s, int64_t len, int64_t N, gffm_stream_t stream);
/* mul!(C, A, s, mod_N) -> k_mul_scalar! (mul_ops.jl:3-11,32-40) */
GFFM_API int gffm_scalar_mul_f64(double *C, const double *A, double s, int64_t len, int64_t N, gffm_stream_t stream);
GFFM_API int gffm_scalar_mul_f32(float *C, const float *A, float s, int64_t len, int64_t N, gffm_stream_t stream);
/* mod!(C, A, N) / mod_elements! -> k_mod! (mod_ops.jl:3-11,13-21) */
GFFM_API int gffm_mod_f64(double *C, const double *A, int64_t len, int64_t N, gffm_stream_t stream);
GFFM_API int gffm_mod_f32(float *C, const float *A, int64_t len, int64_t N, gffm_stream_t stream);
/* div!(C, A, s, mod_N) and A / s (div_ops.jl:13-29): C = A * mod_inv(s, N) mod N */
GFFM_API int gffm_div_scalar_f64(double *C, const double *A, int64_t s, int64_t len, int64_t N, gffm_stream_t stream);
GFFM_API int gffm_div_scalar_f32(float *C, const float *A, int64_t s, int64_t len, int64_t N, gffm_stream_t stream);
/* divide_elements!(B, A, N) (KaratsubaMatrix.jl:733-736): C = div.(A, N), Julia's
 * truncating integer division, no reduction */
GFFM_API int gffm_trunc_div_f64(double *C, const double *A, int64_t len, int64_t N, gffm_stream_t stream);
GFFM_API int gffm_trunc_div_f32(float *C, const float *A, int64_t len, int64_t N, gffm_stream_t stream);
/* mod_inv(p, P) (rref_lu_pluq/pluq_kernels.jl:11-31), on the host: the extended
 * Euclid sequence with truncating division; 0 for p = 0 and a non-inverse when
 * gcd(p, P) > 1, as the reference returns.  1 <= P <= 2^52. */
GFFM_API int gffm_mod_inv(int64_t p, int64_t P, int64_t *out);

/* ---- plain modular GEMM / GEMV: the reference's own method ---------------
 * C = A*B mod N with A (m x k, lda), B (k x n, ldb), C (m x n, ldc).
 * Products are summed exactly in the element type in K-stripes of
 * `stripe` columns (0 = find_max_stripe_ops(type, N), the reference's bound)
 * and reduced mod N after every stripe, as stripe_mul! does
 * (src/CuModMatrix/kernel_mul/stripe_mul.jl:175-244, called by mul!,
 * CuModMatrix.jl:767-787, and *, kernel_ops/mul_ops.jl:54-58); the stripes
 * are reduced in registers instead of by full-matrix mod! passes.  Only the
 * m x n region of C is written.  GFFM_ERR_STRIPE when the stripe bound is
 * below one product.  C must not alias A or B. */
GFFM_API int gffm_matmul_plain_f64(int64_t m, int64_t n, int64_t k, const double *A, int64_t lda, const double *B,
                          int64_t ldb, double *C, int64_t ldc, int64_t N, int64_t stripe, gffm_stream_t stream);
GFFM_API int gffm_matmul_plain_f32(int64_t m, int64_t n, int64_t k, const float *A, int64_t lda, const float *B,
                          int64_t ldb, float *C, int64_t ldc, int64_t N, int64_t stripe, gffm_stream_t stream);
/* z = A*x mod N (stripe_mul! vector form, stripe_mul.jl:82-168; mul!(z, A, x),
 * CuModMatrix.jl:816-836).  Vectors are contiguous. */
GFFM_API int gffm_matvec_plain_f64(int64_t m, int64_t k, const double *A, int64_t lda, const double *x, double *z,
                          int64_t N, int64_t stripe, gffm_stream_t stream);
GFFM_API int gffm_matvec_plain_f32(int64_t m, int64_t k, const float *A, int64_t lda, const float *x, float *z,
                          int64_t N, int64_t stripe, gffm_stream_t stream);

/* ---- limb tensor-core modular GEMM ---------------------------------------
 * Same contract as gffm_matmul_plain_* (replaces stripe_mul! / mul! / * /
 * mat_mul_gpu_type / mat_mul_type_inplace!, mat_mul_gpu_direct.jl:8-85, for
 * 2 <= N < 2^26) but exact for every k: residues are centred, split into
 * balanced base-2^7 digits held in fp16, multiplied on the tcgen05 tensor
 * cores with fp32 accumulation (exact: every partial sum is an integer below
 * 2^24), and recombined and reduced mod N in the epilogue.  Inputs may hold
 * any integer value (they are reduced mod N first), so a modulus override
 * (mat_mul_gpu_type(A, B, mod_N)) is a different N on the same buffers.
 * Workspace: gffm_matmul_limb_workspace_size bytes, or NULL. */
GFFM_API int gffm_matmul_limb_workspace_size(int64_t m, int64_t n, int64_t k, int64_t N, size_t *bytes);
GFFM_API int gffm_matmul_limb_f64(int64_t m, int64_t n, int64_t k, const double *A, int64_t lda, const double *B,
                         int64_t ldb, double *C, int64_t ldc, int64_t N, void *workspace, size_t workspace_bytes,
                         gffm_stream_t stream);
GFFM_API int gffm_matmul_limb_f32(int64_t m, int64_t n, int64_t k, const float *A, int64_t lda, const float *B,
                         int64_t ldb, float *C, int64_t ldc, int64_t N, void *workspace, size_t workspace_bytes,
                         gffm_stream_t stream);

/* ---- tuning of the limb GEMM (no reference counterpart) -----------------------
 * digit_bits: 7 (balanced base-2^7 digits, the default) or 8 (base-2^8: one
 * digit fewer for 16255 < N <= 65279 and 2080639 < N <= 16711423, with 4x more
 * frequent exact-accumulation drains); 0 keeps the table's / default choice.
 * max_ctas: persistent grid size (0 = one CTA per SM); tile_n: 0/64 or 32.
 * form: how the digit products are formed: 1 = schoolbook (L^2 digit products,
 * 16 for four digits), 2 = one level of Karatsuba over 13-bit halves (12 digit
 * products; moduli 2080639 < N < 2^26 only, its own 7/6-bit digits, 128 x 128
 * tiles; digit_bits and tile_n do not apply), 0 = the default: Karatsuba where
 * it applies, k >= 1024 and neither 8-bit digits nor 32-column tiles were
 * asked for, else schoolbook.  The process-wide tune
 * table (written by the autotuner, gffm/autotune.py) maps a modulus range and a
 * work range (m*n*k) to a tuning; gffm_matmul_limb_* and its workspace size
 * consult it, first matching entry wins.  It is the library's only global
 * mutable state. */
typedef struct gffm_limb_tuning {
    int32_t digit_bits;
    int32_t max_ctas;
    int32_t tile_n;           /* output tile width: 64 (default) or 32 with two TMEM accumulator sets */
    int32_t form;             /* 0 default, 1 schoolbook, 2 Karatsuba (12 digit products) */
} gffm_limb_tuning;
typedef struct gffm_tune_entry {
    int64_t N_lo, N_hi;       /* inclusive modulus range */
    double work_lo, work_hi;  /* inclusive m*n*k range */
    gffm_limb_tuning tuning;
} gffm_tune_entry;
GFFM_API int gffm_tune_table_set(const gffm_tune_entry *entries, int64_t count);
GFFM_API int gffm_tune_table_size(int64_t *count);
GFFM_API int gffm_matmul_limb_tuned_workspace_size(int64_t m, int64_t n, int64_t k, int64_t N,
                                                   const gffm_limb_tuning *tuning, size_t *bytes);
GFFM_API int gffm_matmul_limb_tuned_f64(int64_t m, int64_t n, int64_t k, const double *A, int64_t lda,
                                        const double *B, int64_t ldb, double *C, int64_t ldc, int64_t N,
                                        const gffm_limb_tuning *tuning, void *workspace, size_t workspace_bytes,
                                        gffm_stream_t stream);

/* ---- elimination over Z/N, 2 <= N < 2^26 -----------------------------------
 * Blocked right-looking elimination with the reference's exact step
 * semantics; the trailing updates run on the limb tensor-core GEMM.  These
 * calls synchronize `stream` (they return host data).  Workspace:
 * gffm_elim_workspace_size bytes (l_cols = padded width of L; 0 for RREF),
 * or NULL.  U / R may alias A.  Arithmetic follows the reference's mod_inv
 * (extended Euclid) for the pivot inverses, so composite N behaves as the
 * reference's algorithm does. */
GFFM_API int gffm_elim_workspace_size(int64_t m, int64_t n, int64_t l_cols, size_t *bytes);

/* pluq_gpu_kernel(A) -> (U, L, Perm_rows, Perm_cols)
 * (src/CuModMatrix/rref_lu_pluq/pluq_kernels.jl:46-157): pivot = largest
 * residue of the column below the current row (lowest row on ties); a zero
 * column is swapped with the last column and skipped; U is unit upper with the
 * pivot rows scaled by the pivot inverse; L (m x l_cols, the reference's L is
 * (m+32) x (m+32)) holds the pivot values at (row, col) and the eliminated
 * entries below.  row_swaps / col_swaps receive the swap stacks as 1-based
 * (i, j) pairs (capacity 2*m and 2*n int64), in order.  GFFM_ERR_BOUNDS where
 * the reference would index L out of bounds.  There is no row limit: while
 * more rows lie below a panel than the cooperative panel keeps in shared
 * memory (min(SMs, 160) * 288: 43776 on a 152-SM GB300), panels are 32
 * columns wide and factor right-looking in global memory, with the same
 * results.  The same holds for the LU, RREF and inverse entries below. */
GFFM_API int gffm_pluq_f64(int64_t m, int64_t n, const double *A, int64_t lda, double *U, int64_t ldu, double *L,
                           int64_t ldl, int64_t l_cols, int64_t N, int64_t *row_swaps, int64_t *n_row_swaps,
                           int64_t *col_swaps, int64_t *n_col_swaps, int64_t *rank, void *workspace,
                           size_t workspace_bytes, gffm_stream_t stream);
GFFM_API int gffm_pluq_f32(int64_t m, int64_t n, const float *A, int64_t lda, float *U, int64_t ldu, float *L,
                           int64_t ldl, int64_t l_cols, int64_t N, int64_t *row_swaps, int64_t *n_row_swaps,
                           int64_t *col_swaps, int64_t *n_col_swaps, int64_t *rank, void *workspace,
                           size_t workspace_bytes, gffm_stream_t stream);

/* The same factorization with the trailing products on the reference's plain
 * Float64 arithmetic (stripe_mul.jl:175-244: exact FP64 products summed in
 * stripes of find_max_stripe_ops(Float64, N), reduced after each stripe)
 * instead of the limb tensor-core GEMM: the comparison leg of the two forms. */
GFFM_API int gffm_pluq_plain_f64(int64_t m, int64_t n, const double *A, int64_t lda, double *U, int64_t ldu,
                                 double *L, int64_t ldl, int64_t l_cols, int64_t N, int64_t *row_swaps,
                                 int64_t *n_row_swaps, int64_t *col_swaps, int64_t *n_col_swaps, int64_t *rank,
                                 void *workspace, size_t workspace_bytes, gffm_stream_t stream);

/* lu_gpu_type(A) -> (U, L, Perm) (intended API, test/Experiments/rref_gpu_type.jl:60-103):
 * the same pivot rule without column swaps -- a zero column is skipped and
 * L's column index is the pivot count.  L is m x m; perm (host, m int64)
 * receives the 1-based original row index of each row of U. */
GFFM_API int gffm_lu_f64(int64_t m, int64_t n, const double *A, int64_t lda, double *U, int64_t ldu, double *L,
                         int64_t ldl, int64_t N, int64_t *perm, int64_t *rank, void *workspace,
                         size_t workspace_bytes, gffm_stream_t stream);
GFFM_API int gffm_lu_f32(int64_t m, int64_t n, const float *A, int64_t lda, float *U, int64_t ldu, float *L,
                         int64_t ldl, int64_t N, int64_t *perm, int64_t *rank, void *workspace,
                         size_t workspace_bytes, gffm_stream_t stream);

/* rref_gpu_type(A) (intended API, test/Experiments/rref_gpu_type.jl:8-51;
 * called by test/CuModMatrix/benchmark_test.jl:144): the reduced row echelon
 * form mod N into R (unique for prime N).  pivot_cols (host, capacity
 * min(m, n) int64, may be NULL) receives the 1-based pivot columns.
 * GFFM_ERR_NOT_PRIME for a composite N (the form is defined over a field). */
GFFM_API int gffm_rref_f64(int64_t m, int64_t n, const double *A, int64_t lda, double *R, int64_t ldr, int64_t N,
                           int64_t *rank, int64_t *pivot_cols, void *workspace, size_t workspace_bytes,
                           gffm_stream_t stream);
GFFM_API int gffm_rref_f32(int64_t m, int64_t n, const float *A, int64_t lda, float *R, int64_t ldr, int64_t N,
                           int64_t *rank, int64_t *pivot_cols, void *workspace, size_t workspace_bytes,
                           gffm_stream_t stream);

/* inverse(A) / is_invertible_with_inverse(A) (src/CuModMatrix/CuModMatrix.jl:356-422,
 * 480-502): *invertible = 1 and Ainv = A^{-1} mod N when A (n x n) is invertible,
 * else *invertible = 0 and Ainv untouched.  Computed from the RREF of [A | I] (the
 * inverse is unique; the reference composes U^{-1} L^{-1} from PLUQ).  Synchronizes.
 * GFFM_ERR_NOT_PRIME for a composite N.
 * Workspace: gffm_inverse_workspace_size(n) bytes (Float32 needs at most that), or NULL. */
GFFM_API int gffm_inverse_workspace_size(int64_t n, size_t *bytes);
GFFM_API int gffm_inverse_f64(int64_t n, const double *A, int64_t lda, double *Ainv, int64_t ldi, int64_t N,
                              int *invertible, void *workspace, size_t workspace_bytes, gffm_stream_t stream);
GFFM_API int gffm_inverse_f32(int64_t n, const float *A, int64_t lda, float *Ainv, int64_t ldi, int64_t N,
                              int *invertible, void *workspace, size_t workspace_bytes, gffm_stream_t stream);

/* ---- swap-stack permutations (src/CuModMatrix/rref_lu_pluq/permutations.jl) --
 * A is nrows x ncols, column-major; `swaps` is a HOST array of nswaps 1-based
 * (i, j) pairs (the reference's Vector{Tuple{Int,Int}}), applied in order, or
 * in reverse order when `inverse` is non-zero.  Indices are checked on the
 * host (GFFM_ERR_BOUNDS).
 * apply_row_perm! / apply_row_inv_perm! (:73-89) */
GFFM_API int gffm_apply_row_swaps_f64(double *A, int64_t lda, int64_t nrows, int64_t ncols, const int64_t *swaps,
                                      int64_t nswaps, int inverse, gffm_stream_t stream);
GFFM_API int gffm_apply_row_swaps_f32(float *A, int64_t lda, int64_t nrows, int64_t ncols, const int64_t *swaps,
                                      int64_t nswaps, int inverse, gffm_stream_t stream);
/* apply_col_perm! / apply_col_inv_perm! (:11-27) */
GFFM_API int gffm_apply_col_swaps_f64(double *A, int64_t lda, int64_t nrows, int64_t ncols, const int64_t *swaps,
                                      int64_t nswaps, int inverse, gffm_stream_t stream);
GFFM_API int gffm_apply_col_swaps_f32(float *A, int64_t lda, int64_t nrows, int64_t ncols, const int64_t *swaps,
                                      int64_t nswaps, int inverse, gffm_stream_t stream);

/* ---- KaratsubaArray (src/KaratsubaMatrix/) --------------------------------
 * An element is two Float64 digits (d1, d2), d1 in [0, N1), d2 in [0, N2), of
 * the value d1 + N1*d2 in Z/(N1*N2) (KaratsubaMatrix.jl:304,318-336).  Each
 * digit matrix is column-major with its own padding, and both digit matrices of
 * one operand share the leading dimension.  Results are the exact digits in
 * Z/(N1*N2); they equal the reference's kernels whenever N2 divides N1 (all
 * modulus pairs the reference constructs).
 *
 * KMatMul!(C, A, B) (KaratsubaMatrix.jl:133-204, kernels KaratsubaKernels.jl:129-158)
 * and KMatMul_gemv! (:238-300, n = 1): three component products on the limb
 * tensor-core GEMM plus a digit combine; 2 <= N1, N2 < 2^26.  C must not alias
 * A or B.  Workspace: gffm_karatsuba_workspace_size bytes, or NULL. */
GFFM_API int gffm_karatsuba_workspace_size(int64_t m, int64_t n, int64_t k, int64_t N1, int64_t N2, size_t *bytes);
GFFM_API int gffm_karatsuba_matmul_f64(int64_t m, int64_t n, int64_t k, const double *A1, const double *A2,
                                       int64_t lda, const double *B1, const double *B2, int64_t ldb, double *C1,
                                       double *C2, int64_t ldc, int64_t N1, int64_t N2, void *workspace,
                                       size_t workspace_bytes, gffm_stream_t stream);
/* The polynomial reading of the same three products (no reference entry
 * point; the two-component Karatsuba product of KaratsubaMatrix.jl:133-204
 * without carries): (A0 + A1 x)(B0 + B1 x) mod p = C0 + C1 x + C2 x^2 with
 * C0 = A0 B0, C2 = A1 B1, C1 = (A0 + A1)(B0 + B1) - C0 - C2; 2 <= p < 2^26.
 * Outputs must not alias inputs.  Workspace: gffm_karatsuba_poly_workspace_size. */
GFFM_API int gffm_karatsuba_poly_workspace_size(int64_t m, int64_t n, int64_t k, int64_t p, size_t *bytes);
GFFM_API int gffm_karatsuba_poly_matmul_f64(int64_t m, int64_t n, int64_t k, const double *A0, const double *A1,
                                            int64_t lda, const double *B0, const double *B1, int64_t ldb, double *C0,
                                            double *C1, double *C2, int64_t ldc, int64_t p, void *workspace,
                                            size_t workspace_bytes, gffm_stream_t stream);
/* Elementwise digit ops over `len` elements of the (padded) digit arrays;
 * N1*N2 <= 2^52.  add!(K, A, B) -> karatsuba_add_kernel! (KaratsubaMatrix.jl:505-536,
 * KaratsubaKernels.jl:2-50) */
GFFM_API int gffm_karatsuba_add_f64(double *C1, double *C2, const double *A1, const double *A2, const double *B1,
                                    const double *B2, int64_t len, int64_t N1, int64_t N2, gffm_stream_t stream);
/* sub!(K, A, B) -> karatsuba_sub_kernel! (KaratsubaMatrix.jl:583-629, KaratsubaKernels.jl:113-125) */
GFFM_API int gffm_karatsuba_sub_f64(double *C1, double *C2, const double *A1, const double *A2, const double *B1,
                                    const double *B2, int64_t len, int64_t N1, int64_t N2, gffm_stream_t stream);
/* negate!(K, A) -> karatsuba_negate_kernel! (KaratsubaMatrix.jl:691-731, KaratsubaKernels.jl:79-111) */
GFFM_API int gffm_karatsuba_negate_f64(double *C1, double *C2, const double *A1, const double *A2, int64_t len,
                                       int64_t N1, int64_t N2, gffm_stream_t stream);
/* scalar_multiply!(B, A, s) -> karatsuba_scalar_multiply_kernel! (KaratsubaMatrix.jl:631-666,
 * KaratsubaKernels.jl:52-77); any integer s (reduced mod N1*N2) */
GFFM_API int gffm_karatsuba_scalar_mul_f64(double *C1, double *C2, const double *A1, const double *A2, int64_t s,
                                           int64_t len, int64_t N1, int64_t N2, gffm_stream_t stream);
/* MatToKMat / KaratsubaMatrix(T, A, N1, N2, M) digit split (KaratsubaMatrix.jl:358-397):
 * D1 = a mod N1, D2 = floor(a / N1) mod N2 for each (non-negative) value a */
GFFM_API int gffm_karatsuba_from_values_f64(double *D1, double *D2, const double *A, int64_t len, int64_t N1,
                                            int64_t N2, gffm_stream_t stream);
/* Array(K) / getindex (KaratsubaMatrix.jl:304,318-336): A = D1 + N1*D2 */
GFFM_API int gffm_karatsuba_to_values_f64(double *A, const double *D1, const double *D2, int64_t len, int64_t N1,
                                          int64_t N2, gffm_stream_t stream);

/* ---- batched uneven instances ---------------------------------------------
 * No reference entry point: the reference runs one CuModMatrix product
 * (mul!, CuModMatrix.jl:767-787) or one pluq_gpu_kernel (pluq_kernels.jl:46-157)
 * per call.  A batch holds thousands of independent instances, each with its
 * own sizes and modulus (2 <= N < 2^26), each a product or a PLUQ with the
 * semantics of those calls.  Products run in one grouped tcgen05 kernel over
 * all instances' output tiles.  Square PLUQs of n = 32k >= 64 rows with an odd
 * prime (and l_cols >= n) run in panel steps: per step one launch factors a
 * 32-column panel of every running instance and a grouped tcgen05 GEMM applies
 * all their trailing updates; an instance that loses rank in a panel, and every
 * other PLUQ, runs in one persistent kernel (a CTA per instance).  Both give
 * the same factorization.  A plan validates the batch, lays out its workspace,
 * encodes the per-instance TMA descriptors and captures the launches in a CUDA
 * graph once.  A plan is bound to the buffers its descriptors name. */
enum gffm_batch_op { GFFM_BATCH_MATMUL = 0, GFFM_BATCH_PLUQ = 1 };

typedef struct gffm_batch_desc {
    int64_t op;            /* gffm_batch_op */
    int64_t m, n, k;       /* MATMUL: C (m x n) = A (m x k) * B (k x n) mod N; PLUQ: A is m x n */
    int64_t N;
    const double *A;       /* column-major Float64 residues (device) */
    int64_t lda;
    const double *B;       /* MATMUL */
    int64_t ldb;
    double *C;             /* MATMUL: the product; PLUQ: U (may alias A) */
    int64_t ldc;
    double *L;             /* PLUQ: m x l_cols (the reference's L has l_cols = m + 32) */
    int64_t ldl;
    int64_t l_cols;
    int64_t *row_swaps;    /* PLUQ, device, capacity 2*m: 1-based (i, j) pairs */
    int64_t *col_swaps;    /* PLUQ, device, capacity 2*n */
    int64_t *info;         /* PLUQ, device int64[4]: #row swaps, #col swaps, rank, status (0 or GFFM_ERR_BOUNDS) */
} gffm_batch_desc;

/* Tuning of a plan; 0 in a field picks the default.  pluq_panel: 0 takes the
 * panel-step route where it applies (32-column panels elsewhere); 8, 16 or 32
 * factor every PLUQ in the persistent kernel with that panel width;
 * gemm_ctas / pluq_ctas: persistent grid sizes; overlap: 1 runs
 * the products and the PLUQs on two graph branches at once; digit_bits: 7 or 8
 * for every product (0: per instance, whichever needs fewer digits). */
typedef struct gffm_batch_tuning {
    int32_t pluq_panel;
    int32_t gemm_ctas;
    int32_t pluq_ctas;
    int32_t overlap;
    int32_t digit_bits;
} gffm_batch_tuning;

typedef struct gffm_batch_plan_s *gffm_batch_plan;

GFFM_API int gffm_batched_plan_create(const gffm_batch_desc *descs, int64_t count, const gffm_batch_tuning *tuning,
                                      gffm_batch_plan *plan);
/* info[0..5]: device bytes held, products, PLUQs, product output tiles, gemm CTAs, PLUQ CTAs */
GFFM_API int gffm_batched_plan_info(gffm_batch_plan plan, int64_t *info);
/* Launch the plan's graph on `stream` (asynchronous; the PLUQ results are in the descriptors' device arrays).
 * PLUQ instances of more than 1024 rows are not in the graph: after it, run
 * factors them one by one with the single-matrix elimination (gffm_pluq_f64)
 * on the same stream, which synchronizes the stream, and fills the same
 * descriptor arrays. */
GFFM_API int gffm_batched_run(gffm_batch_plan plan, gffm_stream_t stream);
GFFM_API int gffm_batched_plan_destroy(gffm_batch_plan plan);

/* ---- limb GEMM without allocation -----------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory when they multiply: a process whose HBM is already reserved by
 * another allocator (a framework pool holding nearly the whole device) would
 * get an out-of-memory error from the workspace allocation, and a pipeline
 * that must not stall cannot accept the device-wide synchronization of
 * cudaMalloc/cudaFree.  This variant of gffm_matmul_limb_f64 takes inputs and
 * outputs only; its digit-plane scratch is a fixed array of
 * gffm_matmul_limb_static_max_bytes() bytes (32 MiB) that the library keeps
 * on every GPU that loads it until the process exits.  It calls no
 * allocator.  It always forms the products the untuned way (7-bit schoolbook
 * digits, whatever the tune table says), so its scratch need is
 * gffm_matmul_limb_static_scratch_size, which can differ from
 * gffm_matmul_limb_workspace_size; a product needing more than the array
 * holds is rejected with GFFM_ERR_WORKSPACE.  The results equal
 * gffm_matmul_limb_f64's bit for bit.  The first call on a device (and the
 * first after cudaDeviceReset, which replaces the device's context) looks up
 * the array's device address; make that call before any stream capture on
 * that device.  All calls share the array: calls that run concurrently on the
 * GPU (e.g. on two streams) race on it, calls on one stream are safe.  Every
 * call rewrites the scratch it uses, so nothing in it needs to start at zero. */
GFFM_API int gffm_matmul_limb_static_max_bytes(size_t *bytes);
GFFM_API int gffm_matmul_limb_static_scratch_size(int64_t m, int64_t n, int64_t k, int64_t N, size_t *bytes);
GFFM_API int gffm_matmul_limb_static_f64(int64_t m, int64_t n, int64_t k, const double *A, int64_t lda,
                                         const double *B, int64_t ldb, double *C, int64_t ldc, int64_t N,
                                         gffm_stream_t stream);

/* ---- triangular inverses and substitutions (src/CuModMatrix/triangular) ----
 * 2 <= N < 2^26.  A is m x n (lda); the result X is n x m (ldx >= n), the
 * reference's transposed shape.  Only A's triangle is read (diagonal and the
 * upper or lower side); entries outside A count as zero, as the reference's
 * zero padding does.  The pivot inverses are the reference's mod_inv (0 for a
 * zero diagonal entry).
 *
 * gffm_tri_sub32_*: forward_sub_gpu_type_32 (upper = 0) / backward_sub_gpu_type_32
 * (upper = 1) (substitution_inplace.jl:6-88): the inverse of the 32 x 32
 * triangular window of A at (row_shift, col_shift), the diagonal read at
 * (row_shift + r, row_shift + r) as the reference does, written to
 * X[0:min(32, n)][0:min(32, m)]; the rest of X is not touched.
 *
 * gffm_triangular_inverse_*: upper_triangular_inverse_no_copy (upper = 1) /
 * lower_triangular_inverse_no_copy (upper = 0) (triangular_inverse_no_copy.jl:
 * 18-477): the reference's block recursion on the leading k x k triangle, k =
 * min(m, n) (halves split at multiples of 32, 32-blocks by substitution, the
 * off-diagonal blocks -X11 A12 X22 / -X22 A21 X11 by the limb GEMM), written to
 * X's leading k x k, zero elsewhere in X: the inverse for an invertible diagonal,
 * the inverse of the leading square block zero-extended for tall / wide input.
 * Lower and tall (m > n > 32) is GFFM_ERR_SIZE, the reference's
 * InverseNotDefinedException.  Workspace: gffm_triangular_inverse_workspace_size
 * bytes, or NULL. */
GFFM_API int gffm_tri_sub32_f64(int upper, int64_t m, int64_t n, const double *A, int64_t lda, int64_t row_shift,
                                int64_t col_shift, double *X, int64_t ldx, int64_t N, gffm_stream_t stream);
GFFM_API int gffm_tri_sub32_f32(int upper, int64_t m, int64_t n, const float *A, int64_t lda, int64_t row_shift,
                                int64_t col_shift, float *X, int64_t ldx, int64_t N, gffm_stream_t stream);
GFFM_API int gffm_triangular_inverse_workspace_size(int upper, int64_t m, int64_t n, int64_t N, size_t *bytes);
GFFM_API int gffm_triangular_inverse_f64(int upper, int64_t m, int64_t n, const double *A, int64_t lda, double *X,
                                         int64_t ldx, int64_t N, void *workspace, size_t workspace_bytes,
                                         gffm_stream_t stream);
GFFM_API int gffm_triangular_inverse_f32(int upper, int64_t m, int64_t n, const float *A, int64_t lda, float *X,
                                         int64_t ldx, int64_t N, void *workspace, size_t workspace_bytes,
                                         gffm_stream_t stream);

/* ---- limb GEMM on host buffers (the round trip Array -> CuModMatrix -> * ->
 * Array of the reference, CuModMatrix.jl:767-787 with the copies of
 * CuModMatrix(A, N) and Array(C)) ---------------------------------------------
 * C = A*B mod N with A (m x k, lda), B (k x n, ldb) and C (m x n, ldc) in HOST
 * memory, column-major Float64, 2 <= N < 2^26, the same results as
 * gffm_matmul_limb_f64.  A is cut into row blocks and B into column blocks of
 * about 2048; the blocks are copied in on one stream while the block products already resident run on
 * two others, and each finished block of C is copied back on a fourth, so
 * only the first block pair's copy and the last block's copy back are not
 * hidden behind the products.  The library's internal
 * streams wait for the work already on `stream`, and `stream` waits for all of
 * the call: C is complete once `stream` is.  The host buffers must stay
 * valid until then; page-locked buffers (cudaHostAlloc / cudaHostRegister)
 * make the copies asynchronous, pageable ones still give correct results.
 * Workspace: gffm_matmul_host_workspace_size bytes of device memory (staging
 * copies of A, B, C and their digit planes), or NULL. */
GFFM_API int gffm_matmul_host_workspace_size(int64_t m, int64_t n, int64_t k, int64_t N, size_t *bytes);
GFFM_API int gffm_matmul_host_f64(int64_t m, int64_t n, int64_t k, const double *A, int64_t lda, const double *B,
                                  int64_t ldb, double *C, int64_t ldc, int64_t N, void *workspace,
                                  size_t workspace_bytes, gffm_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* GFFM_H */
