/*
 * gffm_oracle.c -- CPU restatement of GPUFiniteFieldMatrices.jl's hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: tests/, the
 * smoke check in __graft_entry__.py and the cpu_baseline / reference arm of
 * bench.py may call it, always as the checker or the timed CPU baseline and
 * never as part of the product path.  The CUDA library does not link it.
 *
 * Every routine restates one function of the reference (citations are paths
 * inside the GPUFiniteFieldMatrices.jl source tree).  Arithmetic is exact
 * integer arithmetic: the reference computes with Float32/Float64 values that
 * hold integers, and for moduli where its floating-point arithmetic is exact
 * (products below 2^53 for Float64) the two agree bit for bit.  The one place
 * where the reference itself is inexact -- the Float32 staging of the pivot
 * row in update_sub_matrix_kernel (src/CuModMatrix/rref_lu_pluq/
 * pluq_kernels.jl:421), which rounds residues >= 2^24 -- is NOT reproduced:
 * the oracle models the reference's algorithm as if every step were exact.
 *
 * Layout: every matrix is column-major with an explicit leading dimension,
 * as CuModArray.data is in the reference (src/CuModMatrix/CuModMatrix.jl:42-99).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef unsigned __int128 u128;
typedef __int128 i128;

/* Julia mod(x, N) for N > 0: the non-negative remainder
 * (used by k_mod!, src/CuModMatrix/kernel_ops/mod_ops.jl:3-11). */
static inline int64_t or_modi(int64_t x, int64_t N) {
    int64_t r = x % N;
    return r < 0 ? r + N : r;
}

static inline int64_t or_mod128(i128 x, int64_t N) {
    i128 r = x % (i128)N;
    if (r < 0) r += N;
    return (int64_t)r;
}

/* a*b mod N for 0 <= a, b < N.  Below 2^26 the product is < 2^52 and a
 * double-precision quotient estimate is within one of the truth. */
static inline int64_t or_mulmod(int64_t a, int64_t b, int64_t N) {
    if (N < (INT64_C(1) << 26)) {
        int64_t x = a * b;
        int64_t q = (int64_t)((double)x / (double)N);
        int64_t r = x - q * N;
        while (r < 0) r += N;
        while (r >= N) r -= N;
        return r;
    }
    return or_mod128((i128)a * (i128)b, N);
}

int64_t or_mod(int64_t x, int64_t N) { return or_modi(x, N); }

/* mod_inv(p, P): extended Euclid exactly as src/CuModMatrix/rref_lu_pluq/
 * pluq_kernels.jl:11-31 (result in [0, P) when gcd(p, P) = 1). */
int64_t or_mod_inv(int64_t p, int64_t P) {
    int64_t inv = 0, new_inv = 1, rem = P, new_rem = p;
    while (new_rem != 0) {
        int64_t q = rem / new_rem;   /* div() on non-negative values */
        int64_t t = inv - q * new_inv;
        inv = new_inv; new_inv = t;
        t = rem - q * new_rem;
        rem = new_rem; new_rem = t;
    }
    if (inv < 0) inv += P;
    return inv;
}

/* find_max_stripe_ops(type, N), src/CuModMatrix/kernel_mul/stripe_mul.jl:13-27:
 * floor((2^bits - 1) / (N-1)^2) - 1 with bits = 53 (Float64) / 24 (Float32). */
int64_t or_find_max_stripe_ops(int bits, int64_t N) {
    if (N <= 1) return INT64_MAX;
    double num = (double)((INT64_C(1) << bits) - 1);
    double den = (double)(N - 1) * (double)(N - 1);
    return (int64_t)(num / den) - 1;
}

/* ---------------------------------------------------------------------- */
/* Dense modular GEMM: C = A*B mod N (stripe_mul!, stripe_mul.jl:175-244). */
/* The stripes of the reference only bound float overflow; the mathematical */
/* result is the exact product reduced mod N, which is what is computed.    */
/* ---------------------------------------------------------------------- */
void or_matmul(int64_t m, int64_t n, int64_t k,
               const int64_t *A, int64_t lda, const int64_t *B, int64_t ldb,
               int64_t *C, int64_t ldc, int64_t N, int nthreads) {
    if (m <= 0 || n <= 0) return;
    if (k <= 0) {
        for (int64_t j = 0; j < n; j++)
            for (int64_t i = 0; i < m; i++) C[i + j * ldc] = 0;
        return;
    }
    if (N <= (INT64_C(1) << 32)) {
        /* operands fit 32 bits: 64-bit partial sums, reduced every `chunk` products */
        uint64_t nm1 = (uint64_t)(N - 1);
        uint64_t chunk = nm1 == 0 ? (uint64_t)k : (UINT64_MAX - nm1) / (nm1 * nm1);
        if (chunk > 4096) chunk = 4096;
        if (chunk < 1) chunk = 1;
        uint32_t *At = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)m * (size_t)k);
        uint32_t *Bt = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)n * (size_t)k);
#ifdef _OPENMP
        if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
        /* operands as uint32 residues, both k-contiguous (A transposed, B as is) */
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
        for (int64_t i = 0; i < m; i++)
            for (int64_t p = 0; p < k; p++) {
                int64_t v = A[i + p * lda];
                At[i * k + p] = (uint32_t)((v >= 0 && v < N) ? v : or_modi(v, N));
            }
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
        for (int64_t j = 0; j < n; j++)
            for (int64_t p = 0; p < k; p++) {
                int64_t v = B[p + j * ldb];
                Bt[j * k + p] = (uint32_t)((v >= 0 && v < N) ? v : or_modi(v, N));
            }
        /* 4 rows x 1 column per inner loop: each b[p] load feeds four products */
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 4)
#endif
        for (int64_t j = 0; j < n; j++) {
            const uint32_t *b = Bt + j * k;
            int64_t i = 0;
            for (; i + 4 <= m; i += 4) {
                const uint32_t *a0 = At + i * k, *a1 = a0 + k, *a2 = a1 + k, *a3 = a2 + k;
                uint64_t r0 = 0, r1 = 0, r2 = 0, r3 = 0;
                for (int64_t p0 = 0; p0 < k; p0 += (int64_t)chunk) {
                    int64_t p1 = p0 + (int64_t)chunk < k ? p0 + (int64_t)chunk : k;
                    uint64_t s0 = 0, s1 = 0, s2 = 0, s3 = 0;
                    for (int64_t p = p0; p < p1; p++) {
                        uint64_t bv = b[p];
                        s0 += (uint64_t)a0[p] * bv;
                        s1 += (uint64_t)a1[p] * bv;
                        s2 += (uint64_t)a2[p] * bv;
                        s3 += (uint64_t)a3[p] * bv;
                    }
                    r0 = (r0 + s0 % (uint64_t)N) % (uint64_t)N;
                    r1 = (r1 + s1 % (uint64_t)N) % (uint64_t)N;
                    r2 = (r2 + s2 % (uint64_t)N) % (uint64_t)N;
                    r3 = (r3 + s3 % (uint64_t)N) % (uint64_t)N;
                }
                C[i + j * ldc] = (int64_t)r0;
                C[i + 1 + j * ldc] = (int64_t)r1;
                C[i + 2 + j * ldc] = (int64_t)r2;
                C[i + 3 + j * ldc] = (int64_t)r3;
            }
            for (; i < m; i++) {
                const uint32_t *a = At + i * k;
                uint64_t res = 0;
                for (int64_t p0 = 0; p0 < k; p0 += (int64_t)chunk) {
                    int64_t p1 = p0 + (int64_t)chunk < k ? p0 + (int64_t)chunk : k;
                    uint64_t s = 0;
                    for (int64_t p = p0; p < p1; p++) s += (uint64_t)a[p] * (uint64_t)b[p];
                    res = (res + s % (uint64_t)N) % (uint64_t)N;
                }
                C[i + j * ldc] = (int64_t)res;
            }
        }
        free(At);
        free(Bt);
        return;
    }
    /* wide moduli (Karatsuba N1*N2): exact 128-bit sums */
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 4)
#endif
    for (int64_t j = 0; j < n; j++)
        for (int64_t i = 0; i < m; i++) {
            i128 s = 0;
            for (int64_t p = 0; p < k; p++) {
                s += (i128)or_modi(A[i + p * lda], N) * (i128)or_modi(B[p + j * ldb], N);
                s %= (i128)N;
            }
            C[i + j * ldc] = (int64_t)s;
        }
}

/* ---------------------------------------------------------------------- */
/* PLUQ: step-by-step restatement of pluq_gpu_kernel                       */
/* (src/CuModMatrix/rref_lu_pluq/pluq_kernels.jl:46-157) with its helpers: */
/*   find_pivot :179-202 (max residue in column below row, first index on  */
/*     ties -- GPUArrays findmax; zero column => swap with the constant    */
/*     last column `cols`, push (col, cols), and the caller advances col   */
/*     without re-examining the column that was swapped in, :97-108)       */
/*   swap_and_mod :247-264 / swap_rows_and_mod :307-320 (row `row` <- old  */
/*     row prow scaled by the pivot inverse, over all columns 1..cols;     */
/*     row prow <- old row `row`; full rows of L swapped; (row, prow)      */
/*     pushed only when they differ)                                       */
/*   move_and_zero_out :340-351 (L[row, col] = pivot -- column index col,  */
/*     not row; L[r, col] = A[r, col] and A[r, col] = 0 below the pivot)   */
/*   update_sub_matrix_kernel :411-440 (A[r,c] = mod(A[r,c] +             */
/*     (N - L[r,col]) * A[row,c], N) for r > row, c > col)                 */
/*                                                                         */
/* A (m x n, lda) is overwritten with U.  L (m x l_cols, ldl) must be      */
/* zero on entry; l_cols is the padded width of L in the reference's       */
/* layout (m + 32).  Swap stacks are 1-based (i, j) pairs, in order.       */
/* Returns 0, or 8 when the reference would index L out of bounds.         */
/* ---------------------------------------------------------------------- */
int or_pluq(int64_t m, int64_t n, int64_t *A, int64_t lda,
            int64_t *L, int64_t ldl, int64_t l_cols, int64_t N,
            int64_t *row_swaps, int64_t *n_row_swaps,
            int64_t *col_swaps, int64_t *n_col_swaps, int64_t *rank) {
    int64_t row = 0, col = 0, last = n - 1;
    int64_t nr = 0, nc = 0, rk = 0;
    while (row < m && col < n) {
        int64_t pv = -1, pidx = -1;
        for (;;) {
            /* find_pivot */
            int64_t best = -1, bi = -1;
            for (int64_t r = row; r < m; r++) {
                int64_t v = A[r + col * lda];
                if (v > best) { best = v; bi = r; }
            }
            if (best > 0) { pv = best; pidx = bi; break; }
            /* zero column: swap_cols(d_A, col, Perm_col_idx) over every row */
            for (int64_t r = 0; r < m; r++) {
                int64_t t = A[r + col * lda];
                A[r + col * lda] = A[r + last * lda];
                A[r + last * lda] = t;
            }
            col_swaps[2 * nc] = col + 1;
            col_swaps[2 * nc + 1] = last + 1;
            nc++;
            col += 1;
            if (col >= n) break;
        }
        if (col >= n) break;
        int64_t inv = or_mod_inv(pv, N);
        int64_t prow = pidx;
        /* swap_rows_and_mod over columns 1..cols */
        for (int64_t c = 0; c < n; c++) {
            int64_t t = A[prow + c * lda];
            A[prow + c * lda] = A[row + c * lda];
            A[row + c * lda] = or_mulmod(t, inv, N);
        }
        /* swap_rows on L: the kernel runs cld(rows, 32) blocks of 32 threads,
         * one per column, so columns 1..32*cld(rows, 32) of L are swapped */
        int64_t l_sw = ((m + 31) / 32) * 32;
        if (l_sw > l_cols) l_sw = l_cols;
        if (prow != row)
            for (int64_t c = 0; c < l_sw; c++) {
                int64_t t = L[row + c * ldl];
                L[row + c * ldl] = L[prow + c * ldl];
                L[prow + c * ldl] = t;
            }
        if (row != prow) {
            row_swaps[2 * nr] = row + 1;
            row_swaps[2 * nr + 1] = prow + 1;
            nr++;
        }
        if (col >= l_cols) return 8;
        /* move_and_zero_out */
        L[row + col * ldl] = pv;
        for (int64_t r = row + 1; r < m; r++) {
            L[r + col * ldl] = A[r + col * lda];
            A[r + col * lda] = 0;
        }
        /* update_sub_matrix_kernel */
        for (int64_t c = col + 1; c < n; c++) {
            int64_t s = A[row + c * lda];
            if (s == 0) continue;
            for (int64_t r = row + 1; r < m; r++) {
                int64_t l = L[r + col * ldl];
                if (l == 0) continue;
                int64_t v = A[r + c * lda] + or_mulmod(N - l, s, N);
                A[r + c * lda] = v >= N ? v - N : v;
            }
        }
        rk++;
        row++;
        col++;
    }
    *n_row_swaps = nr;
    *n_col_swaps = nc;
    *rank = rk;
    return 0;
}

/* ---------------------------------------------------------------------- */
/* LU: lu_gpu_type (intended API, test/Experiments/rref_gpu_type.jl:60-103)*/
/* as the elimination above without column swaps: a zero column is        */
/* skipped (col += 1), the pivot value and multipliers go to L's column    */
/* `row` (the pivot count), and perm tracks the row order (0-based).       */
/* ---------------------------------------------------------------------- */
int or_lu(int64_t m, int64_t n, int64_t *A, int64_t lda, int64_t *L, int64_t ldl, int64_t N,
          int64_t *perm, int64_t *rank) {
    int64_t row = 0, col = 0;
    for (int64_t i = 0; i < m; i++) perm[i] = i;
    while (row < m && col < n) {
        int64_t best = -1, bi = -1;
        for (int64_t r = row; r < m; r++) {
            int64_t v = A[r + col * lda];
            if (v > best) { best = v; bi = r; }
        }
        if (best <= 0) { col++; continue; }
        int64_t inv = or_mod_inv(best, N);
        for (int64_t c = 0; c < n; c++) {
            int64_t t = A[bi + c * lda];
            A[bi + c * lda] = A[row + c * lda];
            A[row + c * lda] = or_mulmod(t, inv, N);
        }
        if (bi != row) {
            for (int64_t c = 0; c < m; c++) {
                int64_t t = L[row + c * ldl];
                L[row + c * ldl] = L[bi + c * ldl];
                L[bi + c * ldl] = t;
            }
            int64_t t = perm[row]; perm[row] = perm[bi]; perm[bi] = t;
        }
        L[row + row * ldl] = best;
        for (int64_t r = row + 1; r < m; r++) {
            L[r + row * ldl] = A[r + col * lda];
            A[r + col * lda] = 0;
        }
        for (int64_t c = col + 1; c < n; c++) {
            int64_t s = A[row + c * lda];
            if (s == 0) continue;
            for (int64_t r = row + 1; r < m; r++) {
                int64_t l = L[r + row * ldl];
                if (l == 0) continue;
                int64_t v = A[r + c * lda] + or_mulmod(N - l, s, N);
                A[r + c * lda] = v >= N ? v - N : v;
            }
        }
        row++;
        col++;
    }
    *rank = row;
    return 0;
}

/* ---------------------------------------------------------------------- */
/* RREF: the reduced row echelon form over Z/p (p prime).  It is unique,   */
/* so any pivot order gives the same matrix; this is plain Gauss-Jordan    */
/* with the first non-zero entry as pivot.  (Intended API:                 */
/* rref_gpu_type, test/Experiments/rref_gpu_type.jl:8-51.)                 */
/* ---------------------------------------------------------------------- */
int or_rref(int64_t m, int64_t n, int64_t *A, int64_t lda, int64_t N,
            int64_t *rank, int64_t *pivot_cols) {
    int64_t row = 0;
    for (int64_t col = 0; col < n && row < m; col++) {
        int64_t pr = -1;
        for (int64_t r = row; r < m; r++)
            if (A[r + col * lda] != 0) { pr = r; break; }
        if (pr < 0) continue;
        if (pr != row)
            for (int64_t c = 0; c < n; c++) {
                int64_t t = A[pr + c * lda];
                A[pr + c * lda] = A[row + c * lda];
                A[row + c * lda] = t;
            }
        int64_t inv = or_mod_inv(A[row + col * lda], N);
        for (int64_t c = col; c < n; c++) A[row + c * lda] = or_mulmod(A[row + c * lda], inv, N);
        for (int64_t c = col + 1; c < n; c++) {
            int64_t s = A[row + c * lda];
            if (s == 0) continue;
            for (int64_t r = 0; r < m; r++) {
                if (r == row) continue;
                int64_t l = A[r + col * lda];
                if (l == 0) continue;
                int64_t v = A[r + c * lda] + or_mulmod(N - l, s, N);
                A[r + c * lda] = v >= N ? v - N : v;
            }
        }
        for (int64_t r = 0; r < m; r++)
            if (r != row) A[r + col * lda] = 0;
        if (pivot_cols) pivot_cols[row] = col;
        row++;
    }
    *rank = row;
    return 0;
}

/* ---------------------------------------------------------------------- */
/* Karatsuba digits (src/KaratsubaMatrix/KaratsubaMatrix.jl:304,318-336:   */
/* an element is d1 + N1*d2 of Z/(N1*N2)).  C = A*B in Z/(N1*N2), returned */
/* as digits (C mod N1, C div N1).  KMatMul! (:133-204) with kernels       */
/* karatsuba_matmul_kernel_1!/2! (KaratsubaKernels.jl:129-158) computes    */
/* this product whenever N2 divides N1 (then N1^2 * A2*B2 vanishes).       */
/* ---------------------------------------------------------------------- */
void or_karatsuba_matmul(int64_t m, int64_t n, int64_t k,
                         const int64_t *A1, const int64_t *A2, int64_t lda,
                         const int64_t *B1, const int64_t *B2, int64_t ldb,
                         int64_t *C1, int64_t *C2, int64_t ldc,
                         int64_t N1, int64_t N2, int nthreads) {
    i128 M = (i128)N1 * (i128)N2;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 4)
#endif
    for (int64_t j = 0; j < n; j++)
        for (int64_t i = 0; i < m; i++) {
            i128 s = 0;
            for (int64_t p = 0; p < k; p++) {
                i128 a = (i128)A1[i + p * lda] + (i128)N1 * A2[i + p * lda];
                i128 b = (i128)B1[p + j * ldb] + (i128)N1 * B2[p + j * ldb];
                a %= M; b %= M;
                /* a, b < 2^63: split b to keep the product inside 128 bits */
                i128 prod = ((a * (b >> 32)) % M * ((i128)1 << 32) + a * (b & 0xffffffff)) % M;
                s = (s + prod) % M;
            }
            C1[i + j * ldc] = (int64_t)(s % N1);
            C2[i + j * ldc] = (int64_t)(s / N1);
        }
}

/* Karatsuba digit add / sub (karatsuba_add_kernel!, karatsuba_sub_kernel!,
 * KaratsubaKernels.jl:2-50,113-125): exact (A +- B) mod N1*N2 as digits. */
void or_karatsuba_addsub(int64_t len, const int64_t *A1, const int64_t *A2,
                         const int64_t *B1, const int64_t *B2,
                         int64_t *C1, int64_t *C2, int64_t N1, int64_t N2, int sub) {
    i128 M = (i128)N1 * (i128)N2;
    for (int64_t i = 0; i < len; i++) {
        i128 a = (i128)A1[i] + (i128)N1 * A2[i];
        i128 b = (i128)B1[i] + (i128)N1 * B2[i];
        i128 c = sub ? a - b : a + b;
        c %= M;
        if (c < 0) c += M;
        C1[i] = (int64_t)(c % N1);
        C2[i] = (int64_t)(c / N1);
    }
}

/* Karatsuba digit negation and scalar product (karatsuba_negate_kernel!,
 * karatsuba_scalar_multiply_kernel!, KaratsubaKernels.jl:52-111): exact
 * (-A) and (s*A) mod N1*N2 as digits, s any integer. */
void or_karatsuba_scale(int64_t len, const int64_t *A1, const int64_t *A2, int64_t s, int negate,
                        int64_t *C1, int64_t *C2, int64_t N1, int64_t N2) {
    i128 M = (i128)N1 * (i128)N2;
    i128 sm = (i128)s % M;
    if (sm < 0) sm += M;
    for (int64_t i = 0; i < len; i++) {
        i128 a = ((i128)A1[i] + (i128)N1 * A2[i]) % M;
        if (a < 0) a += M;
        i128 c = negate ? (M - a) % M : (a * sm) % M;
        C1[i] = (int64_t)(c % N1);
        C2[i] = (int64_t)(c / N1);
    }
}

/* ---- triangular inverses (src/CuModMatrix/triangular) ---- */

static int64_t or_tri_at(const int64_t *A, int64_t lda, int64_t m, int64_t n, int64_t i, int64_t j, int64_t N) {
    return (i >= 0 && j >= 0 && i < m && j < n) ? or_modi(A[i + j * lda], N) : 0; /* the zero padding */
}

/* forward_sub_kernel_32 (upper = 0) / backward_sub_kernel_32 (upper = 1)
 * (substitution_inplace.jl:6-35, 63-88), in exact arithmetic: the inverse of the
 * 32 x 32 triangular window of A (m x n) at (rs, cs), one result column c per
 * reference thread, rows in order (forward) or reverse order (backward):
 *   X[r][c] = mod_inv(A[rs + r][rs + r]) * ([r == c] - sum_k A[rs + r][cs + k] X[k][c]) mod N,
 * k < r (forward) or k > r (backward).  X is 32 x 32, column-major. */
void or_tri_window(int upper, int64_t m, int64_t n, const int64_t *A, int64_t lda, int64_t rs, int64_t cs,
                   int64_t N, int64_t *X) {
    for (int c = 0; c < 32; c++) {
        for (int q = 0; q < 32; q++) {
            const int r = upper ? 31 - q : q;
            i128 sum = 0;
            if (upper) {
                for (int k = r + 1; k < 32; k++) sum += (i128)or_tri_at(A, lda, m, n, rs + r, cs + k, N) * X[k + 32 * c];
            } else {
                for (int k = 0; k < r; k++) sum += (i128)or_tri_at(A, lda, m, n, rs + r, cs + k, N) * X[k + 32 * c];
            }
            const int64_t rhs = (r == c) ? 1 : 0;
            const int64_t d = or_mod_inv(or_tri_at(A, lda, m, n, rs + r, rs + r, N), N);
            X[r + 32 * c] = or_mulmod(d, or_mod128((i128)rhs - sum, N), N);
        }
    }
}

/* _recursive_upper/lower_triangular_inverse_no_copy (triangular_inverse_no_copy.jl:
 * 18-195, 246-448) on the square block [lo, hi) of the leading triangle: a block
 * of at most 32 by its window; otherwise the split mid = lo + 32 * q with
 * q = floor(size / 64 + 1/2), both halves (the reference's second branch does
 * them by window directly, its third by recursion -- the same blocks), then
 *   upper: X[lo:mid][mid:hi] = -(X11 A12 mod N) X22 mod N
 *   lower: X[mid:hi][lo:mid] = -(X22 A21 mod N) X11 mod N.
 * X is column-major with leading dimension ldx. */
static void or_tri_rec(int upper, int64_t m, int64_t n, const int64_t *A, int64_t lda, int64_t N, int64_t lo,
                       int64_t hi, int64_t *X, int64_t ldx) {
    const int64_t s = hi - lo;
    if (s <= 32) {
        int64_t W[32 * 32];
        or_tri_window(upper, m, n, A, lda, lo, lo, N, W);
        for (int64_t c = 0; c < s; c++)
            for (int64_t r = 0; r < s; r++) X[(lo + r) + (lo + c) * ldx] = W[r + 32 * c];
        return;
    }
    int64_t q = (int64_t)((double)s / 64.0 + 0.5);
    if (q < 1) q = 1;
    const int64_t mid = lo + 32 * q, s1 = mid - lo, s2 = hi - mid;
    or_tri_rec(upper, m, n, A, lda, N, lo, mid, X, ldx);
    or_tri_rec(upper, m, n, A, lda, N, mid, hi, X, ldx);
    /* T = first product (s1 x s2 upper, s2 x s1 lower), then the block */
    int64_t *T = (int64_t *)malloc(sizeof(int64_t) * (size_t)(s1 * s2));
    if (upper) {
        for (int64_t j = 0; j < s2; j++)
            for (int64_t i = 0; i < s1; i++) {
                i128 acc = 0;
                for (int64_t t = 0; t < s1; t++)
                    acc += (i128)X[(lo + i) + (lo + t) * ldx] * or_tri_at(A, lda, m, n, lo + t, mid + j, N);
                T[i + j * s1] = or_mod128(acc, N);
            }
        for (int64_t j = 0; j < s2; j++)
            for (int64_t i = 0; i < s1; i++) {
                i128 acc = 0;
                for (int64_t t = 0; t < s2; t++) acc += (i128)T[i + t * s1] * X[(mid + t) + (mid + j) * ldx];
                X[(lo + i) + (mid + j) * ldx] = or_mod128(-acc, N);
            }
    } else {
        for (int64_t j = 0; j < s1; j++)
            for (int64_t i = 0; i < s2; i++) {
                i128 acc = 0;
                for (int64_t t = 0; t < s2; t++)
                    acc += (i128)X[(mid + i) + (mid + t) * ldx] * or_tri_at(A, lda, m, n, mid + t, lo + j, N);
                T[i + j * s2] = or_mod128(acc, N);
            }
        for (int64_t j = 0; j < s1; j++)
            for (int64_t i = 0; i < s2; i++) {
                i128 acc = 0;
                for (int64_t t = 0; t < s1; t++) acc += (i128)T[i + t * s2] * X[(lo + t) + (lo + j) * ldx];
                X[(mid + i) + (lo + j) * ldx] = or_mod128(-acc, N);
            }
    }
    free(T);
}

/* upper_triangular_inverse_no_copy (upper = 1, triangular_inverse_no_copy.jl:197-245)
 * / lower_triangular_inverse_no_copy (upper = 0, :450-477) of A (m x n): X is
 * n x m (ld n), zero-initialised here.  A single window when rows (upper) or
 * columns (lower) are at most 32 (the window fills X's leading min(32, n) x
 * min(32, m)); lower and tall beyond that is the reference's
 * InverseNotDefinedException (returns 2); otherwise the recursion on the leading
 * min(m, n) square. */
int or_tri_inverse(int upper, int64_t m, int64_t n, const int64_t *A, int64_t lda, int64_t N, int64_t *X) {
    const int64_t ldx = n;
    for (int64_t e = 0; e < n * m; e++) X[e] = 0;
    if (upper ? m <= 32 : n <= 32) {
        int64_t W[32 * 32];
        or_tri_window(upper, m, n, A, lda, 0, 0, N, W);
        for (int64_t c = 0; c < (m < 32 ? m : 32); c++)
            for (int64_t r = 0; r < (n < 32 ? n : 32); r++) X[r + c * ldx] = W[r + 32 * c];
        return 0;
    }
    if (!upper && m > n) return 2;
    const int64_t k = m < n ? m : n;
    or_tri_rec(upper, m, n, A, lda, N, 0, k, X, ldx);
    return 0;
}
