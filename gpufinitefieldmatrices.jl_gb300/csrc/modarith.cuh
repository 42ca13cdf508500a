// modarith.cuh -- 32-bit modular arithmetic for moduli N < 2^26 shared by the
// elimination kernels: Barrett multiplication, the pivot inverse (the
// reference's extended Euclid) and the host-side primality test.
#pragma once

#include "gffm_common.cuh"

namespace elim {

struct ModP {
    uint32_t n;
    uint64_t minv;
};

__device__ __forceinline__ uint32_t mulmod(uint32_t a, uint32_t b, const ModP &M) {
    return (uint32_t)gffm_dev::barrett64((uint64_t)a * b, M.n, M.minv);
}

// floor(a / b) for 0 <= a < 2^26, 1 <= b <= a: float estimate, corrected to the
// exact quotient (32-bit arithmetic; the remainder a - q*b stays below 2^27)
__device__ __forceinline__ uint32_t udiv26(uint32_t a, uint32_t b) {
    int32_t q = (int32_t)__fdividef((float)a, (float)b);
    int32_t r = (int32_t)a - q * (int32_t)b;
    while (r < 0) {
        q--;
        r += (int32_t)b;
    }
    while (r >= (int32_t)b) {
        q++;
        r -= (int32_t)b;
    }
    return (uint32_t)q;
}

// mod_inv(p, P) of the reference (src/CuModMatrix/rref_lu_pluq/pluq_kernels.jl:11-31)
// for any 64-bit p and P > 0 (|P| < 2^62): the extended Euclid sequence with
// truncating division (Julia's div), 0 for p = 0, a non-inverse when gcd(p, P) > 1.
__host__ __device__ inline int64_t ref_mod_inv(int64_t p, int64_t P) {
    int64_t inv = 0, new_inv = 1, rem = P, new_rem = p;
    while (new_rem != 0) {
        const int64_t q = rem / new_rem;
        const int64_t t = inv - q * new_inv;
        inv = new_inv;
        new_inv = t;
        const int64_t r = rem - q * new_rem;
        rem = new_rem;
        new_rem = r;
    }
    if (inv < 0) inv += P;
    return inv;
}

// mod_inv(p, P), src/CuModMatrix/rref_lu_pluq/pluq_kernels.jl:11-31, for
// 0 <= p < P < 2^26: the same extended Euclid sequence (exact quotients, so the
// same result for any P; Bezout coefficients below P in magnitude fit 32 bits),
// with the quotients 1, 2 and 3 -- about two thirds of them -- found by
// comparisons instead of a division: the loop stays on the integer ALU, away from
// the multiply pipe that a concurrent trailing update keeps busy.
__device__ __forceinline__ uint32_t mod_inv_euclid_alu(uint32_t p, uint32_t P) {
    int32_t inv = 0, new_inv = 1;
    uint32_t rem = P, new_rem = p;
    while (new_rem != 0) {
        uint32_t q, r2;
        int32_t t;
        if (rem < 2 * new_rem) {
            q = 1;
            r2 = rem - new_rem;
            t = inv - new_inv;
        } else if (rem < 4 * new_rem) {
            r2 = rem - 2 * new_rem;
            q = 2;
            t = inv - 2 * new_inv;
            if (r2 >= new_rem) {
                r2 -= new_rem;
                q = 3;
                t -= new_inv;
            }
        } else {
            q = udiv26(rem, new_rem);
            r2 = rem - q * new_rem;
            t = inv - (int32_t)q * new_inv;
        }
        inv = new_inv;
        new_inv = t;
        rem = new_rem;
        new_rem = r2;
    }
    if (inv < 0) inv += (int32_t)P;
    return (uint32_t)inv;
}

// host: deterministic Miller-Rabin for 32-bit n (bases 2, 7, 61)
inline bool is_prime_u32(uint32_t n) {
    if (n < 2) return false;
    for (uint32_t p : {2u, 3u, 5u, 7u, 11u, 13u, 61u})
        if (n % p == 0) return n == p;
    uint32_t d = n - 1;
    int s = 0;
    while ((d & 1) == 0) {
        d >>= 1;
        s++;
    }
    auto powm = [n](uint64_t b, uint32_t e) {
        uint64_t r = 1;
        b %= n;
        while (e) {
            if (e & 1) r = r * b % n;
            b = b * b % n;
            e >>= 1;
        }
        return r;
    };
    for (uint32_t a : {2u, 7u, 61u}) {
        uint64_t x = powm(a, d);
        if (x == 1 || x == n - 1) continue;
        bool comp = true;
        for (int i = 1; i < s; i++) {
            x = x * x % n;
            if (x == n - 1) {
                comp = false;
                break;
            }
        }
        if (comp) return false;
    }
    return true;
}

}  // namespace elim
