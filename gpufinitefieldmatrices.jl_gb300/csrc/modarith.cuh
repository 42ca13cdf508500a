// modarith.cuh -- 32-bit modular arithmetic for moduli N < 2^26 shared by the
// elimination kernels: Barrett, Shoup and Montgomery multiplication and the
// pivot inverse (the reference's extended Euclid, or Fermat for prime N).
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

// mod_inv(p, P), src/CuModMatrix/rref_lu_pluq/pluq_kernels.jl:11-31: the same
// extended Euclid sequence (exact quotients), so the same result for any P.
// The Bezout coefficients stay below P < 2^26 in magnitude: 32-bit integers.
__device__ __forceinline__ uint32_t mod_inv_euclid(uint32_t p, uint32_t P) {
    int32_t inv = 0, new_inv = 1;
    uint32_t rem = P, new_rem = p;
    while (new_rem != 0) {
        const uint32_t q = udiv26(rem, new_rem);
        const int32_t t = inv - (int32_t)q * new_inv;
        inv = new_inv;
        new_inv = t;
        const uint32_t r2 = rem - q * new_rem;
        rem = new_rem;
        new_rem = r2;
    }
    if (inv < 0) inv += (int32_t)P;
    return (uint32_t)inv;
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

// The same extended Euclid sequence as mod_inv_euclid (so the same result for any
// P), with the quotients 1, 2 and 3 -- about two thirds of them -- found by
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

// Montgomery arithmetic modulo an odd N < 2^26 with R = 2^32:
// mont_mul(a, b) = a * b * R^{-1} mod N for a, b < N (t + m*N < 2^59).
struct Mont {
    uint32_t n, nprime;  // nprime = -N^{-1} mod 2^32
    uint32_t r2;         // R^2 mod N
    int prime;           // N is prime (then the inverse is v^(N-2))
};
__device__ __forceinline__ uint32_t mont_mul(uint32_t a, uint32_t b, const Mont &M) {
    const uint64_t t = (uint64_t)a * b;
    const uint32_t m = (uint32_t)t * M.nprime;
    const uint32_t u = (uint32_t)((t + (uint64_t)m * M.n) >> 32);
    return u >= M.n ? u - M.n : u;
}
// The inverse of v in [1, N): for prime N by Fermat (v^(N-2), square-and-multiply
// in Montgomery form -- the unique inverse, equal to what the reference's Euclid
// returns), otherwise the reference's extended Euclid itself.
__device__ __forceinline__ uint32_t mod_inverse(uint32_t v, const Mont &M) {
    if (!M.prime) return mod_inv_euclid(v, M.n);
    const uint32_t e = M.n - 2;
    const uint32_t vm = mont_mul(v, M.r2, M);
    uint32_t x = vm;
    for (int bit = 30 - __clz(e); bit >= 0; bit--) {
        x = mont_mul(x, x, M);
        if ((e >> bit) & 1u) x = mont_mul(x, vm, M);
    }
    return mont_mul(x, 1u, M);
}

// Shoup's modular multiplication by a fixed u in [0, N): u' = floor(u * 2^32 / N)
// (possibly one less, from floor((2^64 - 1) / N)); then l * u mod N for l in
// [0, N) takes 32-bit operations only.
__device__ __forceinline__ uint32_t shoup_pre(uint32_t u, const ModP &M) {
    return (uint32_t)(((uint64_t)u * M.minv) >> 32);
}
__device__ __forceinline__ uint32_t shoup_mul(uint32_t l, uint32_t u, uint32_t us, uint32_t n) {
    const uint32_t q = __umulhi(l, us);
    uint32_t r = l * u - q * n;  // exact: the true value lies in [0, 3n) < 2^28
    if (r >= n) r -= n;
    if (r >= n) r -= n;
    return r;
}


// host: deterministic Miller-Rabin for 32-bit n (bases 2, 7, 61) and the
// Montgomery constants of n
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

inline Mont make_mont(uint32_t n) {
    Mont M{};
    M.n = n;
    M.prime = (n & 1u) && is_prime_u32(n);
    if (n & 1u) {
        uint32_t inv = n;  // Newton iteration for n^{-1} mod 2^32
        for (int i = 0; i < 5; i++) inv *= 2u - n * inv;
        M.nprime = 0u - inv;
        M.r2 = (uint32_t)(((unsigned __int128)1 << 64) % n);
    }
    return M;
}

}  // namespace elim
