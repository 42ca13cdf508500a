"""The integer arithmetic of the tensor-core GEMMs' fast drain, restated and checked
at its bounds on the CPU (the GPU parity tests run the kernels themselves).

A shift sum C (|C| <= 2^22) is exact in fp32; adding 1.5 * 2^23 puts 0x4B400000 + C in
the word's bits.  With 7-bit digits shifts s and s + 1 are read as one int32,
bits_s + (bits_{s+1} << 7) in wrapping arithmetic, which is C_s + 2^7 C_{s+1} plus the
constant 129 * 0x4B400000 mod 2^32; one wide multiply-add by Wm[s] = 2^(7s) 2^32 mod N
takes the pair.  The constants go into the initial value, which keeps the sum x in
(0, 2^32 N), so one Montgomery step and one subtraction give x 2^-32 mod N
(gpufinitefieldmatrices.jl_gb300/csrc/gemm_limb.cuh, fast_pair; k_gemm_limb.cu,
fast_consts)."""
import random

import numpy as np

MAGIC_BITS = 0x4B400000
PAIR_OFFSET = -348127232


def i32(x):
    x &= 0xFFFFFFFF
    return x - (1 << 32) if x >= 1 << 31 else x


def fp32_bits(c):
    """Bits of float32(c) + 1.5 * 2^23, as the kernel's FADD forms them."""
    f = np.float32(c) + np.float32(12582912.0)
    return int(np.array(f, dtype=np.float32).view(np.uint32))


def fast_consts(N, L, paired):
    """Paired: 7-bit digits (weights 2^(7s)); single shifts: 8-bit digits (2^(8s))."""
    inv = 1
    for _ in range(5):
        inv = (inv * (2 - N * inv)) & 0xFFFFFFFF
    ninv = (-inv) & 0xFFFFFFFF
    ns = 2 * L - 1
    base = 128 if paired else 256
    Wm = [((pow(base, s, N)) << 32) % N for s in range(7)]
    if paired:
        b = N << 31
        for s in range(0, ns - 1, 2):
            b -= PAIR_OFFSET * Wm[s]
        return ninv, Wm, b - MAGIC_BITS * Wm[ns - 1]
    return ninv, Wm, N * (1 << 25) - MAGIC_BITS * sum(Wm[:ns])


def drain(C, N, L, paired):
    ninv, Wm, acc = fast_consts(N, L, paired)
    ns = 2 * L - 1
    bits = [fp32_bits(c) for c in C]
    step = 2 if paired else 1
    for s in range(0, ns, step):
        d = bits[s]
        if paired and s + 1 < ns:
            d = (d + (bits[s + 1] << 7)) & 0xFFFFFFFF
        acc += i32(d) * Wm[s]
        assert -(1 << 63) <= acc < 1 << 63
    assert 0 < acc < (1 << 32) * N
    m = (acc * ninv) & 0xFFFFFFFF
    t = (acc + m * N) >> 32
    assert t < 2 * N
    return t - N if t >= N else t


def test_magic_number_read_is_exact_at_the_bounds():
    assert i32(129 * MAGIC_BITS) == PAIR_OFFSET
    for c in (-(1 << 22), -1, 0, 1, (1 << 22) - 1, 1 << 22):
        assert fp32_bits(c) == MAGIC_BITS + c


def test_paired_and_single_drains_reduce_exactly():
    rng = random.Random(7)
    lim = 1 << 22
    moduli = [3, 5, 65521, 2080639, 16777213, 33554393, 67108859]
    for trial in range(4000):
        L = rng.choice([1, 2, 3, 4])
        N = rng.choice(moduli + [rng.randrange(3, 1 << 26) | 1])
        if trial % 3 == 0:
            C = [rng.choice([-lim, lim]) for _ in range(2 * L - 1)]
        else:
            C = [rng.randrange(-lim, lim + 1) for _ in range(2 * L - 1)]
        assert drain(C, N, L, True) == sum(c * pow(128, s, N) for s, c in enumerate(C)) % N
        assert drain(C, N, L, False) == sum(c * pow(256, s, N) for s, c in enumerate(C)) % N
