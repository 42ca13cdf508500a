"""The benchmark configurations checked at their stated sizes.

* 512 x 512 product mod 65521 (the reference's single-stripe `*`, mul_ops.jl:54-58
  -> stripe_mul.jl:212-216): exact against the oracle on the limb and the plain path,
  Float64 and Float32 storage.
* Full-rank 16384 x 16384 PLUQ mod 67108859 (pluq_kernels.jl:46-157): Freivalds'
  L U x = P A x on two vectors, a unit upper U and a lower L with the pivots on
  its diagonal (sampled rows), no column swaps, and the first 256 pivot steps
  (row swaps, U's leading square, L's first columns) equal to the oracle's
  factorization of the leading 16384 x 256 column block.
* The full 4096-instance batched workload: every product C = A B and every PLUQ
  L U = P A checked by Freivalds (exact, on the host), every PLUQ full rank.
"""
import numpy as np
import pytest

import oracle
from oracle import checks

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

P26 = 67108859


def dev_int64(M):
    """The true-size contents of a CuModArray as an int64 (rows x cols) Fortran-ordered array."""
    r, c = M.size
    return M.data[:c, :r].to(torch.int64).cpu().numpy().T


@pytest.mark.parametrize("dtype", ["float64", "float32"])
@pytest.mark.parametrize("method", ["limb", "plain"])
def test_config1_product_512_mod_65521(gffm, method, dtype):
    rng = np.random.default_rng(512)
    A = rng.integers(0, 65521, size=(512, 512))
    B = rng.integers(0, 65521, size=(512, 512))
    dt = getattr(torch, dtype)
    Ag = gffm.CuModMatrix(A, 65521, elem_type=dt)
    Bg = gffm.CuModMatrix(B, 65521, elem_type=dt)
    want = oracle.matmul(A, B, 65521)
    if method == "plain" and dtype == "float32":
        # 65520^2 exceeds Float32's 24-bit mantissa: the reference's stripe bound is 0 and it
        # throws "cannot perform a single multiplication" (stripe_mul.jl:200-202)
        with pytest.raises(gffm.GFFMError, match="cannot perform a single multiplication"):
            gffm.mat_mul_gpu_type(Ag, Bg, method=method)
        return
    C = gffm.mat_mul_gpu_type(Ag, Bg, method=method)
    assert np.array_equal(dev_int64(C), want)
    # the reference's `*` on the same operands (auto method)
    assert np.array_equal(dev_int64(Ag * Bg), want)
    assert gffm.load_library().gffm_device_status(None) == 0


def test_config5_pluq_16384(gffm):
    n = 16384
    g = torch.Generator(device="cuda")
    g.manual_seed(4321)                       # the benchmark's seed for this matrix
    A = gffm.rand(torch.float64, n, n, P26, generator=g)
    U, L, rs, cs = gffm.pluq_gpu_kernel(A)
    assert cs == []
    assert gffm.load_library().gffm_device_status(None) == 0
    Ah, Uh = dev_int64(A), dev_int64(U)
    Lh = dev_int64(L)
    rng = np.random.default_rng(16384)
    assert checks.freivalds_pluq(Ah, Uh, Lh, rs, P26, rng)
    assert (np.diag(Uh) == 1).all()
    # L's diagonal holds the pivots (non-zero); L strictly upper and U strictly lower are zero (sampled rows)
    assert (np.diag(Lh) != 0).all()
    for i in rng.integers(0, n, size=64):
        assert (Uh[i, :i] == 0).all() and (Lh[i, i + 1:] == 0).all()
    w = 256
    res = checks.pluq_leading_block(Ah[:, :w], Uh[:w, :w], Lh[:, :w], rs, P26)
    assert all(res.values()), res


def test_config4_full_batch(gffm):
    from gffm import batched
    specs = batched.config4_specs(4096, seed=1234)
    g = torch.Generator(device="cuda")
    g.manual_seed(1234)
    inst = batched.build_config4(specs, generator=g)
    plan = gffm.BatchPlan(inst, "auto")
    res = plan.run().results()
    assert gffm.load_library().gffm_device_status(None) == 0
    rng = np.random.default_rng(4096)
    bad = []
    for i, ((op, n, p), spec, got) in enumerate(zip(specs, inst, res)):
        if op == "matmul":
            ok = checks.freivalds_product(dev_int64(spec[1]), dev_int64(spec[2]), dev_int64(got), p, rng)
        else:
            U, L, rs, cs = got
            Uh = dev_int64(U)
            ok = (cs == [] and (np.diag(Uh) == 1).all()
                  and checks.freivalds_pluq(dev_int64(spec[1]), Uh, dev_int64(L), rs, p, rng))
        if not ok:
            bad.append(i)
    assert bad == []
