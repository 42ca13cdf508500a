"""GPU parity tests of the batched uneven-instance form: every product and
every PLUQ of a mixed batch (own sizes, own modulus) bit-exact against the
oracle, for several tunings of the plan."""
import numpy as np
import pytest

import oracle
from test_gpu_elim import make

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

P26 = 67108859
P25 = 33554393

MM = [(1, 1, 1, 2), (5, 7, 3, 7), (130, 200, 70, 65521), (64, 64, 64, P26), (300, 17, 129, 2 ** 20),
      (128, 512, 64, 1021), (33, 0, 20, 11), (257, 300, 190, 2080639), (96, 96, 96, 127), (40, 5000, 40, P25),
      (200, 700, 100, 8388593), (64, 2000, 64, 16711423), (70, 300, 50, 65279)]
PQ = [("uniform", 1, 1, 7), ("uniform", 5, 5, 7), ("uniform", 33, 20, 3), ("uniform", 20, 33, 65521),
      ("uniform", 64, 64, P26), ("uniform", 100, 130, 11579), ("uniform", 200, 200, P25), ("uniform", 300, 300, 1021),
      ("zero_cols", 40, 40, 13), ("zero_cols", 100, 130, 65521), ("lead_zero", 70, 80, 7), ("rank30", 96, 96, P26),
      ("ties", 70, 70, 3), ("ties", 130, 90, 11), ("zeros", 10, 12, 7), ("tall_low", 90, 90, P26),
      ("uniform", 100, 100, 1000), ("uniform", 90, 90, 255255), ("rank1", 40, 40, 5),
      ("wide_quirk", 3, 40, 7), ("wide_quirk", 5, 45, 11), ("wide_quirk", 4, 38, 65521), ("uniform", 520, 300, P26)]


def as_int(M):
    return np.rint(M.Array()).astype(np.int64)


def build(gffm, seed):
    rng = np.random.default_rng(seed)
    inst, want = [], []
    for (m, k, n, N) in MM:
        A, B = rng.integers(0, N, size=(m, k)), rng.integers(0, N, size=(k, n))
        inst.append(("matmul", gffm.CuModMatrix(A, N, elem_type=torch.float64),
                     gffm.CuModMatrix(B, N, elem_type=torch.float64)))
        want.append(("matmul", oracle.matmul(A, B, N) if k > 0 else np.zeros((m, n), dtype=np.int64)))
    for (kind, m, n, N) in PQ:
        A = make(kind, m, n, N, rng)
        inst.append(("pluq", gffm.CuModMatrix(A, N, elem_type=torch.float64)))
        try:
            want.append(("pluq", oracle.pluq(A, N)))
        except IndexError:
            want.append(("pluq", None))
    order = rng.permutation(len(inst))
    return [inst[i] for i in order], [want[i] for i in order]


def check(gffm, inst, want, results):
    for (kind, *_), (_, w), got in zip(inst, want, results):
        if kind == "matmul":
            assert np.array_equal(as_int(got), w)
            continue
        if w is None:                       # the reference's BoundsError
            assert isinstance(got, gffm.GFFMError) and got.status == 8
            continue
        U0, L0, rs0, cs0, _ = w
        U, L, rs, cs = got
        m = U.rows()
        assert rs == rs0 and cs == cs0
        assert np.array_equal(as_int(U), U0)
        Ld = np.rint(L.data.cpu().numpy().T).astype(np.int64)
        assert np.array_equal(Ld[:m, :m + 32], L0)


@pytest.mark.parametrize("tuning", [None, (8, 0, 0, 0, 7), (16, 3, 5, 1, 8), (32, 1, 1, 0, 0), (32, 0, 0, 1, 0)],
                         ids=["default", "nb8-7bit", "nb16-small-grids-overlap-8bit", "one-cta-each", "overlap"])
def test_mixed_batch_matches_oracle(gffm, tuning):
    inst, want = build(gffm, 77)
    tu = gffm.BatchTuning(*tuning) if tuning else None
    plan = gffm.BatchPlan(inst, tu)
    info = plan.info()
    assert info["products"] == len(MM) - 0 and info["pluqs"] == len(PQ)
    check(gffm, inst, want, plan.run().results())
    # a plan runs again on the same buffers with the same result
    check(gffm, inst, want, plan.run().results())
    assert gffm.load_library().gffm_device_status(None) == 0


def test_config4_sample(gffm):
    """512 instances drawn like the 4096-instance workload (n in 32..512, the 32 primes,
    half products, half PLUQs); every PLUQ full rank with a unit diagonal, and 24
    instances checked against the oracle."""
    from gffm import batched
    specs = batched.config4_specs(512, seed=4)
    g = torch.Generator(device="cuda")
    g.manual_seed(4)
    inst = batched.build_config4(specs, generator=g)
    plan = gffm.BatchPlan(inst)
    res = plan.run().results()
    rng = np.random.default_rng(0)
    checked = set(rng.choice(len(specs), size=24, replace=False).tolist())
    for i, ((op, n, p), spec, got) in enumerate(zip(specs, inst, res)):
        if op == "pluq":
            U, L, rs, cs = got
            Uh = as_int(U)
            if cs == [] and (np.diag(Uh) == 1).all():
                pass
            else:
                assert (np.diag(Uh)[: n - len(cs)] == 1).all()   # a rare singular draw
        if i not in checked:
            continue
        if op == "matmul":
            assert np.array_equal(as_int(got), oracle.matmul(as_int(spec[1]), as_int(spec[2]), p))
        else:
            U0, L0, rs0, cs0, _ = oracle.pluq(as_int(spec[1]), p)
            U, L, rs, cs = got
            assert rs == rs0 and cs == cs0 and np.array_equal(as_int(U), U0)
            Ld = np.rint(L.data.cpu().numpy().T).astype(np.int64)
            assert np.array_equal(Ld[:n, :n + 32], L0)
    assert gffm.load_library().gffm_device_status(None) == 0


def test_batched_pluq_1024_rows(gffm):
    rng = np.random.default_rng(1024)
    A = rng.integers(0, P26, size=(1024, 200))
    B = make("rank70", 300, 260, 65521, rng)
    plan = gffm.BatchPlan([("pluq", gffm.CuModMatrix(A, P26, elem_type=torch.float64)),
                           ("pluq", gffm.CuModMatrix(B, 65521, elem_type=torch.float64))])
    res = plan.run().results()
    for X, N, got in ((A, P26, res[0]), (B, 65521, res[1])):
        U0, L0, rs0, cs0, _ = oracle.pluq(X, N)
        U, L, rs, cs = got
        assert rs == rs0 and cs == cs0 and np.array_equal(as_int(U), U0)
        m = X.shape[0]
        Ld = np.rint(L.data.cpu().numpy().T).astype(np.int64)
        assert np.array_equal(Ld[:m, :m + 32], L0)


def test_batched_errors(gffm):
    A = gffm.CuModMatrix([[1, 2], [3, 4]], 2 ** 26, elem_type=torch.float64)
    with pytest.raises(gffm.GFFMError) as ei:
        gffm.BatchPlan([("matmul", A, A)])
    assert ei.value.status == 3
    with pytest.raises(gffm.GFFMError) as ei:
        gffm.BatchPlan([("pluq", gffm.zeros(torch.float64, 4, 4, 7))], gffm.BatchTuning(12, 0, 0, 0, 0))
    assert ei.value.status == 1
    empty = gffm.BatchPlan([])
    empty.run()
    assert gffm.load_library().gffm_device_status(None) == 0


def test_batched_pluq_taller_than_1024_rows(gffm):
    """PLUQ instances of more than 1024 rows are factored after the graph by the
    single-matrix elimination, into the same result arrays; mixed with graph instances."""
    rng = np.random.default_rng(1100)
    specs = [("uniform", 1100, 4, 7), ("uniform", 1300, 200, P26), ("wide_quirk", 1025, 1100, 11),
             ("rank30", 2000, 90, 65521), ("uniform", 300, 300, 1021)]
    inst, want = [], []
    for (kind, m, n, N) in specs:
        A = make(kind, m, n, N, rng)
        inst.append(("pluq", gffm.CuModMatrix(A, N, elem_type=torch.float64)))
        try:
            want.append(("pluq", oracle.pluq(A, N)))
        except IndexError:
            want.append(("pluq", None))
    A, B = rng.integers(0, 65521, size=(200, 300)), rng.integers(0, 65521, size=(300, 100))
    inst.append(("matmul", gffm.CuModMatrix(A, 65521, elem_type=torch.float64),
                 gffm.CuModMatrix(B, 65521, elem_type=torch.float64)))
    want.append(("matmul", oracle.matmul(A, B, 65521)))
    plan = gffm.BatchPlan(inst)
    assert plan.info()["pluqs"] == len(specs)
    for _ in range(2):                      # a plan runs again on the same buffers
        check(gffm, inst, want, plan.run().results())
    assert gffm.load_library().gffm_device_status(None) == 0


# Square PLUQs of n = 32 k >= 64 with an odd prime take the panel-step route (tensor-core
# trailing updates) under the default tuning; those that lose rank in a panel are factored
# again by the per-instance kernel.  Sizes, primes and rank patterns of both kinds.
STEP_PQ = [("uniform", 64, 64, P26), ("uniform", 96, 96, 65521), ("uniform", 128, 128, 2080639),
           ("uniform", 160, 160, 3), ("uniform", 256, 256, P25), ("uniform", 288, 288, 8191),
           ("uniform", 448, 448, 65521), ("uniform", 512, 512, P26), ("uniform", 192, 192, 127),
           ("rank30", 96, 96, P26), ("zero_cols", 128, 128, 13), ("ties", 128, 128, 11),
           ("lead_zero", 64, 64, 7), ("uniform", 64, 64, 2), ("uniform", 100, 100, P26),
           ("tall_low", 128, 128, P26)]


def test_step_route_matches_oracle(gffm):
    rng = np.random.default_rng(3232)
    inst, want = [], []
    for (kind, m, n, N) in STEP_PQ:
        A = make(kind, m, n, N, rng)
        inst.append(("pluq", gffm.CuModMatrix(A, N, elem_type=torch.float64)))
        want.append(("pluq", oracle.pluq(A, N)))
    A, B = rng.integers(0, P25, size=(300, 200)), rng.integers(0, P25, size=(200, 260))
    inst.append(("matmul", gffm.CuModMatrix(A, P25, elem_type=torch.float64),
                 gffm.CuModMatrix(B, P25, elem_type=torch.float64)))
    want.append(("matmul", oracle.matmul(A, B, P25)))
    plan = gffm.BatchPlan(inst)
    res = plan.run().results()
    check(gffm, inst, want, res)
    # the same factorization as the per-instance kernel, bit for bit, and again on a rerun
    per_inst = gffm.BatchPlan(inst, gffm.BatchTuning(32, 0, 0, 0, 0)).run().results()
    for (kind, *_), a, b in zip(inst, res, per_inst):
        if kind == "pluq":
            assert a[2] == b[2] and a[3] == b[3]
            assert torch.equal(a[0].data, b[0].data) and torch.equal(a[1].data, b[1].data)
    check(gffm, inst, want, plan.run().results())
    assert gffm.load_library().gffm_device_status(None) == 0


def test_step_chains_match_per_instance_kernel(gffm):
    """A batch large enough for the step route's two chains (>= 64 step instances): every
    PLUQ bit for bit equal to the per-instance kernel's, rank-deficient ones included."""
    rng = np.random.default_rng(6464)
    primes = [8191, 65521, 2080639, 16777213, P26]
    inst = []
    for i in range(128):
        n, N = 32 * int(rng.integers(2, 17)), primes[i % len(primes)]
        kind = "rank%d" % (n - 5) if i % 16 == 3 else ("zero_cols" if i % 16 == 7 else "uniform")
        inst.append(("pluq", gffm.CuModMatrix(make(kind, n, n, N, rng), N, elem_type=torch.float64)))
    steps = gffm.BatchPlan(inst).run().results()
    per_inst = gffm.BatchPlan(inst, gffm.BatchTuning(32, 0, 0, 0, 0)).run().results()
    for a, b in zip(steps, per_inst):
        assert a[2] == b[2] and a[3] == b[3]
        assert torch.equal(a[0].data, b[0].data) and torch.equal(a[1].data, b[1].data)
    assert gffm.load_library().gffm_device_status(None) == 0
