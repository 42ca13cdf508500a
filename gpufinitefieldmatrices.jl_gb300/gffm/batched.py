"""Batched uneven instances over libgffm's grouped kernels.

The reference runs one product (mul!, src/CuModMatrix/CuModMatrix.jl:767-787)
or one pluq_gpu_kernel (src/CuModMatrix/rref_lu_pluq/pluq_kernels.jl:46-157)
per call; a BatchPlan runs thousands of them, each with its own sizes and
modulus, as one CUDA graph: a grouped tensor-core product kernel, square
PLUQs (n = 32k, odd prime) in panel steps whose trailing updates are one
grouped tensor-core GEMM per step, and a persistent per-instance PLUQ kernel
for the others.  Both PLUQ routes give the reference's factorization.
Instances are CuModArrays; results land in the arrays the plan was built with.
"""
import ctypes

import numpy as np
import torch

from . import cumod
from ._lib import call, load
from .cumod import CuModArray, _stream

MATMUL, PLUQ = 0, 1


class _Desc(ctypes.Structure):
    _fields_ = [(name, ctypes.c_int64) for name in ("op", "m", "n", "k", "N")] + [
        ("A", ctypes.c_void_p), ("lda", ctypes.c_int64), ("B", ctypes.c_void_p), ("ldb", ctypes.c_int64),
        ("C", ctypes.c_void_p), ("ldc", ctypes.c_int64), ("L", ctypes.c_void_p), ("ldl", ctypes.c_int64),
        ("l_cols", ctypes.c_int64), ("row_swaps", ctypes.c_void_p), ("col_swaps", ctypes.c_void_p),
        ("info", ctypes.c_void_p)]


class Tuning(ctypes.Structure):
    """gffm_batch_tuning: 0 in a field picks the library default."""
    _fields_ = [("pluq_panel", ctypes.c_int32), ("gemm_ctas", ctypes.c_int32), ("pluq_ctas", ctypes.c_int32),
                ("overlap", ctypes.c_int32), ("digit_bits", ctypes.c_int32)]


class BatchPlan:
    """A batch of products and PLUQs bound to their arrays.

    ``instances`` holds tuples ``("matmul", A, B)`` (C = A*B mod A.N is
    allocated) or ``("matmul", A, B, C)``, and ``("pluq", A)`` (U, L and the
    swap stacks are allocated; U is a fresh array, A is left unchanged).
    """

    def __init__(self, instances, tuning=None):
        self._keep = []
        self.outputs = []
        descs = (_Desc * max(1, len(instances)))()
        for i, spec in enumerate(instances):
            kind, A = spec[0], spec[1]
            if A.dtype != torch.float64:
                raise TypeError("batched instances take Float64 storage")
            d = descs[i]
            if kind == "matmul":
                B = spec[2]
                if A.N != B.N:
                    raise cumod.CuModArrayModulusMismatchException("All matrices must have the same modulus N")
                if A.cols() != B.rows():
                    raise cumod.CuModArraySizeMismatchException("Matrix dimensions do not match for multiplication")
                C = spec[3] if len(spec) > 3 else cumod.zeros(A.dtype, A.rows(), B.cols(), A.N)
                d.op, d.m, d.n, d.k, d.N = MATMUL, A.rows(), B.cols(), A.cols(), A.N
                d.A, d.lda, d.B, d.ldb = A.data.data_ptr(), A.ld, B.data.data_ptr(), B.ld
                d.C, d.ldc = C.data.data_ptr(), C.ld
                self._keep += [A, B, C]
                self.outputs.append(C)
            elif kind == "pluq":
                m, n = A.rows(), A.cols()
                U = cumod.zeros(A.dtype, m, n, A.N)
                L = cumod.zeros(A.dtype, m, m, A.N)            # padded (m+32) x (m+32), as the reference's L
                rs = torch.zeros(2 * max(m, 1), dtype=torch.int64, device=A.data.device)
                cs = torch.zeros(2 * max(n, 1), dtype=torch.int64, device=A.data.device)
                info = torch.zeros(4, dtype=torch.int64, device=A.data.device)
                d.op, d.m, d.n, d.k, d.N = PLUQ, m, n, 0, A.N
                d.A, d.lda = A.data.data_ptr(), A.ld
                d.C, d.ldc = U.data.data_ptr(), U.ld
                d.L, d.ldl, d.l_cols = L.data.data_ptr(), L.ld, m + cumod.TILE_WIDTH
                d.row_swaps, d.col_swaps, d.info = rs.data_ptr(), cs.data_ptr(), info.data_ptr()
                self._keep += [A, U, L, rs, cs, info]
                self.outputs.append((U, L, rs, cs, info))
            else:
                raise ValueError("instance kind must be 'matmul' or 'pluq'")
        self._plan = ctypes.c_void_p()
        if isinstance(tuning, str):
            if tuning != "auto":
                raise ValueError("tuning must be a Tuning, None or 'auto'")
            from . import autotune
            best = autotune.lookup_batched(instances)
            tuning = None if best is None else Tuning(best["pluq_panel"], best["gemm_ctas"], best["pluq_ctas"],
                                                       best["overlap"], best.get("digit_bits", 0))
        tu = tuning if tuning is not None else Tuning()
        call("gffm_batched_plan_create", ctypes.cast(descs, ctypes.c_void_p), len(instances), ctypes.byref(tu),
             ctypes.byref(self._plan))
        self.kinds = [spec[0] for spec in instances]

    def info(self):
        out = (ctypes.c_int64 * 6)()
        call("gffm_batched_plan_info", self._plan, out)
        keys = ("device_bytes", "products", "pluqs", "product_tiles", "gemm_ctas", "pluq_ctas")
        return dict(zip(keys, list(out)))

    def run(self, stream=None):
        """Launch the plan's graph on ``stream`` (default: torch's current stream)."""
        s = ctypes.c_void_p(stream) if stream is not None else _stream()
        call("gffm_batched_run", self._plan, s)
        return self

    def results(self):
        """Per instance: C for a product; (U, L, Perm_rows, Perm_cols) for a PLUQ, as
        pluq_gpu_kernel returns them (1-based swap stacks).  Synchronizes."""
        torch.cuda.current_stream().synchronize()
        out = []
        for kind, o in zip(self.kinds, self.outputs):
            if kind == "matmul":
                out.append(o)
                continue
            U, L, rs, cs, info = o
            nr, nc, rank, status = (int(x) for x in info.cpu().tolist())
            if status:
                from ._lib import GFFMError
                out.append(GFFMError(status, "the reference indexes L out of bounds for this instance"))
                continue
            r = rs.cpu().numpy()[: 2 * nr].reshape(-1, 2)
            c = cs.cpu().numpy()[: 2 * nc].reshape(-1, 2)
            out.append((U, L, [tuple(map(int, x)) for x in r], [tuple(map(int, x)) for x in c]))
        return out

    def pluq_info(self):
        return [o[4].cpu().tolist() if k == "pluq" else None for k, o in zip(self.kinds, self.outputs)]

    def __del__(self):
        plan = getattr(self, "_plan", None)
        if plan:
            try:
                load().gffm_batched_plan_destroy(plan)
            except Exception:
                pass


def batched_plan(instances, tuning=None):
    return BatchPlan(instances, tuning)


def fixed_primes():
    """The 32 primes of the batched workload: the largest prime <= round(2^(10 + 16 i / 32)), i = 0..31."""
    def is_prime(x):
        if x < 2:
            return False
        i = 2
        while i * i <= x:
            if x % i == 0:
                return False
            i += 1
        return True
    out = []
    for i in range(32):
        x = int(round(2 ** (10 + 16 * i / 32)))
        while not is_prime(x):
            x -= 1
        out.append(x)
    return out


def config4_specs(count=4096, seed=1234):
    """Sizes, primes and ops of the batched uneven-instance workload: n uniform over
    the multiples of 32 in [32, 512], p uniform over the 32 fixed primes, even
    instances a product, odd ones a PLUQ."""
    rng = np.random.default_rng(seed)
    primes = fixed_primes()
    ns = 32 * rng.integers(1, 17, size=count)
    ps = [primes[i] for i in rng.integers(0, 32, size=count)]
    ops = ["matmul" if i % 2 == 0 else "pluq" for i in range(count)]
    return list(zip(ops, (int(x) for x in ns), ps))


def ops_of(specs):
    """Modular operations of a batch: 2 n^3 per product, (2/3) n^3 per PLUQ (square n)."""
    return sum(2 * n ** 3 if op == "matmul" else (2 * n ** 3) / 3 for op, n, _ in specs)


def build_config4(specs, generator=None, device="cuda"):
    """CuModMatrix instances for the specs, seeded uniform residues on the device (PLUQ
    instances full rank with overwhelming probability for these primes and sizes)."""
    inst = []
    for op, n, p in specs:
        A = cumod.rand(torch.float64, n, n, p, generator=generator)
        if op == "matmul":
            B = cumod.rand(torch.float64, n, n, p, generator=generator)
            inst.append(("matmul", A, B))
        else:
            inst.append(("pluq", A))
    return inst
