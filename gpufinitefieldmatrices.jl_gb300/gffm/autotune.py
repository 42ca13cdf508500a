"""Autotuner for the limb GEMM and the batched plans.

It times candidate configurations on the device (CUDA events, after warm-up)
and keeps the winners in a small JSON table, ``gffm/tuning.json``:

* ``"gemm"``: a list of entries ``{N_lo, N_hi, work_lo, work_hi, digit_bits,
  max_ctas}`` that :func:`apply` loads into the library's process-wide tune
  table (``gffm_tune_table_set``); every ``gffm_matmul_limb_*`` call and its
  workspace-size query consult it (first matching modulus and m*n*k range).
  Candidates are the digit width (7-bit digits, or 8-bit digits where they
  need one digit fewer), the persistent grid size and the output tile width
  (64 columns, or 32 with two accumulator sets).
* ``"batched"``: per batch signature (the multiset of instance shapes, ops and
  digit counts), the best ``gffm_batch_tuning`` -- the PLUQ route (0: panel
  steps with tensor-core trailing updates where they apply; 8/16/32: the
  persistent kernel with that panel width), grid split, overlap of the two
  graph branches, digit width.
  ``BatchPlan(instances, tuning="auto")`` looks it up.

The table is plain data and ships with the package; re-tuning rewrites it.
"""
import ctypes
import hashlib
import json
import os

import torch

from ._lib import call, load

TABLE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning.json")

# moduli whose 8-bit digit split needs one digit fewer than the 7-bit one
BITS8_RANGES = [(16256, 65279), (2080640, 16711423)]


class _LimbTuning(ctypes.Structure):
    _fields_ = [("digit_bits", ctypes.c_int32), ("max_ctas", ctypes.c_int32), ("tile_n", ctypes.c_int32),
                ("form", ctypes.c_int32)]


class _Entry(ctypes.Structure):
    _fields_ = [("N_lo", ctypes.c_int64), ("N_hi", ctypes.c_int64), ("work_lo", ctypes.c_double),
                ("work_hi", ctypes.c_double), ("tuning", _LimbTuning)]


def load_table(path=TABLE):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {"gemm": [], "batched": {}}


def save_table(table, path=TABLE):
    with open(path, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)


def apply(table=None):
    """Load the table's GEMM entries into the library's tune table."""
    table = load_table() if table is None else table
    ents = table.get("gemm", [])
    arr = (_Entry * max(1, len(ents)))()
    for i, e in enumerate(ents):
        arr[i] = _Entry(int(e["N_lo"]), int(e["N_hi"]), float(e["work_lo"]), float(e["work_hi"]),
                        _LimbTuning(int(e["digit_bits"]), int(e.get("max_ctas", 0)), int(e.get("tile_n", 0)),
                                    int(e.get("form", 0))))
    call("gffm_tune_table_set", ctypes.cast(arr, ctypes.c_void_p), len(ents))
    return len(ents)


def _time(fn, reps):
    fn()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def time_gemm(m, n, k, N, digit_bits, max_ctas=0, reps=5, generator=None, tile_n=0, form=0):
    """Milliseconds of one C = A*B mod N (resident Float64 operands) with a given tuning."""
    from .cumod import rand, zeros
    A = rand(torch.float64, m, k, N, generator=generator)
    B = rand(torch.float64, k, n, N, generator=generator)
    C = zeros(torch.float64, m, n, N)
    tu = _LimbTuning(digit_bits, max_ctas, tile_n, form)
    ws = ctypes.c_size_t(0)
    call("gffm_matmul_limb_tuned_workspace_size", m, n, k, N, ctypes.byref(tu), ctypes.byref(ws))
    buf = torch.empty(max(1, ws.value), dtype=torch.uint8, device="cuda")
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def run():
        call("gffm_matmul_limb_tuned_f64", m, n, k, A.data.data_ptr(), A.ld, B.data.data_ptr(), B.ld,
             C.data.data_ptr(), C.ld, N, ctypes.byref(tu), ctypes.c_void_p(buf.data_ptr()), ws.value, s)

    return _time(run, reps)


# moduli of four 7-bit digits where the Karatsuba form applies (kara_host.h), beyond the
# ranges where 8-bit digits save a digit
KARA_RANGE = (16711424, 2 ** 26 - 1)


def tune_gemm(shapes=((512, 512, 512), (2048, 2048, 2048), (8192, 8192, 8192)),
              moduli=(32749, 8388593, 67108859), reps=5):
    """For each modulus (one per range where 8-bit digits save a digit, and one where only
    the Karatsuba form saves products) and size, time 7- and 8-bit schoolbook digits, the
    Karatsuba form where it applies, and a few grid sizes; return table entries covering
    each modulus range over a work range around each size."""
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    g = torch.Generator(device="cuda")
    g.manual_seed(11)
    entries, log = [], []
    works = sorted(m * n * k for (m, n, k) in shapes)
    for N in moduli:
        rng = next(((lo, hi) for lo, hi in BITS8_RANGES + [KARA_RANGE] if lo <= N <= hi), (N, N))
        kara = 2080639 < N < 2 ** 26
        for (m, n, k) in shapes:
            best = None
            cands = [(bits, ctas, tile_n, 1) for bits in (7, 8) for ctas in (0, sms // 2) for tile_n in (64, 32)]
            if kara:
                cands += [(7, ctas, 64, 2) for ctas in (0, sms // 2)]
            for bits, ctas, tile_n, form in cands:
                t = time_gemm(m, n, k, N, bits, ctas, reps, g, tile_n, form)
                log.append({"N": N, "m": m, "n": n, "k": k, "digit_bits": bits, "max_ctas": ctas,
                            "tile_n": tile_n, "form": form, "ms": round(t, 4)})
                if best is None or t < best[0]:
                    best = (t, bits, ctas, tile_n, form)
            w = m * n * k
            i = works.index(w)
            lo = 0.0 if i == 0 else (works[i - 1] * w) ** 0.5
            hi = 1e30 if i == len(works) - 1 else (works[i + 1] * w) ** 0.5
            entries.append({"N_lo": rng[0], "N_hi": rng[1], "work_lo": lo, "work_hi": hi,
                            "digit_bits": best[1], "max_ctas": best[2], "tile_n": best[3], "form": best[4],
                            "tuned_on": [m, n, k, N],
                            "ms": round(best[0], 4)})
    return entries, log


def batch_signature(instances):
    """A stable key for a batch: its sorted (op, m, n, k, digits) multiset."""
    from . import limbs_for
    rows = []
    for spec in instances:
        A = spec[1]
        if spec[0] == "matmul":
            rows.append(("matmul", A.rows(), spec[2].cols(), A.cols(), limbs_for(A.N, 7), limbs_for(A.N, 8)))
        else:
            rows.append(("pluq", A.rows(), A.cols(), 0, 0, 0))
    rows.sort()
    return hashlib.sha1(repr(rows).encode()).hexdigest()[:16]


BATCH_CANDIDATES = [
    {"pluq_panel": 0, "gemm_ctas": 0, "pluq_ctas": 0, "overlap": 0, "digit_bits": 0},
    {"pluq_panel": 0, "gemm_ctas": 0, "pluq_ctas": 0, "overlap": 1, "digit_bits": 0},
    {"pluq_panel": 0, "gemm_ctas": 0, "pluq_ctas": 0, "overlap": 1, "digit_bits": 7},
    {"pluq_panel": 32, "gemm_ctas": 0, "pluq_ctas": 0, "overlap": 0, "digit_bits": 0},
    {"pluq_panel": 32, "gemm_ctas": 0, "pluq_ctas": 0, "overlap": 0, "digit_bits": 7},
    {"pluq_panel": 16, "gemm_ctas": 0, "pluq_ctas": 0, "overlap": 0, "digit_bits": 0},
    {"pluq_panel": 32, "gemm_ctas": 0, "pluq_ctas": 0, "overlap": 1, "digit_bits": 0},
    {"pluq_panel": 32, "gemm_ctas": 76, "pluq_ctas": 152, "overlap": 1, "digit_bits": 0},
]


def tune_batched(instances, reps=3, candidates=None):
    """Time candidate tunings of a batch; return (best dict, log)."""
    from .batched import BatchPlan, Tuning
    best, log = None, []
    for c in candidates or BATCH_CANDIDATES:
        plan = BatchPlan(instances, Tuning(c["pluq_panel"], c["gemm_ctas"], c["pluq_ctas"], c["overlap"],
                                           c["digit_bits"]))
        t = _time(plan.run, reps)
        log.append(dict(c, ms=round(t, 4)))
        if best is None or t < best[0]:
            best = (t, c)
        del plan
    return dict(best[1], ms=round(best[0], 4)), log


def lookup_batched(instances, table=None):
    table = load_table() if table is None else table
    return table.get("batched", {}).get(batch_signature(instances))


def main():
    """Tune the GEMM digit width / grid and the batched workload, then write the table."""
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=TABLE)
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--log", default=None)
    ap.add_argument("--gemm-only", action="store_true", help="retune the GEMM entries, keep the batched ones")
    ap.add_argument("--batched-only", action="store_true", help="retune the batched entry, keep the GEMM ones")
    args = ap.parse_args()
    load()
    table = load_table(args.out)
    entries, glog = (table.get("gemm", []), []) if args.batched_only else tune_gemm()
    table["gemm"] = entries
    if args.gemm_only:
        save_table(table, args.out)
        if args.log:
            with open(args.log, "w") as f:
                json.dump({"gemm": glog}, f, indent=1)
        print(json.dumps({"gemm": entries}))
        return
    from . import batched
    specs = batched.config4_specs(args.batch, seed=1234)
    g = torch.Generator(device="cuda")
    g.manual_seed(1234)
    inst = batched.build_config4(specs, generator=g)
    best, blog = tune_batched(inst)
    table.setdefault("batched", {})[batch_signature(inst)] = dict(best, workload="%d instances, config4_specs seed 1234"
                                                                     % args.batch)
    save_table(table, args.out)
    if args.log:
        with open(args.log, "w") as f:
            json.dump({"gemm": glog, "batched": blog}, f, indent=1)
    print(json.dumps({"gemm": entries, "batched": best}))


if __name__ == "__main__":
    main()
