"""Benchmark: bit-exact modular GEMM 8192 x 8192 x 8192 mod 67108859 (the largest
prime below 2^26) on one GB300, through the library's C ABI.

A step is one C = A*B mod p of two resident Float64 CuModMatrix operands on
the limb tensor-core path (digit split of A and B + the tcgen05 GEMM with its
fused recombination / Barrett epilogue).  Operands are 2 x 541 MB, larger than
the 129 MB L2, so no flush is needed between steps.

Printed JSON line (one, from rank 0):
  value        whole-job Gop/s (2*m*n*k per step, all ranks)
  e2e          the same metric through the C ABI with host buffers: every step
               copies A and B from pinned host memory and C back (the median of
               three timed runs, all three listed)
  roofline     the tcgen05 GEMM kernel's tensor FLOP/s (digit products) vs the
               measured dense bf16/fp16 peak; traffic from an ncu capture (its
               source is named in the line: no run reads DRAM counters itself)
  config1_512  the 512 x 512 mod 65521 product on both paths, in microseconds
  plain_fp64   the plain path (the reference's Float64 method) on the same GPU
  pluq         PLUQ timings when the elimination is built (see --pluq)
  cpu_baseline the oracle (exact C restatement) on the host cores, bounded sample
--impl reference times the reference's CPU path (the oracle port; the Julia
reference cannot run here) on the same workload and metric.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG_DIR = os.path.join(ROOT, "gpufinitefieldmatrices.jl_gb300")
for _p in (ROOT, PKG_DIR):
    if _p not in sys.path:
        sys.path.insert(0, _p)

P26 = 67108859
M = N = K = 8192
METRIC = "bit-exact mod-p GEMM Gop/s & PLUQ time: limb tensor-core vs plain FP64, same GB300"
WORKLOAD = "modular GEMM 8192x8192x8192 mod 67108859, Float64 CuModMatrix operands, limb tensor-core path"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP64 comparison")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--pluq", type=int, default=-1, help="PLUQ size to time (-1: 16384, 0: skip)")
    ap.add_argument("--no-pluq-plain", action="store_true", help="skip the plain-Float64 PLUQ (about 10-30 s)")
    ap.add_argument("--no-karatsuba", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--batch", type=int, default=4096, help="instances of the batched workload")
    ap.add_argument("--batch-pluqs", action="store_true", help="the batched leg with its PLUQ half only")
    ap.add_argument("--batch-uniform", default=None, metavar="COUNTxN",
                    help="with --only batched: COUNT seeded full-rank N x N PLUQ instances mod 67108859 instead of "
                         "the mixed workload (a case for profiling the batched PLUQ kernel)")
    ap.add_argument("--only", default=None, choices=["gemm", "pluq", "karatsuba", "batched"],
                    help="run one leg alone and print its fields (for profiling; not the benchmark line)")
    ap.add_argument("--size", type=int, default=8192, help="m = n = k (8192 is the benchmark workload)")
    return ap.parse_args()


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return d.get("bf16_tflops"), d.get("hbm_gbs"), "measured"
    except (OSError, ValueError):
        return 1900.0, 6800.0, "fallback"


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per launch of the headline
# GEMM kernel, from an ncu capture of the same kernel (one pass, -c 1,
# --clock-control none); a benchmark run cannot read DRAM counters itself, so the
# figure is reported with its source and is not measured in the run.
GEMM_TRAFFIC = {"bytes": 9.425913088e9 + 5.21232384e8,
                "source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of this benchmark's own 8192^3 "
                          "k_gemm_kara launch (one pass, -c 1; not measured in this run)"}


# ---------------------------------------------------------------------------
# replicas: one process per GPU, independent products, the slowest rank's time
# ---------------------------------------------------------------------------
def job_time_ms(ms, dist=None, dev="cpu"):
    """The whole job's time: the slowest rank's, agreed on by every rank (max over ranks)."""
    if dist is None:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate_gops(ops_per_rank_step, steps, world, ms):
    """Whole-job Gop/s: the work of every rank over the job's (slowest rank's) time."""
    return ops_per_rank_step * steps * world / (ms / 1e3) / 1e9


# ---------------------------------------------------------------------------
# CPU side (oracle): cpu_baseline and the reference arm
# ---------------------------------------------------------------------------
def cpu_sample(target_s=12.0):
    """Time the oracle's exact matmul on a row sample of the 8192^3 workload with
    every host thread; returns (Gop/s, threads, description)."""
    import numpy as np
    import oracle
    threads = os.cpu_count() or 1
    rng = np.random.default_rng(7)
    B = np.asfortranarray(rng.integers(0, P26, size=(K, N)))
    rows = 16
    while True:
        A = np.asfortranarray(rng.integers(0, P26, size=(rows, K)))
        t0 = time.perf_counter()
        oracle.matmul(A, B, P26, threads)
        dt = time.perf_counter() - t0
        if dt >= target_s / 4 or rows >= M:
            break
        rows = min(M, rows * max(2, int(target_s / 4 / max(dt, 1e-3))))
    gops = 2.0 * rows * N * K / dt / 1e9
    return gops, threads, "%d x %d x %d row slice of the workload (exact Int128-free uint64 C, OpenMP)" % (rows, N, K)


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import numpy as np
    import oracle
    oracle.build()
    threads = os.cpu_count() or 1
    rng = np.random.default_rng(11)
    B = np.asfortranarray(rng.integers(0, P26, size=(K, N)))
    # calibrate one step to ~2 s of CPU work
    rows = 8
    while True:
        A = np.asfortranarray(rng.integers(0, P26, size=(rows, K)))
        t0 = time.perf_counter()
        oracle.matmul(A, B, P26, threads)
        dt = time.perf_counter() - t0
        if dt > 1.0 or rows >= 1024:
            break
        rows *= 2
    A = np.asfortranarray(rng.integers(0, P26, size=(rows, K)))
    for _ in range(args.warmup):
        oracle.matmul(A, B, P26, threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        oracle.matmul(A, B, P26, threads)
    dt = time.perf_counter() - t0
    gops = 2.0 * rows * N * K * args.steps / dt / 1e9
    sample = "each step: %d x %d x %d row slice of the 8192^3 workload" % (rows, N, K)
    line = {
        "impl": "reference", "metric": METRIC, "value": round(gops, 3), "unit": "Gop/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt / args.steps * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "m": M, "n": N, "k": K, "modulus": P26},
        "cpu_baseline": {"value": round(gops, 3), "unit": "Gop/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(gops, 3), "unit": "Gop/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "GPUFiniteFieldMatrices.jl is Julia (CUDA.jl); no Julia toolchain exists on this box, so its CPU "
                "path (Int64 matmul then mod) is stood in for by the exact C restatement in oracle/",
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def run_ours(args):
    import torch
    import gffm

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    else:
        torch.cuda.set_device(0)
    gffm.build()
    L = gffm.load_library()
    dev = torch.device("cuda", local if world > 1 else 0)
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)

    if args.only in ("pluq", "karatsuba", "batched"):
        leg = {"pluq": lambda: pluq_run(args, L, sp, dev), "karatsuba": lambda: karatsuba_run(L, sp, dev),
               "batched": lambda: batched_run(args, dev, 112000.0)}[args.only]()
        print(json.dumps({"only": args.only, args.only: leg}), flush=True)
        return

    g = torch.Generator(device=dev)
    g.manual_seed(1234 + rank)
    A = gffm.rand(torch.float64, M, K, P26, generator=g)
    B = gffm.rand(torch.float64, K, N, P26, generator=g)
    C = gffm.zeros(torch.float64, M, N, P26)
    ws = ctypes.c_size_t(0)
    assert L.gffm_matmul_limb_workspace_size(M, N, K, P26, ctypes.byref(ws)) == 0
    wbuf = torch.empty(ws.value, dtype=torch.uint8, device=dev)

    def step(ev=None):
        if ev is not None:
            L.gffm_profile_next_kernel(ctypes.c_void_p(ev[0].cuda_event), ctypes.c_void_p(ev[1].cuda_event))
        st = L.gffm_matmul_limb_f64(M, N, K, A.data.data_ptr(), A.ld, B.data.data_ptr(), B.ld, C.data.data_ptr(),
                                    C.ld, P26, wbuf.data_ptr(), ws.value, sp)
        if st != 0:
            raise RuntimeError(L.gffm_last_error_string().decode())

    def barrier():
        if dist is not None:
            dist.barrier()

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    # correctness spot check of the warm-up output (Freivalds on one vector, exact on the host)
    spot_ok = freivalds(A, B, C)

    kev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for a, b in kev:        # torch creates the CUDA event on its first record
        a.record()
        b.record()
    clocks = ClockSampler(local if world > 1 else 0)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for i in range(args.steps):
        step(kev[i])
    e1.record()
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    kern_ms = [a.elapsed_time(b) for a, b in kev]
    ms = job_time_ms(ms, dist, dev)
    ops_step = 2.0 * M * N * K
    value = job_rate_gops(ops_step, args.steps, world, ms)
    st = L.gffm_device_status(sp)
    if st != 0:
        raise RuntimeError("device status %d" % st)

    # roofline of the tcgen05 GEMM kernel: digit-product tensor FLOPs per launch.  At this
    # modulus and k the library's default is the Karatsuba form: 12 fp16 digit products per
    # modular multiply-add on 128 x 128 tiles (the schoolbook form: 16, 128 x 64 tiles)
    Ld = 4
    products = 12
    Mp, Np, Kp = (M + 127) // 128 * 128, (N + 127) // 128 * 128, (K + 63) // 64 * 64
    tflop = 2.0 * products * Mp * Np * Kp / 1e12
    kavg = statistics.mean(kern_ms)
    peak, hbm_peak, peak_kind = measured_peaks()
    achieved = tflop / (kavg / 1e3)
    roofline = {"bound": "tensor", "kernel": "kara::k_gemm_kara<EPI_STORE_F64>", "achieved": round(achieved, 1),
                "peak": peak, "unit": "TFLOP/s", "frac": round(achieved / peak, 4), "peak_kind": peak_kind,
                "traffic": GEMM_TRAFFIC["bytes"], "traffic_source": GEMM_TRAFFIC["source"],
                "kernel_ms": round(kavg, 4),
                "algorithmic": "12 fp16 digit products per modular MAC (one-level Karatsuba over 13-bit halves): "
                               "2*12*8192^3 FLOP per launch"}

    out = {
        "metric": METRIC, "value": round(value, 1), "unit": "Gop/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f16", "data": "synthetic",
        "config": {"workload": WORKLOAD, "m": M, "n": N, "k": K, "modulus": P26, "digits": Ld,
                   "l2": "inputs larger than L2 (2 x 541 MB Float64 operands); no flush",
                   "parallelism": "replicas x%d" % world},
        "clocks": clk, "gpu_launches": 3 * args.steps, "roofline": roofline, "spot_check_ok": spot_ok,
    }

    if args.only == "gemm":
        print(json.dumps(out), flush=True)
        return
    if not args.no_e2e:
        out["e2e"] = e2e_run(args, L, sp, dev, world, dist)
    if not args.no_plain:
        out["plain_fp64"] = plain_run(L, sp, dev)
        out["plain_fp64"]["limb_speedup"] = round(value / world / out["plain_fp64"]["value"], 1)
    out["config1_512"] = config1_run(L, sp, dev)
    if args.pluq != 0:
        out["pluq"] = pluq_run(args, L, sp, dev)
    if not args.no_karatsuba:
        out["karatsuba"] = karatsuba_run(L, sp, dev)
    if not args.no_batched:
        out["batched"] = batched_run(args, dev, value / world)
    if rank == 0 and not args.no_cpu:
        gops, threads, desc = cpu_sample()
        out["cpu_baseline"] = {"value": round(gops, 3), "unit": "Gop/s", "cores": threads, "kind": "port",
                               "sample": desc}
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(out), flush=True)


def freivalds(A, B, C):
    import numpy as np
    import oracle
    rng = np.random.default_rng(3)
    x = rng.integers(0, P26, size=(K, 1))
    Ah = np.rint(A.Array()).astype(np.int64)
    Bh = np.rint(B.Array()).astype(np.int64)
    Ch = np.rint(C.Array()).astype(np.int64)
    return bool(np.array_equal(oracle.matmul(Ch, x, P26), oracle.matmul(Ah, oracle.matmul(Bh, x, P26), P26)))


def e2e_run(args, L, sp, dev, world, dist):
    """C = A*B mod p from pinned host Float64 buffers (the padded CuModMatrix layout)
    through the host-buffer C ABI call gffm_matmul_host_f64: every step copies A and
    B in and C out, the library overlapping the block copies with its block products.
    For comparison, ``serial`` times the same step as separate whole-matrix copies
    around gffm_matmul_limb_f64."""
    import torch
    pad = 32
    shapeA = (K + pad, M + pad)
    shapeB = (N + pad, K + pad)
    shapeC = (N + pad, M + pad)
    g = torch.Generator()
    g.manual_seed(77)
    hA = torch.zeros(shapeA, dtype=torch.float64).pin_memory()
    hB = torch.zeros(shapeB, dtype=torch.float64).pin_memory()
    hC = torch.zeros(shapeC, dtype=torch.float64).pin_memory()
    hA[:K, :M] = torch.randint(0, P26, (K, M), generator=g).double()
    hB[:N, :K] = torch.randint(0, P26, (N, K), generator=g).double()
    ws = ctypes.c_size_t(0)
    L.gffm_matmul_host_workspace_size(M, N, K, P26, ctypes.byref(ws))
    wbuf = torch.empty(ws.value, dtype=torch.uint8, device=dev)

    def step():
        st = L.gffm_matmul_host_f64(M, N, K, hA.data_ptr(), M + pad, hB.data_ptr(), K + pad, hC.data_ptr(), M + pad,
                                    P26, wbuf.data_ptr(), ws.value, sp)
        assert st == 0

    def timed(fn, steps):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return job_time_ms(e0.elapsed_time(e1), dist, dev)

    # the host link is shared with the machine's other jobs: three timed runs of `steps`
    # steps each, the median reported and all three listed
    steps = max(5, args.steps // 6)
    runs = [timed(step, steps) for _ in range(3)]
    ms = statistics.median(runs)
    # the same product through the device-buffer call with whole-matrix copies around it
    del wbuf
    dA = torch.empty(shapeA, dtype=torch.float64, device=dev)
    dB = torch.empty(shapeB, dtype=torch.float64, device=dev)
    dC = torch.zeros(shapeC, dtype=torch.float64, device=dev)
    L.gffm_matmul_limb_workspace_size(M, N, K, P26, ctypes.byref(ws))
    wbuf = torch.empty(ws.value, dtype=torch.uint8, device=dev)

    def serial_step():
        dA.copy_(hA, non_blocking=True)
        dB.copy_(hB, non_blocking=True)
        st = L.gffm_matmul_limb_f64(M, N, K, dA.data_ptr(), M + pad, dB.data_ptr(), K + pad, dC.data_ptr(), M + pad,
                                    P26, wbuf.data_ptr(), ws.value, sp)
        assert st == 0
        hC.copy_(dC, non_blocking=True)

    runs_serial = [timed(serial_step, steps) for _ in range(3)]
    ms_serial = statistics.median(runs_serial)
    h2d = (M * K + K * N) * 8
    d2h = M * N * 8
    blocks = [(x + 2047) // 2048 for x in (M, N)]
    gops = lambda t: round(job_rate_gops(2.0 * M * N * K, steps, world, t), 1)
    return {"value": gops(ms), "unit": "Gop/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "steps": steps, "ms_per_step": round(ms / steps, 3),
            "runs_ms_per_step": [round(t / steps, 3) for t in runs], "of_runs": "median",
            "call": "gffm_matmul_host_f64 (%d x %d blocks)" % tuple(blocks),
            "gpu_launches": (blocks[0] + blocks[1] + blocks[0] * blocks[1]) * steps,
            "serial": {"value": gops(ms_serial), "ms_per_step": round(ms_serial / steps, 3),
                       "runs_ms_per_step": [round(t / steps, 3) for t in runs_serial],
                       "call": "torch copies + gffm_matmul_limb_f64"}}


def plain_run(L, sp, dev):
    """The plain path (the reference's Float64 method, stripe width 1 at this modulus)
    on a k-slice of the same workload; its time is linear in k."""
    import torch
    import gffm
    ks = 512
    g = torch.Generator(device=dev)
    g.manual_seed(99)
    A = gffm.rand(torch.float64, M, ks, P26, generator=g)
    B = gffm.rand(torch.float64, ks, N, P26, generator=g)
    C = gffm.zeros(torch.float64, M, N, P26)

    def run():
        st = L.gffm_matmul_plain_f64(M, N, ks, A.data.data_ptr(), A.ld, B.data.data_ptr(), B.ld, C.data.data_ptr(),
                                     C.ld, P26, 0, sp)
        assert st == 0

    run()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(2):
        run()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / 2
    gops = 2.0 * M * N * ks / (ms / 1e3) / 1e9
    peak = fp64_peak_tflops(dev)
    # at this modulus every product is reduced at once (stripe 1): an fma for the product and
    # fmul, frnd, fma for the reduction, all on the FP64 pipe
    instr = 4
    return {"value": round(gops, 2), "unit": "Gop/s",
            "sample": "8192 x 8192 x %d k-slice (time is linear in k)" % ks, "ms": round(ms, 2),
            "stripe": 1, "fp64_peak_tflops": round(peak, 2),
            "fp64_peak_source": "cuBLAS DGEMM 4096^3 through torch, best of 5, this run",
            "frac": round(gops / 1e3 / peak, 4),
            "fp64_instructions_per_modular_mac": instr,
            "frac_of_fp64_issue": round(gops / 2 * instr / 1e3 / (peak / 2), 4)}


def fp64_peak_tflops(dev):
    """Dense FP64 rate of this GPU: a cuBLAS DGEMM of 4096^3, best of 5 (CUDA events)."""
    import torch
    a = torch.rand(4096, 4096, dtype=torch.float64, device=dev)
    b = torch.rand(4096, 4096, dtype=torch.float64, device=dev)
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e9
    for _ in range(5):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return 2.0 * 4096 ** 3 / (best / 1e3) / 1e12


def pluq_run(args, L, sp, dev):
    """Full-rank PLUQ mod p26 at 16384^2 on both forms (limb tensor-core trailing
    products vs the plain Float64 ones), and the 1024^2 rank-900 PLUQ + RREF."""
    import numpy as np
    import torch
    import gffm
    import oracle
    from gffm import elimination
    out = {}
    out["limb"], fact = elimination.bench_pluq(args.pluq, sp, dev, reps=2, outputs=True)
    # the factorization just timed, checked outside the timed runs
    out["check"] = check_pluq(*fact)
    out["check_ok"] = all(out["check"].values())
    del fact
    if not args.no_pluq_plain and args.only != "pluq":
        out["plain"] = elimination.bench_pluq(args.pluq, sp, dev, reps=1, method="plain", warmup=0)
        out["limb_speedup"] = round(out["plain"]["seconds"] / out["limb"]["seconds"], 1)
    # 1024 x 1024 of rank 900: (1024 x 900)(900 x 1024) mod p26, seeded
    rng = np.random.default_rng(900)
    X = rng.integers(0, P26, size=(1024, 900))
    Y = rng.integers(0, P26, size=(900, 1024))
    A = gffm.CuModMatrix(oracle.matmul(X, Y, P26), P26, elem_type=torch.float64)
    t = {}
    for name, fn in (("pluq", lambda: gffm.pluq_gpu_kernel(A)), ("rref", lambda: gffm.rref_gpu_type(A))):
        fn()
        torch.cuda.synchronize()
        best = 1e9
        for _ in range(5):
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            best = min(best, time.perf_counter() - t0)
        t[name + "_ms"] = round(best * 1e3, 3)
    t["rank"] = elimination.pluq_rank(A)
    out["rank900_1024"] = t
    # the CPU elimination beside it: the oracle's exact restatement of the reference's
    # step-by-step algorithm (one host thread) on the same 1024 x 1024 rank-900 matrix
    Ah = oracle.matmul(X, Y, P26)
    t0 = time.perf_counter()
    oracle.pluq(Ah, P26)
    cpu_s = time.perf_counter() - t0
    out["rank900_1024"]["cpu_pluq_ms"] = round(cpu_s * 1e3, 1)
    out["rank900_1024"]["cpu_kind"] = "port (oracle/or_pluq, 1 thread)"
    # inverse of a 4096 x 4096 matrix mod p26 (RREF of [A | I]) and of the config-2 size
    g = torch.Generator(device=dev)
    g.manual_seed(41)
    for n in (1024, 4096):
        B = gffm.rand(torch.float64, n, n, P26, generator=g)
        gffm.inverse(B)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        gffm.inverse(B)
        torch.cuda.synchronize()
        out["inverse_%d_ms" % n] = round((time.perf_counter() - t0) * 1e3, 2)
    return out


def dev_int64(M):
    """The true-size contents of a CuModArray as an int64 (rows x cols) Fortran-ordered host array."""
    import torch
    r, c = M.size
    return M.data[:c, :r].to(torch.int64).cpu().numpy().T


def check_pluq(A, U, L, rs, cs, width=256):
    """Exact host checks of a full-rank factorization P A = L U mod p26: Freivalds on two
    vectors, U unit upper / L lower with pivots on the diagonal (sampled rows), no column
    swaps, and the first `width` pivot steps equal to the oracle's factorization of the
    leading column block."""
    import numpy as np
    from oracle import checks
    n = A.size[0]
    Ah, Uh, Lh = dev_int64(A), dev_int64(U), dev_int64(L)
    rng = np.random.default_rng(16384)
    rows = rng.integers(0, n, size=64)
    out = {"no_col_swaps": cs == [],
           "freivalds_LU_eq_PA": checks.freivalds_pluq(Ah, Uh, Lh, rs, P26, rng),
           "unit_upper_U": bool((np.diag(Uh) == 1).all()) and all((Uh[i, :i] == 0).all() for i in rows),
           "lower_L": bool((np.diag(Lh) != 0).all()) and all((Lh[i, i + 1:] == 0).all() for i in rows)}
    w = min(width, n)
    blk = checks.pluq_leading_block(Ah[:, :w], Uh[:w, :w], Lh[:, :w], rs, P26)
    out.update({"first_%d_steps_%s" % (w, k): v for k, v in blk.items()})
    return out


def config1_run(L, sp, dev):
    """The reference's single-stripe product at its own size: 512 x 512 mod 65521, Float64
    CuModMatrix operands, on both paths; microseconds per product, exact against the oracle."""
    import numpy as np
    import torch
    import gffm
    import oracle
    n, p = 512, 65521
    rng = np.random.default_rng(512)
    Ah = rng.integers(0, p, size=(n, n))
    Bh = rng.integers(0, p, size=(n, n))
    A = gffm.CuModMatrix(Ah, p, elem_type=torch.float64)
    B = gffm.CuModMatrix(Bh, p, elem_type=torch.float64)
    want = oracle.matmul(Ah, Bh, p)
    out = {"size": n, "modulus": p, "ops": 2 * n ** 3}
    for method in ("limb", "plain"):
        C = gffm.zeros(torch.float64, n, n, p)
        fn = lambda: gffm.mat_mul_type_inplace_(C, A, B, method=method)
        for _ in range(5):
            fn()
        torch.cuda.synchronize()
        reps = 200
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        us = e0.elapsed_time(e1) * 1e3 / reps
        out[method + "_us"] = round(us, 2)
        out[method + "_gops"] = round(2 * n ** 3 / us / 1e3, 1)
        out[method + "_exact"] = bool(np.array_equal(dev_int64(C), want))
    return out


def karatsuba_run(L, sp, dev):
    """4096^2 two-component products mod p25 (3 component products, 4.12e11 counted
    modular ops): the polynomial form, the reference's digit form (N1 = N2 = p25), and
    the 4-product schoolbook on the same GEMM for comparison."""
    import torch
    import gffm
    n, p = 4096, 33554393
    g = torch.Generator(device=dev)
    g.manual_seed(5)
    Ms = [gffm.rand(torch.float64, n, n, p, generator=g) for _ in range(4)]
    C = [gffm.zeros(torch.float64, n, n, p) for _ in range(3)]
    ws = ctypes.c_size_t(0)
    L.gffm_karatsuba_workspace_size(n, n, n, p, p, ctypes.byref(ws))
    wbuf = torch.empty(ws.value, dtype=torch.uint8, device=dev)
    d = [x.data.data_ptr() for x in Ms]
    c = [x.data.data_ptr() for x in C]
    ld = Ms[0].ld

    def poly():
        assert L.gffm_karatsuba_poly_matmul_f64(n, n, n, d[0], d[1], ld, d[2], d[3], ld, c[0], c[1], c[2], ld, p,
                                                wbuf.data_ptr(), ws.value, sp) == 0

    def digit():
        assert L.gffm_karatsuba_matmul_f64(n, n, n, d[0], d[1], ld, d[2], d[3], ld, c[0], c[1], ld, p, p,
                                           wbuf.data_ptr(), ws.value, sp) == 0

    def timed(fn, reps=5):
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

    ops = 3 * 2.0 * n ** 3
    tp, td = timed(poly), timed(digit)
    # schoolbook: four products and one modular add (C1 = A0 B1 + A1 B0)
    T = gffm.zeros(torch.float64, n, n, p)

    def school4():
        for (a, b, cc) in ((0, 2, c[0]), (1, 3, c[2]), (0, 3, c[1]), (1, 2, T.data.data_ptr())):
            assert L.gffm_matmul_limb_f64(n, n, n, d[a], ld, d[b], ld, cc, ld, p, wbuf.data_ptr(), ws.value, sp) == 0
        assert L.gffm_add_f64(c[1], c[1], T.data.data_ptr(), C[1].data.numel(), p, sp) == 0

    ts = timed(school4)
    return {"size": n, "modulus": p, "ops_counted": ops,
            "poly_ms": round(tp, 3), "poly_gops": round(ops / tp / 1e6, 1),
            "digit_form_ms": round(td, 3), "digit_form_gops": round(ops / td / 1e6, 1),
            "schoolbook4_ms": round(ts, 3), "karatsuba_speedup_vs_schoolbook": round(ts / tp, 2)}


def check_batch(specs, inst, results):
    """Freivalds (exact, on the host) for every product C = A B and every PLUQ L U = P A of
    a batch; PLUQs must be full rank (no column swaps, unit diagonal of U)."""
    import numpy as np
    from oracle import checks
    rng = np.random.default_rng(4096)
    failed, products, pluqs = [], 0, 0
    for i, ((op, n, p), spec, got) in enumerate(zip(specs, inst, results)):
        if op == "matmul":
            products += 1
            ok = checks.freivalds_product(dev_int64(spec[1]), dev_int64(spec[2]), dev_int64(got), p, rng)
        else:
            pluqs += 1
            if not isinstance(got, tuple):
                ok = False
            else:
                U, L, rs, cs = got
                Uh = dev_int64(U)
                ok = (cs == [] and bool((np.diag(Uh) == 1).all())
                      and checks.freivalds_pluq(dev_int64(spec[1]), Uh, dev_int64(L), rs, p, rng))
        if not ok:
            failed.append(i)
    return {"products_checked": products, "pluqs_checked": pluqs, "failed": len(failed),
            "first_failed": failed[:8], "method": "Freivalds, 2 vectors per instance, exact mod p on the host"}


def batched_run(args, dev, large_gemm_gops):
    """The batched uneven-instance workload: 4096 instances, n uniform over the multiples
    of 32 in [32, 512], p over the 32 fixed primes, half products half PLUQs, one graph."""
    import torch
    import gffm
    from gffm import batched
    if args.batch_uniform:
        count, n = (int(x) for x in args.batch_uniform.lower().split("x"))
        specs = [("pluq", n, P26)] * count
    else:
        specs = batched.config4_specs(args.batch, seed=1234)
    g = torch.Generator(device=dev)
    g.manual_seed(1234)
    inst = batched.build_config4(specs, generator=g)
    if args.batch_pluqs:
        keep = [i for i, s in enumerate(specs) if s[0] == "pluq"]
        specs, inst = [specs[i] for i in keep], [inst[i] for i in keep]
    ops = batched.ops_of(specs)

    def timed(plan, reps=5):
        plan.run()
        plan.run()
        plan.run()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            plan.run()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    plan = gffm.BatchPlan(inst, "auto")
    ms = timed(plan)
    info = [x for x in plan.pluq_info() if x is not None]
    full_rank = sum(1 for (op, n, _), x in zip([s for s in specs if s[0] == "pluq"], info) if x[2] == n)
    out = {"instances": len(specs), "ops": ops, "ms": round(ms, 3), "gops": round(ops / ms / 1e6, 1),
           "frac_of_large_gemm": round(ops / ms / 1e6 / large_gemm_gops, 3), "plan": plan.info(),
           "pluq_full_rank": "%d/%d" % (full_rank, len(info))}
    # every instance of the batch just timed, checked outside the timed runs
    out["check"] = check_batch(specs, inst, plan.results())
    out["check_ok"] = out["check"]["failed"] == 0
    if args.only == "batched":
        return out
    best = (ms, None)
    # the step route without branch overlap, and the per-instance kernel (32- and 16-column panels)
    for tu in ((0, 0, 0, 0, 0), (32, 0, 0, 1, 0), (16, 0, 0, 0, 0)):
        p2 = gffm.BatchPlan(inst, gffm.BatchTuning(*tu))
        t2 = timed(p2)
        out["tuning_%d_%d_%d_%d_%d_ms" % tu] = round(t2, 3)
        if t2 < best[0]:
            best = (t2, tu)
        del p2
    mm = gffm.BatchPlan([x for x in inst if x[0] == "matmul"])
    out["products_only_ms"] = round(timed(mm), 3)
    del mm
    pq = gffm.BatchPlan([x for x in inst if x[0] == "pluq"])
    out["pluqs_only_ms"] = round(timed(pq), 3)
    del pq
    if best[1] is not None:
        out["best_ms"] = round(best[0], 3)
        out["best_tuning"] = list(best[1])
        out["best_gops"] = round(ops / best[0] / 1e6, 1)
        out["best_frac_of_large_gemm"] = round(ops / best[0] / 1e6 / large_gemm_gops, 3)
    return out


def main():
    global M, N, K, WORKLOAD
    args = parse_args()
    if args.size != 8192:
        M = N = K = args.size
        WORKLOAD = WORKLOAD.replace("8192x8192x8192", "%dx%dx%d" % (M, N, K))
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
