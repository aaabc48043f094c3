"""Benchmark of the tall-skinny products on GB300, in the measurement contract of this repository.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

Default workload "tsmm-sweep" (the configuration the reference's GB/s-vs-M=N metric is quoted on):
TSMM C(KxN) = alpha A(KxM) B(MxN) + beta C with alpha = 1, beta = 0.5, FP64 and complex FP64,
M = N in {1,2,4,8,16,32,64} plus (M,N) in {(4,16),(16,4),(8,32)}, K chosen so A is 1 GiB, plus the
in-place form (C = A) for every M = N; entries U[-1,1) from a seeded generator.  One step runs every
shape once.  Each shape's operands are larger than L2 (129 MB), so no L2 flush is needed.

The default line also carries "split_vs_fp64" (TSMTTSM FP64 64x64, K = 2^24, s*2^e entries: plain
FP64 vs split precision vs double-double, with errors), "tsmttsm_sweep" (the metric's TSMTTSM half:
FP64 M = N in {1..64} with A and B of 1 GiB, and C1) and "serving" (C5: 20000 requests of the serving
mix through the request loop vs one launch per call); --no-extras skips them.

The reference arm (--impl reference) times the oracle port of the reference's loops on the host
cores (its value) and, on the default workload, the reference's own GPU kernels on the same box
("gpu_kernels": compiled from its headers into oracle/_ref, best variant and blockCount per shape).

Other workloads: "tsmttsm-c1" (TSMTTSM FP64 8x8, K = 2^20, 16 rotating input copies),
"precision-c3" (M = N in {32, 64, 128}), "svqb-c4", "serve-c5" (20000 requests), and probes for ncu.

Byte and flop formulas follow the reference's perf harness (perf.cu:208-232):
  TSMM beta != 0: (M K + 2 N K + M N) s bytes, in place (M K + N K + M N) s; flops (MNK + NK) f
  TSMTTSM: (M + N) K s bytes ((M K) s for Gram); flops M N K f;  f = 2 real, 8 complex.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "TSMTTSM/TSMM GB/s,%roofline vs M=N; split-vs-FP64 & served p99 at ≤1e-14 err"
SWEEP = [(1, 1), (2, 2), (4, 4), (8, 8), (16, 16), (32, 32), (64, 64), (4, 16), (16, 4), (8, 32)]
FALLBACK_HBM_GBS = 6800.0
# FP64 FMA peak of this GB300 measured with a DFMA throughput loop (2 flops per FMA): 595 G FMA/s.
FP64_PEAK_TFLOPS = 1.19


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return FALLBACK_HBM_GBS, "fallback"


# ----------------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while the timed region runs."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# -------------------------------------------------------------------------------- workloads
def tsmm_bytes(M, N, K, s, inplace):
    return (M * K + (1 if inplace else 2) * N * K + M * N) * s


def sweep_items(include_c64=True):
    items = []
    for dt in (["f64", "c64"] if include_c64 else ["f64"]):
        s = 8 if dt == "f64" else 16
        for (M, N) in SWEEP:
            K = (1 << 30) // (s * M)
            items.append(dict(op="tsmm", dt=dt, M=M, N=N, K=K, inplace=False, s=s))
    for (M, N) in SWEEP:
        if M == N:
            K = (1 << 30) // (8 * M)
            items.append(dict(op="tsmm", dt="f64", M=M, N=N, K=K, inplace=True, s=8))
    for it in items:
        f = 8 if it["dt"] == "c64" else 2
        it["bytes"] = tsmm_bytes(it["M"], it["N"], it["K"], it["s"], it["inplace"])
        it["flops"] = (it["M"] * it["N"] * it["K"] + it["N"] * it["K"]) * f
    return items


def c1_items():
    M = N = 8
    K = 1 << 20
    return [dict(op="tsmttsm", dt="f64", M=M, N=N, K=K, inplace=False, s=8, bytes=(M + N) * K * 8,
                 flops=2 * M * N * K, copies=16)]


def c3_items():
    K = 1 << 24
    return [dict(op="tsmttsm", dt="f64", M=M, N=M, K=K, inplace=False, s=8, bytes=2 * M * K * 8,
                 flops=2 * M * M * K, copies=1) for M in (32, 64, 128)]


def c4_items():
    K = 1 << 24
    return [dict(op="tsmttsm", dt="f64", M=M, N=M, K=K, inplace=False, s=8, bytes=3 * M * K * 8,
                 flops=4 * M * M * K, copies=1) for M in (16, 32, 64)]


def c5_items():
    reqs = c5_requests(200, 2024)
    return [dict(op=r["op"] if r["op"] != "svqb" else "tsmttsm", dt=r["dt"] if r["dt"] != "f32" else "f64",
                 M=r["M"], N=r["N"], K=r["K"] // 16 * 16 or 16, inplace=False, s=r["s"] if r["dt"] != "f32" else 8,
                 bytes=r["bytes"], flops=0) for r in reqs[:20]]


TS_SWEEP = (1, 2, 4, 8, 16, 32, 64)


def tsmttsm_sweep_items():
    """TSMTTSM FP64 C(MxM) = A^T B, M = N in {1..64}, A and B of 1 GiB each, alpha 1, beta 0."""
    items = []
    for M in TS_SWEEP:
        K = (1 << 30) // (8 * M)
        items.append(dict(op="tsmttsm", dt="f64", M=M, N=M, K=K, inplace=False, s=8, bytes=2 * M * K * 8,
                          flops=2 * M * M * K, copies=1))
    return items


def launch_time(fn, reps):
    """Mean device seconds of fn(1)..fn(reps), launched back to back on the current stream.  fn(0)
    runs first, untimed, and keeps the GPU busy while the timed launches are enqueued, so the
    events bracket device work only: a launch timed alone on an idle GPU would also count the
    host's call path (~20 us through Python), which is a fifth of a 100 us product.  Returns None
    when a call returns False (a launcher that refused the shape)."""
    import torch
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ok = fn(0) is not False
    e0.record()
    for i in range(1, reps + 1):
        ok = (fn(i) is not False) and ok
    e1.record()
    e1.synchronize()
    return e0.elapsed_time(e1) * 1e-3 / reps if ok else None


def tsmttsm_sweep(h, dev, reps=5):
    """The metric's TSMTTSM half: every shape of tsmttsm_sweep_items() plus C1 (8 x 8, K = 2^20, 16
    rotating input copies so the inputs exceed L2), each with the library's choice (auto) and the
    CUDA-core FP64 kernel (native): after two warm-ups, the mean device time of `reps` launches
    timed back to back with CUDA events (launch_time)."""
    import torch
    hbm, _ = peaks()
    rows = []
    for it in tsmttsm_sweep_items() + c1_items():
        ops = make_operands(it, dev, 500 + it["M"])
        row = {"M": it["M"], "N": it["N"], "K": it["K"], "config": "C1" if it.get("copies", 1) > 1 else "1 GiB"}
        for method in ("auto", "native"):
            for i in range(2):
                call(h, it, ops, i, method)
            t = launch_time(lambda i: call(h, it, ops, i, method), reps)
            gbs = it["bytes"] / t / 1e9
            row[method] = {"us": round(t * 1e6, 1), "GB/s": round(gbs, 1), "hbm_frac": round(gbs / hbm, 4),
                           "fp64_equivalent_tflops": round(it["flops"] / t / 1e12, 3),
                           "kernel": kernel_of(it, method)}
        rows.append(row)
        del ops
        torch.cuda.empty_cache()
    return rows


def probe_tsmm_items():
    M = N = 8
    K = 1 << 22
    it = dict(op="tsmm", dt="f64", M=M, N=N, K=K, inplace=False, s=8)
    it["bytes"] = tsmm_bytes(M, N, K, 8, False)
    it["flops"] = (M * N * K + N * K) * 2
    return [it]


def probe_tsmm64_items():
    M = N = 64
    K = 1 << 20
    it = dict(op="tsmm", dt="f64", M=M, N=N, K=K, inplace=False, s=8)
    it["bytes"] = tsmm_bytes(M, N, K, 8, False)
    it["flops"] = (M * N * K + N * K) * 2
    return [it]


def probe_tsmttsm_items():
    M = N = 8
    K = 1 << 22
    return [dict(op="tsmttsm", dt="f64", M=M, N=N, K=K, inplace=False, s=8, bytes=(M + N) * K * 8,
                 flops=2 * M * N * K, copies=1)]


def probe_tsmttsm1_items():
    K = 1 << 25
    return [dict(op="tsmttsm", dt="f64", M=1, N=1, K=K, inplace=False, s=8, bytes=2 * K * 8, flops=2 * K, copies=1)]


def probe_split_items():
    return probe_tsmttsm_items()


def probe_split_wide_items():
    M = N = 64
    K = 1 << 21
    return [dict(op="tsmttsm", dt="f64", M=M, N=N, K=K, inplace=False, s=8, bytes=(M + N) * K * 8,
                 flops=2 * M * N * K, copies=1)]


def probe_split_wide32_items():
    M = N = 32
    K = 1 << 22
    return [dict(op="tsmttsm", dt="f64", M=M, N=N, K=K, inplace=False, s=8, bytes=(M + N) * K * 8,
                 flops=2 * M * N * K, copies=1)]


WORKLOADS = {
    "probe-split-tsmm64": (probe_tsmm64_items, "TSMM FP64 64x64, K = 2^20 (512 MiB A), alpha 1, beta 0.5, run "
                           "with --method split: small case for ncu"),
    "probe-split-tsmm": (probe_tsmm_items, "TSMM FP64 8x8, K = 2^22, run with --method split: small case for ncu"),
    "probe-split": (probe_split_items, "TSMTTSM FP64 8x8, K = 2^22, run with --method split: small case for ncu"),
    "probe-split-wide": (probe_split_wide_items, "TSMTTSM FP64 64x64, K = 2^21 (2 x 1 GiB), run with --method "
                         "split: small case for ncu"),
    "probe-split-wide32": (probe_split_wide32_items, "TSMTTSM FP64 32x32, K = 2^22 (2 x 1 GiB), run with --method "
                           "split: folded stages, small case for ncu"),
    "probe-tsmm": (probe_tsmm_items, "TSMM FP64 8x8, K = 2^22 (256 MiB A), alpha 1, beta 0.5: small case for ncu"),
    "probe-tsmttsm": (probe_tsmttsm_items, "TSMTTSM FP64 8x8, K = 2^22 (2 x 256 MiB): small case for ncu"),
    "probe-tsmttsm1": (probe_tsmttsm1_items, "TSMTTSM FP64 1x1, K = 2^25 (2 x 256 MiB): small case for ncu"),
    "tsmm-sweep": (sweep_items, "TSMM FP64 + complex FP64, alpha 1, beta 0.5, A = 1 GiB per shape, "
                   "M=N in {1..64} + (4,16),(16,4),(8,32), plus in-place FP64 (C = A) for M = N"),
    "tsmttsm-sweep": (tsmttsm_sweep_items, "TSMTTSM FP64 C(MxM) = A^T B, M = N in {1..64}, A and B of 1 GiB "
                      "each, alpha 1, beta 0"),
    "tsmttsm-c1": (c1_items, "TSMTTSM FP64 C(8x8) = A^T B, K = 2^20, alpha 1, beta 0, "
                   "16 rotating input copies (2 GiB > L2)"),
    "group-small": (c5_items, "the serving mix's small requests (TSMTTSM / TSMM of cost <= 32 MiB, FP64 / complex "
                    "FP64 / FP32, operands in HBM): grouped launches vs one launch per request"),
    "serve-c5": (c5_items, "Poisson stream of TSMTTSM 50% / TSMM 35% / SVQB 15% requests, K log-uniform "
                 "[2^14, 2^24], M, N in {1..64}, FP64 60% / complex FP64 25% / FP32 15%, operands resident in "
                 "HBM; request loop vs one launch per call"),
    "svqb-c4": (c4_items, "SVQB of X (K = 2^24, M in {16, 32, 64}, condition 1e8), Gram in plain FP64, split "
                "precision or double-double; time and ||Q^T Q - I||_F"),
    "precision-c3": (c3_items, "TSMTTSM FP64 M = N in {32, 64, 128}, K = 2^24, entries s*2^e, plain FP64 vs "
                     "split precision vs double-double; normwise error against the double-double result"),
}


def torch_dtype(dt):
    import torch
    return {"f64": torch.float64, "c64": torch.complex128, "f32": torch.float32}[dt]


def make_operands(it, device, seed):
    import torch
    g = torch.Generator(device=device).manual_seed(seed)
    tdt = torch_dtype(it["dt"])

    def u(n):
        if tdt.is_complex:
            r = torch.rand(2 * n, dtype=torch.float64, device=device, generator=g) * 2 - 1
            return torch.view_as_complex(r.view(n, 2))
        return torch.rand(n, dtype=tdt, device=device, generator=g) * 2 - 1

    M, N, K = it["M"], it["N"], it["K"]
    if it["op"] == "tsmm":
        A = u(K * M)
        B = u(M * N)
        C = A if it["inplace"] else u(K * N)
        return dict(A=[A], B=[B], C=C)
    copies = it.get("copies", 1)
    return dict(A=[u(K * M) for _ in range(copies)], B=[u(K * N) for _ in range(copies)],
                C=torch.zeros(M * N, dtype=tdt, device=device))


def kernel_of(it, method):
    """The kernel family a shape runs on under `method`, by the library's selection rules (the ncu
    launch lists in profiles/ confirm them)."""
    M, N, K = it["M"], it["N"], it["K"]
    fp64 = it["dt"] in ("f64", "c64")
    if it["op"] == "tsmttsm":
        Mr, Nr = (2 * M, 2 * N) if it["dt"] == "c64" else (M, N)
        wide = Mr > 16 or Nr > 16
        nblk = ((Mr + 63) // 64) * ((Nr + 63) // 64)
        auto_split = K >= 4096 and (Mr * Nr >= 256 or (Mr >= 8 and Nr >= 8)) and \
            (not wide or Mr * Nr >= (128 if Mr <= 32 and Nr <= 32 else 320) * nblk)
        if fp64 and (method == "split" or (method == "auto" and auto_split)):
            return "split_wide_kernel" if wide else "split_tsmttsm_kernel"
        p2 = lambda x: 1 << (x - 1).bit_length()
        cap = 16 if it["dt"] == "c64" else 64  # register tiles of the row-streaming kernel
        if M <= 8 and N <= 8 and p2(M) * p2(N) <= cap:
            return "tsmttsm_rows_kernel"
        return "tsmttsm_kernel"
    Mr, Nr = (2 * M, 2 * N) if it["dt"] == "c64" else (M, N)
    auto_split = K >= 8192 and (Mr * Nr >= 128 or (it["dt"] == "c64" and Mr * Nr >= 64)) and Nr >= 8 and Mr >= 4
    if fp64 and (method == "split" or (method == "auto" and auto_split)):
        return "split_tsmm_kernel"
    return "tsmm_kernel"


def call(h, it, ops, i, method):
    M, N, K = it["M"], it["N"], it["K"]
    # FP64 and complex FP64 take the method (split covers complex TSMM); dd covers every dtype,
    # split FP64 and complex FP64 only
    acc = method if it["dt"] in ("f64", "c64") or method == "dd" else "native"
    if it["op"] == "tsmm":
        ld_c = M if it["inplace"] else N
        h.tsmm(M, N, K, ops["A"][0], M, 1.0, ops["B"][0], M, 0.5, ops["C"], ld_c, acc=acc)
    else:
        j = i % len(ops["A"])
        h.tsmttsm(M, N, K, ops["A"][j], M, 1.0, ops["B"][j], N, 0.0, ops["C"], M, acc=acc)


# ------------------------------------------------------------------------------ CPU baseline
def cpu_sample(items, seconds_budget=12.0):
    """Times the oracle's OpenMP loops (the reference harness's loop form) on a row sample of each
    shape; returns (GB/s, cores, description)."""
    import numpy as np
    from oracle import oracle as O
    rng = np.random.default_rng(1)
    cores = O.max_threads()
    tot_b, tot_t = 0.0, 0.0
    frac = 1 / 16
    for it in items:
        M, N = it["M"], it["N"]
        Ks = max(1024, int(it["K"] * frac))
        npdt = np.complex128 if it["dt"] == "c64" else np.float64
        def u(n):
            if npdt == np.complex128:
                return rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)
            return rng.uniform(-1, 1, n)
        A, B = u(Ks * M), u((M * N) if it["op"] == "tsmm" else Ks * N)
        if it["op"] == "tsmm":
            C = A if it["inplace"] else u(Ks * N)
            t0 = time.perf_counter()
            O.tsmm(M, N, Ks, A, M, 1.0, B, M, 0.5, C, M if it["inplace"] else N)
            dt = time.perf_counter() - t0
            tot_b += tsmm_bytes(M, N, Ks, it["s"], it["inplace"])
        else:
            C = np.zeros(M * N, dtype=npdt)
            t0 = time.perf_counter()
            O.tsmttsm(M, N, Ks, A, M, 1.0, B, N, 0.0, C, M)
            dt = time.perf_counter() - t0
            tot_b += (M + N) * Ks * it["s"]
        tot_t += dt
        if tot_t > seconds_budget:
            break
    return tot_b / tot_t / 1e9, cores, f"oracle OpenMP loops on every shape with K/16 rows (>=1024), {cores} threads"


# ------------------------------------------------------------------------------------- main
def dist_setup(n_gpus):
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    elif torch.cuda.is_available():
        torch.cuda.set_device(0)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def _reduce_device():
    """Where a reduction's tensor lives: the GPU under NCCL, the host under gloo (the CPU tests)."""
    import torch.distributed as dist
    return "cpu" if dist.get_backend() == "gloo" else "cuda"


def max_over_ranks(v, world):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device=_reduce_device())
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(v, world):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device=_reduce_device())
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


REF_TSMM_VARIANTS = {False: ("FIX3", "FIX_FB"), True: ("FIX3", "FIX_IP_GHOST")}
REF_TSMTTSM_VARIANTS = ("GENV5", "GENV3X", "SPECSMALL")


def reference_gpu_kernels(items, reps=3):
    """The reference's own GPU kernels (its headers compiled for sm_103a into oracle/_ref) timed on
    this machine's GPU, on the workload's real FP64 shapes they cover (the reference has no complex
    out-of-place TSMM kernel among those built, and GENV5 / SPECSMALL stop at M, N = 32), with its
    perf harness's launch search (perf.cu:166-190): blockCount = 1..8 x SMs, median of 3, best.
    Operands get the padding those kernels' over-reads need; alpha 1, beta 0.5 (TSMM) / 0 (TSMTTSM)."""
    try:
        import torch
        if not torch.cuda.is_available():
            return {"unavailable": "no CUDA device"}
        from oracle import ref_gpu
        msg = ref_gpu.init()
        if msg:
            return {"unavailable": msg}
    except Exception as e:  # noqa: BLE001
        return {"unavailable": f"{type(e).__name__}: {e}"}
    hbm, _ = peaks()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    out, tot_b, tot_t = [], 0.0, 0.0
    g = torch.Generator(device="cuda").manual_seed(99)
    for it in items:
        if it["dt"] != "f64":
            continue
        M, N, K = it["M"], it["N"], it["K"]
        tsmm = it["op"] == "tsmm"
        if not tsmm and max(M, N) > 32:
            continue
        copies = it.get("copies", 1)

        def rnd(n):
            t = ref_gpu.padded(n, torch.float64)
            t.copy_(torch.rand(n, dtype=torch.float64, device="cuda", generator=g) * 2 - 1)
            return t
        if tsmm:
            A = [rnd(K * M)]
            B = [rnd(M * N)]
            C = A[0] if it["inplace"] else rnd(K * N)
            variants = REF_TSMM_VARIANTS[it["inplace"]]
        else:
            A = [rnd(K * M) for _ in range(copies)]
            B = [rnd(K * N) for _ in range(copies)]
            C = rnd(M * N)
            variants = REF_TSMTTSM_VARIANTS
        temp = torch.empty(8 * sms * N * M * 8 + 256, dtype=torch.uint8, device="cuda")
        best = {}
        for v in variants:
            for bc in ([sms] if v == "FIX_IP_GHOST" else [sms * m for m in range(1, 9)]):
                def one(r):
                    if tsmm:
                        return ref_gpu.tsmm(v, M, N, K, A[0], M, 1.0, B[0], M, 0.5, C, M if it["inplace"] else N,
                                            bc)
                    return ref_gpu.tsmttsm(v, M, N, K, A[r % copies], M, 1.0, B[r % copies], N, 0.0, C, M, bc,
                                           temp=temp)
                if not one(0):
                    continue
                t = launch_time(one, reps)
                if t is None:
                    continue
                if v not in best or t < best[v][0]:
                    best[v] = (t, bc)
        del A, B, C, temp
        torch.cuda.empty_cache()
        if not best:
            continue
        vbest = min(best, key=lambda k: best[k][0])
        t, bc = best[vbest]
        gbs = it["bytes"] / t / 1e9
        tot_b += it["bytes"]
        tot_t += t
        out.append({"op": it["op"], "M": M, "N": N, "K": K, "inplace": it["inplace"], "best": vbest,
                    "blockCount": bc, "us": round(t * 1e6, 1), "GB/s": round(gbs, 1), "hbm_frac": round(gbs / hbm, 4),
                    "variants_GBs": {k: round(it["bytes"] / v[0] / 1e9, 1) for k, v in best.items()}})
    return {"what": "the reference's own GPU kernels, compiled from its headers for sm_103a, best variant and "
                    "blockCount per shape (its perf harness's search)",
            "aggregate_GBs": round(tot_b / tot_t / 1e9, 1) if tot_t else None, "shapes": out}


def run_reference(args):
    """The reference arm: the reference has no CPU implementation of its products (its own oracle
    is cuBLAS), so this arm times the oracle port of its loops on the host cores.  Beside that
    value it reports the reference's own GPU kernels on the same box (reference_gpu_kernels)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    items = WORKLOADS[args.workload][0]()
    vals = []
    for _ in range(args.warmup):
        cpu_sample(items[:1], 2.0)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        v, cores, desc = cpu_sample(items, seconds_budget=max(2.0, 60.0 / max(1, args.steps)))
        vals.append(v)
    wall = time.perf_counter() - t0
    v = sum(vals) / len(vals)
    line = {"metric": METRIC, "value": round(v, 3), "unit": "GB/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(wall / args.steps * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic U[-1,1) seeded",
            "config": {"workload": args.workload, "description": WORKLOADS[args.workload][1]},
            "impl": "reference",
            "cpu_baseline": {"value": round(v, 3), "unit": "GB/s", "cores": cores, "kind": "port", "sample": desc},
            "e2e": {"value": round(v, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if args.workload == "tsmm-sweep" and not args.no_extras:
        line["gpu_kernels"] = reference_gpu_kernels(items + tsmttsm_sweep_items() + c1_items())
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="tsmm-sweep", choices=sorted(WORKLOADS))
    ap.add_argument("--method", default="auto", choices=["auto", "native", "split", "dd"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--requests", type=int, default=20000, help="serve-c5: number of requests")
    ap.add_argument("--store", default=None, help="append every measured shape to this JSONL results store")
    ap.add_argument("--no-extras", action="store_true",
                    help="default workload: skip the compact split-vs-FP64 and serving measurements")
    ap.add_argument("--rate", type=float, default=2000.0, help="serve-c5: Poisson arrival rate per second")
    ap.add_argument("--streams", type=int, default=8, help="serve-c5: request-loop streams")
    ap.add_argument("--inflight", type=int, default=16, help="serve-c5: requests in flight at most")
    ap.add_argument("--group-bytes", type=int, default=32 << 20,
                    help="serve-c5: requests up to this many bytes run in grouped launches (0: off)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "precision-c3":
        return run_precision(args)
    if args.workload == "svqb-c4":
        return run_svqb(args)
    if args.workload == "serve-c5":
        return run_serve(args)
    if args.workload == "group-small":
        return run_group(args)

    import torch
    from skinny_matmul_gb300 import Handle, build, lib
    rank, world, local = dist_setup(args.gpus)
    build.build()
    h = Handle(torch.cuda.current_device())
    L = lib.load()
    items = WORKLOADS[args.workload][0]()
    dev = torch.device("cuda", torch.cuda.current_device())
    ops = [make_operands(it, dev, 1000 + i + 77 * rank) for i, it in enumerate(items)]
    torch.cuda.synchronize()

    def step(i, events=None):
        for j, (it, op) in enumerate(zip(items, ops)):
            if events is not None:
                events[j][0].record()
            call(h, it, op, i, args.method)
            if events is not None:
                events[j][1].record()

    for i in range(args.warmup):
        step(i)
    torch.cuda.synchronize()
    h.check_device()

    # ---- timed region: K steps, barrier + synchronize on both sides, CUDA events per launch
    ev = [[(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in items]
          for _ in range(args.steps)]
    e_start, e_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n0 = L.skinny_kernel_launches()
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        e_start.record()
        for i in range(args.steps):
            step(i, ev[i])
        e_end.record()
        torch.cuda.synchronize()
    barrier(world)
    launches = L.skinny_kernel_launches() - n0
    total_ms = e_start.elapsed_time(e_end)
    total_ms = max_over_ranks(total_ms, world)
    bytes_step = sum(it["bytes"] for it in items)
    flops_step = sum(it["flops"] for it in items)
    all_bytes = sum_over_ranks(bytes_step * args.steps, world)
    value = all_bytes / (total_ms * 1e-3) / 1e9
    hbm, peak_kind = peaks()

    # per-shape table and the dominant kernel's roofline (sum over its launches)
    per = []
    kern_ms = 0.0
    by_kernel = {}
    for j, it in enumerate(items):
        ts = sorted(ev[i][j][0].elapsed_time(ev[i][j][1]) for i in range(args.steps))
        t = ts[len(ts) // 2] * 1e-3
        kern_ms += sum(ev[i][j][0].elapsed_time(ev[i][j][1]) for i in range(args.steps))
        kname = kernel_of(it, args.method)
        kb, kt, kf = by_kernel.get(kname, (0.0, 0.0, 0.0))
        by_kernel[kname] = (kb + it["bytes"], kt + t, kf + it["flops"])
        gbs = it["bytes"] / t / 1e9
        tf = it["flops"] / t / 1e12
        per.append({"op": it["op"], "dtype": it["dt"], "M": it["M"], "N": it["N"], "K": it["K"],
                    "inplace": it["inplace"], "us": round(t * 1e6, 1), "GB/s": round(gbs, 1),
                    "hbm_frac": round(gbs / hbm, 4), "TFLOP/s": round(tf, 3),
                    "fp64_frac": round(tf / (FP64_PEAK_TFLOPS * (1 if it["dt"] != "c64" else 1)), 4)})
    # the dominant kernel family (most of the step's time): its algorithmic bytes over its time
    step_achieved = bytes_step * args.steps / (kern_ms * 1e-3) / 1e9
    dom = max(by_kernel, key=lambda k: by_kernel[k][1])
    dom_b, dom_t, dom_f = by_kernel[dom]
    achieved = dom_b / dom_t / 1e9
    tot_t = sum(v[1] for v in by_kernel.values())
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                "frac": round(achieved / hbm, 4), "traffic": TRAFFIC.get(args.workload),
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind,
                "kernel": dom, "traffic_probe": PROBE_TRAFFIC.get(args.workload),
                "kernel_time_shares": {k: round(v[1] / tot_t, 3) for k, v in by_kernel.items()},
                "fp64_equivalent_tflops": round(dom_f / dom_t / 1e12, 3),
                "fp64_peak_tflops_measured": FP64_PEAK_TFLOPS,
                "step": {"achieved": round(step_achieved, 1), "frac": round(step_achieved / hbm, 4),
                         "fp64_equivalent_tflops": round(flops_step * args.steps / (kern_ms * 1e-3) / 1e12, 3)}}

    # ---- end to end through the public API with pinned host buffers
    e2e = None
    if not args.no_e2e:
        e2e = measure_e2e(h, items, ops, args, world)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        v, cores, desc = cpu_sample(items)
        cpu = {"value": round(v, 3), "unit": "GB/s", "cores": cores, "kind": "port", "sample": desc}

    # the metric's other two parts, measured compactly beside the sweep on the same GPU: split vs
    # plain FP64 TSMTTSM (M = N = 64, K = 2^24, s*2^e data) and the served stream (C5, 20000 requests)
    extras = {}
    if args.workload == "tsmm-sweep" and world == 1 and not args.no_extras:
        del ops
        torch.cuda.empty_cache()
        rows, _, _ = precision_rows(h, dev, (64,), 3, 2, rank, world)
        byk = {r["method"]: r for r in rows}
        extras["split_vs_fp64"] = {
            "config": "TSMTTSM FP64 M = N = 64, K = 2^24, entries s*2^e (e in [-20, 20]); errors normwise "
                      "against the double-double result",
            "native_ms": byk["native"]["ms"], "split_ms": byk["split"]["ms"], "dd_ms": byk["dd"]["ms"],
            "speedup": byk["split"]["speedup_vs_native"], "split_err": byk["split"]["normwise_err_vs_dd"],
            "native_err": byk["native"]["normwise_err_vs_dd"]}
        extras["tsmttsm_sweep"] = {
            "config": "TSMTTSM FP64 C(MxM) = A^T B, M = N in {1..64}, A and B of 1 GiB each (> L2), plus C1 "
                      "(8 x 8, K = 2^20, 16 rotating copies); auto = the library's choice, native = CUDA-core FP64",
            "shapes": tsmttsm_sweep(h, dev)}
        seq, srv, _, wall_srv = serve_measure(h, dev, 20000, 2000.0, rank)
        extras["serving"] = {
            "config": "C5: 20000 requests of the serving mix (Poisson, 2000/s), operands resident in HBM",
            "served": srv, "one_launch_per_call": seq, "throughput_ratio": round(seq["wall_s"] / wall_srv, 3),
            "p99_ratio": round(srv["p99_ms"] / seq["p99_ms"], 3) if seq["p99_ms"] else None}

    if rank == 0 and args.store:
        from skinny_matmul_gb300 import results
        device = torch.cuda.get_device_name(dev)
        for it, r in zip(items, per):
            results.record(args.store, {
                "multype": it["op"].upper(), "device": device, "types": it["dt"], "M": it["M"], "N": it["N"],
                "name": f"gb300-{args.method}", "inplace": int(it["inplace"]), "zerobeta": int(it["op"] == "tsmttsm"),
                "K": it["K"], "time": r["us"] * 1e-6, "flops": r["TFLOP/s"] * 1e3, "bw": r["GB/s"],
                "blockCount": 0})
    if rank == 0:
        line = {"metric": METRIC, "value": round(value, 1), "unit": "GB/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 3), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic U[-1,1) from a seeded generator",
                "config": {"workload": args.workload, "description": WORKLOADS[args.workload][1],
                           "method_fp64": args.method, "l2": "operands larger than L2 (no flush needed)",
                           "parallelism": "replicas" if world > 1 else "single GPU"},
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(launches),
                "clocks": clk.summary(), "sweep": per}
        line.update(extras)
        print(json.dumps(line), flush=True)
    h.check_device()
    h.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


# DRAM bytes per step of the dominant kernel from one ncu capture (profiles/), or None.
TRAFFIC = {}
# DRAM traffic of one launch of the dominant kernel family, captured by ncu on a probe shape (the
# family's launches differ in size, so one per-launch figure of the step does not exist).
PROBE_TRAFFIC = {
    "tsmm-sweep": {"kernel": "split_tsmm_kernel<64>", "shape": "FP64 TSMM 64 x 64, K = 2^20, beta 0.5",
                   "dram_bytes": 1073.9e6 + 486.3e6, "algorithmic_bytes": 1611e6},
}


# ------------------------------------------------------------------------------ serving (C5)
C5_WIDTHS = (1, 2, 4, 8, 16, 32, 64)


def c5_requests(n, seed):
    """The serving mix: TSMTTSM 50 %, TSMM 35 %, SVQB 15 %; K log-uniform in [2^14, 2^24]; M, N
    from {1, 2, 4, 8, 16, 32, 64}; FP64 60 %, complex FP64 25 %, FP32 15 % (SVQB: FP64)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    reqs = []
    for _ in range(n):
        op = str(rng.choice(["tsmttsm", "tsmm", "svqb"], p=[0.5, 0.35, 0.15]))
        dt = str(rng.choice(["f64", "c64", "f32"], p=[0.6, 0.25, 0.15]))
        if op == "svqb":
            dt = "f64"
        K = int(2 ** rng.uniform(14, 24))
        M = int(rng.choice(C5_WIDTHS))
        N = M if op == "svqb" else int(rng.choice(C5_WIDTHS))
        s = {"f64": 8, "c64": 16, "f32": 4}[dt]
        if op == "tsmttsm":
            by = (M + N) * K * s
        elif op == "tsmm":
            by = (M * K + N * K + M * N) * s  # beta = 0
        else:
            by = 3 * K * M * 8
        reqs.append(dict(op=op, dt=dt, K=K, M=M, N=N, s=s, bytes=by, u=float(rng.random()), v=float(rng.random())))
    return reqs


class C5Pools:
    """Operands resident in HBM: one FP64 pool (read as FP64 or interleaved complex FP64), one FP32
    pool, an SVQB pool (updated in place), and output scratch.  A request reads a slice of a pool at
    a seeded offset; outputs (alpha = 1, beta = 0) go to scratch that no request reads."""

    def __init__(self, dev, seed, elems=(1 << 24) * 64 * 2, elems32=(1 << 24) * 64):
        """elems / elems32: the largest FP64 (complex: two doubles per element) and FP32 operand of
        any request (defaults: K = 2^24, width 64)."""
        import torch
        g = torch.Generator(device=dev).manual_seed(seed)
        n64 = elems + (1 << 20)
        self.p64 = torch.rand(n64, dtype=torch.float64, device=dev, generator=g) * 2 - 1
        self.p32 = torch.rand(elems32 + (1 << 20), dtype=torch.float32, device=dev, generator=g) * 2 - 1
        self.psv = torch.randn(elems * 3 // 2, dtype=torch.float64, device=dev, generator=g)
        self.out = torch.empty(elems, dtype=torch.float64, device=dev)
        self.outs = torch.empty(1 << 16, dtype=torch.float64, device=dev)

    def slice(self, pool, count, u):
        off = int(u * (pool.numel() - count)) & ~255
        return pool[off:off + count]

    def operands(self, r):
        """(A, B, C) device views for request r; element counts in the pool's own type."""
        M, N, K = r["M"], r["N"], r["K"]
        w = 2 if r["dt"] == "c64" else 1  # doubles per element
        if r["op"] == "svqb":
            X = self.slice(self.psv, K * M, r["u"])
            return X, None, X
        pool = self.p32 if r["dt"] == "f32" else self.p64
        A = self.slice(pool, K * M * w, r["u"])
        if r["op"] == "tsmttsm":
            B = self.slice(pool, K * N * w, r["v"])
            C = self.outs[: M * N * w] if r["dt"] != "f32" else self.outs.view(torch_f32())[: M * N]
        else:
            B = self.slice(pool, M * N * w, r["v"])
            C = self.out[: K * N * w] if r["dt"] != "f32" else self.out.view(torch_f32())[: K * N]
        return A, B, C


def torch_f32():
    import torch
    return torch.float32


def c5_call(h, r, ops, stream=None):
    from skinny_matmul_gb300 import lib as SL
    A, B, C = ops
    acc = "auto" if r["dt"] != "f32" else "native"
    dt = {"f64": SL.R64, "c64": SL.C64, "f32": SL.R32}[r["dt"]]
    if r["op"] == "svqb":
        h.svqb(r["K"], r["M"], C, r["M"], gram_acc="auto", orth_err=False, stream=stream)
    elif r["op"] == "tsmttsm":
        h.tsmttsm(r["M"], r["N"], r["K"], A, r["M"], 1.0, B, r["N"], 0.0, C, r["M"], acc=acc, stream=stream, dtype=dt)
    else:
        h.tsmm(r["M"], r["N"], r["K"], A, r["M"], 1.0, B, r["M"], 0.0, C, r["N"], acc=acc, stream=stream, dtype=dt)


def serve_measure(h, dev, n, rate, rank, streams=8, inflight=16, group_bytes=32 << 20):
    """Run the C5 stream both ways; returns (one-per-call stats, served stats, bytes, served wall)."""
    import numpy as np
    import torch
    from skinny_matmul_gb300 import Server, lib
    reqs = c5_requests(n, 2024 + rank)
    pools = C5Pools(dev, 99 + rank)
    ops = [pools.operands(r) for r in reqs]
    total_bytes = float(sum(r["bytes"] for r in reqs))
    rng = np.random.default_rng(7 + rank)
    gaps = rng.exponential(1.0 / rate, n)
    arrivals = np.cumsum(gaps) - gaps[0]
    # warm-up: every (op, dtype, width) kind once, small K
    seen = set()
    for r, o in zip(reqs, ops):
        key = (r["op"], r["dt"], r["M"], r["N"])
        if key not in seen:
            seen.add(key)
            c5_call(h, dict(r, K=min(r["K"], 1 << 14)), o)
    torch.cuda.synchronize()
    h.check_device()

    def one_per_call():
        lat = []
        t0 = time.perf_counter()
        for i, (r, o) in enumerate(zip(reqs, ops)):
            while time.perf_counter() - t0 < arrivals[i]:
                pass
            c5_call(h, r, o)
            torch.cuda.synchronize()
            lat.append(time.perf_counter() - t0 - arrivals[i])
        return time.perf_counter() - t0, lat

    def served():
        srv = Server(h, 120 * (1 << 30), num_streams=streams, max_inflight=inflight, group_bytes=group_bytes)
        tickets = []
        t0 = time.perf_counter()
        for i, (r, o) in enumerate(zip(reqs, ops)):
            while time.perf_counter() - t0 < arrivals[i]:
                pass
            A, B, C = o
            dt = {"f64": "float64", "c64": "complex128", "f32": "float32"}[r["dt"]]
            acc = "auto" if r["dt"] != "f32" else "native"
            if r["op"] == "svqb":
                st, t = srv.submit("svqb", dt, r["M"], r["M"], r["K"], C, r["M"], None, 0, C, r["M"], 1.0, 0.0, "auto",
                                   device=True)
            elif r["op"] == "tsmttsm":
                st, t = srv.submit("tsmttsm", dt, r["M"], r["N"], r["K"], A, r["M"], B, r["N"], C, r["M"], 1.0, 0.0,
                                   acc, device=True)
            else:
                st, t = srv.submit("tsmm", dt, r["M"], r["N"], r["K"], A, r["M"], B, r["M"], C, r["N"], 1.0, 0.0,
                                   acc, device=True)
            if st != lib.OK:
                raise RuntimeError(f"submit failed: {st}")
            tickets.append(t)
        srv.drain(3600.0)
        wall = time.perf_counter() - t0
        stats = srv.stats()
        srv.close()
        return wall, stats

    wall_seq, lat_seq = one_per_call()
    wall_srv, st_srv = served()
    lat_seq = sorted(lat_seq)
    p = lambda v, q: v[min(len(v) - 1, int(round(q * (len(v) - 1))))]
    seq = {"GB/s": round(total_bytes / wall_seq / 1e9, 1), "requests_per_s": round(n / wall_seq, 1),
           "p50_ms": round(p(lat_seq, 0.5) * 1e3, 3), "p99_ms": round(p(lat_seq, 0.99) * 1e3, 3),
           "wall_s": round(wall_seq, 3)}
    srv = {"GB/s": round(total_bytes / wall_srv / 1e9, 1), "requests_per_s": round(n / wall_srv, 1),
           "p50_ms": round(st_srv["p50_latency_us"] / 1e3, 3), "p99_ms": round(st_srv["p99_latency_us"] / 1e3, 3),
           "wall_s": round(wall_srv, 3), "completed": int(st_srv["completed"]), "failed": int(st_srv["failed"]),
           "max_inflight_seen": int(st_srv["max_inflight_seen"]), "grouped": int(st_srv["grouped"]),
           "group_launches": int(st_srv["group_launches"]), "group_bytes": int(group_bytes),
           "peak_bytes_in_use": int(st_srv["peak_bytes_in_use"])}
    del pools, ops
    torch.cuda.empty_cache()
    return seq, srv, total_bytes, wall_srv


def run_serve(args):
    """A seeded Poisson stream of requests on operands resident in HBM, run two ways: through the
    request loop (continuous batching: admission by a 120 GB budget, up to 16 requests in flight on
    8 streams) and one launch per call (each request launched when it arrives and waited for before
    the next, as the reference's drivers call its launchers).  Throughput = algorithmic bytes of all
    requests / (last completion - first arrival); latency = completion - arrival."""
    import numpy as np
    import torch
    from skinny_matmul_gb300 import Handle, Server, build, lib
    rank, world, local = dist_setup(args.gpus)
    build.build()
    h = Handle(torch.cuda.current_device())
    L = lib.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    n = args.requests
    n0 = L.skinny_kernel_launches()
    with ClockSampler(local) as clk:
        seq, srv, total_bytes, wall_srv = serve_measure(h, dev, n, args.rate, rank, args.streams, args.inflight,
                                                        args.group_bytes)
    launches = L.skinny_kernel_launches() - n0
    h.check_device()
    value = sum_over_ranks(total_bytes / wall_srv / 1e9, world)
    if rank == 0:
        hbm, _ = peaks()
        line = {"metric": METRIC, "value": round(value, 1), "unit": "GB/s", "n_gpus": world, "steps": 1,
                "warmup": 1, "ms_per_step": round(wall_srv * 1e3, 3), "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "mixed (f64 60%, c64 25%, f32 15%)",
                "data": "synthetic U[-1,1) operands resident in HBM, seeded; Poisson arrivals",
                "config": {"workload": "serve-c5", "description": WORKLOADS["serve-c5"][1], "requests": n,
                           "arrival_rate_per_s": args.rate, "streams": args.streams, "max_inflight": args.inflight, "l2": "operands larger than L2 for most requests",
                           "parallelism": "replicas" if world > 1 else "single GPU"},
                "roofline": {"bound": "hbm", "achieved": round(value, 1), "peak": hbm, "unit": "GB/s",
                             "frac": round(value / hbm, 4), "traffic": None, "kernel": "request mix"},
                "serving": {"served": srv, "one_launch_per_call": seq,
                            "throughput_ratio": round(seq["wall_s"] / wall_srv, 3),
                            "p99_ratio": round(srv["p99_ms"] / seq["p99_ms"], 3) if seq["p99_ms"] else None},
                "gpu_launches": int(launches), "clocks": clk.summary(), "cpu_baseline": None, "e2e": None}
        print(json.dumps(line), flush=True)
    h.close()


# --------------------------------------------------------------------------------- SVQB (C4)
def svqb_operand(K, M, cond, gen, device):
    """X = G R: G standard Gaussian K x M, R upper triangular with singular values log-spaced from
    1 to 1/cond (R is the triangular factor of U diag(sigma) V^T, U and V orthogonal factors of
    seeded Gaussian matrices)."""
    import torch
    U, _ = torch.linalg.qr(torch.randn(M, M, dtype=torch.float64, device=device, generator=gen))
    V, _ = torch.linalg.qr(torch.randn(M, M, dtype=torch.float64, device=device, generator=gen))
    sig = torch.logspace(0, -math.log10(cond), M, dtype=torch.float64, device=device)
    _, R = torch.linalg.qr(U @ torch.diag(sig) @ V.T)
    G = torch.randn(K, M, dtype=torch.float64, device=device, generator=gen)
    return (G @ R).contiguous().view(-1)


def run_svqb(args):
    """SVQB of X (K = 2^24, M in {16, 32, 64}, condition 1e8): Gram S = X^T X, diagonal scaling,
    on-device FP64 eigensolve, X <- X (D^-1/2 U Lambda^-1/2) by in-place TSMM; the Gram in plain
    FP64, split precision or double-double.  Reports time and ||Q^T Q - I||_F per Gram method."""
    import torch
    from skinny_matmul_gb300 import Handle, build, lib
    rank, world, local = dist_setup(args.gpus)
    build.build()
    h = Handle(torch.cuda.current_device())
    L = lib.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    K = 1 << 24
    rows = []
    n0 = L.skinny_kernel_launches()
    total_bytes, total_ms = 0.0, 0.0
    with ClockSampler(local) as clk:
        for M in (16, 32, 64):
            g = torch.Generator(device=dev).manual_seed(777 + M + 13 * rank)
            X0 = svqb_operand(K, M, 1e8, g, dev)
            X = torch.empty_like(X0)
            for meth in ("native", "split", "dd"):
                ts, errs = [], []
                for it in range(max(1, args.warmup // 3) + max(1, min(args.steps, 3))):
                    X.copy_(X0)
                    torch.cuda.synchronize()
                    barrier(world)
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record()
                    h.svqb(K, M, X, M, gram_acc=meth, orth_err=False)
                    e1.record()
                    torch.cuda.synchronize()
                    if it >= max(1, args.warmup // 3):
                        ts.append(max_over_ranks(e0.elapsed_time(e1), world))
                X.copy_(X0)
                err = h.svqb(K, M, X, M, gram_acc=meth, orth_err=True)
                ms = sorted(ts)[len(ts) // 2]
                by = 3 * K * M * 8
                rows.append({"M": M, "K": K, "cond": 1e8, "gram": meth, "ms": round(ms, 3),
                             "GB/s": round(by / (ms * 1e-3) / 1e9, 1), "orth_err": err})
                total_bytes += by
                total_ms += ms
            del X0, X
            torch.cuda.empty_cache()
    launches = L.skinny_kernel_launches() - n0
    h.check_device()
    if rank == 0:
        hbm, _ = peaks()
        value = total_bytes / (total_ms * 1e-3) / 1e9
        line = {"metric": METRIC, "value": round(value, 1), "unit": "GB/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": round(total_ms, 3), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic X = G R (Gaussian G, triangular R with singular values 1..1e-8), seeded",
                "config": {"workload": "svqb-c4", "description": WORKLOADS["svqb-c4"][1],
                           "l2": "operands larger than L2 (no flush needed)",
                           "parallelism": "replicas" if world > 1 else "single GPU"},
                "roofline": {"bound": "hbm", "achieved": round(value, 1), "peak": hbm, "unit": "GB/s",
                             "frac": round(value / hbm, 4), "traffic": None, "kernel": "svqb pipeline",
                             "note": "3 K M 8 bytes per SVQB (Gram read, TSMM read and write)"},
                "svqb": rows, "gpu_launches": int(launches), "clocks": clk.summary(), "cpu_baseline": None,
                "e2e": None}
        print(json.dumps(line), flush=True)
    h.close()


# ------------------------------------------------------------------------------ grouped launches
def c5_cost(r):
    """A request's cost in bytes-equivalent as the request loop prices it for grouping: the larger
    of its bytes and its FMAs at ~11.3 bytes per FP64 FMA (0.18 per FP32 FMA)."""
    w = 4 if r["dt"] == "c64" else 1
    fma = r["M"] * r["N"] * w * r["K"] + (r["N"] * w * r["K"] if r["op"] == "tsmm" else 0)
    return max(r["bytes"], fma * (0.18 if r["dt"] == "f32" else 11.3))


def run_group(args):
    """The small requests of the serving mix (TSMTTSM / TSMM whose cost -- bytes, or FMAs priced at
    the HBM-to-FMA rate ratio -- is at most 32 MiB; operands resident in HBM) run three ways: grouped launches (skinny_group, one per dtype
    present), one launch per request back to back on one stream, and one launch per request with
    a synchronisation after each (as a caller of the reference's launchers would).  Reports
    algorithmic GB/s and microseconds per request of each."""
    import numpy as np
    import torch
    from skinny_matmul_gb300 import Handle, build, lib
    rank, world, local = dist_setup(args.gpus)
    build.build()
    h = Handle(torch.cuda.current_device())
    L = lib.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    n = min(args.requests, 4096)
    reqs = [r for r in c5_requests(40 * n, 4242 + rank) if r["op"] != "svqb" and c5_cost(r) <= (32 << 20)][:n]
    w = lambda r: 2 if r["dt"] == "c64" else 1
    need = [r["K"] * max(r["M"], r["N"]) * w(r) for r in reqs]
    pools = C5Pools(dev, 17 + rank, elems=max(need),
                    elems32=max([n for n, r in zip(need, reqs) if r["dt"] == "f32"] or [1]))
    ops = [pools.operands(r) for r in reqs]
    by_dt = {}
    for r, (A, B, C) in zip(reqs, ops):
        lda = r["M"]
        it = dict(op=r["op"], M=r["M"], N=r["N"], K=r["K"], A=A, lda=lda, B=B, ldb=r["N"] if r["op"] == "tsmttsm"
                  else r["M"], C=C, ldc=r["M"] if r["op"] == "tsmttsm" else r["N"], alpha=1.0, beta=0.0)
        by_dt.setdefault({"f64": "float64", "c64": "complex128", "f32": "float32"}[r["dt"]], []).append(it)
    total_bytes = float(sum(r["bytes"] for r in reqs))

    def grouped():
        for dt, items in by_dt.items():
            h.group(items, dtype=dt)

    def one_stream():
        for r, o in zip(reqs, ops):
            c5_call(h, r, o)

    def timed(fn, steps):
        ts = []
        for _ in range(steps):
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        return sorted(ts)[len(ts) // 2]

    n0 = L.skinny_kernel_launches()
    with ClockSampler(local) as clk:
        for _ in range(max(3, args.warmup)):
            grouped()
            one_stream()
        torch.cuda.synchronize()
        l0 = L.skinny_kernel_launches()
        ms_g = timed(grouped, max(1, args.steps))
        launches_g = (L.skinny_kernel_launches() - l0) // max(1, args.steps)
        ms_s = timed(one_stream, max(1, args.steps))
        t0 = time.perf_counter()
        for r, o in zip(reqs, ops):
            c5_call(h, r, o)
            torch.cuda.synchronize()
        ms_c = (time.perf_counter() - t0) * 1e3
    launches = L.skinny_kernel_launches() - n0
    h.check_device()
    if rank == 0:
        hbm, _ = peaks()
        gbs = lambda ms: round(total_bytes / (ms * 1e-3) / 1e9, 1)
        value = total_bytes / (ms_g * 1e-3) / 1e9
        line = {"metric": METRIC, "value": round(value, 1), "unit": "GB/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": round(ms_g, 3), "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "mixed (f64, c64, f32)",
                "data": "synthetic U[-1,1) operands resident in HBM, seeded",
                "config": {"workload": "group-small", "description": WORKLOADS["group-small"][1], "requests": len(reqs),
                           "bytes": total_bytes, "l2": "operands mostly L2-resident between steps (small requests)",
                           "parallelism": "replicas" if world > 1 else "single GPU"},
                "roofline": {"bound": "hbm", "achieved": round(value, 1), "peak": hbm, "unit": "GB/s",
                             "frac": round(value / hbm, 4), "traffic": None, "kernel": "group_kernel"},
                "group": {"grouped": {"ms": round(ms_g, 3), "GB/s": gbs(ms_g), "launches": int(launches_g),
                                      "us_per_request": round(ms_g * 1e3 / len(reqs), 2)},
                          "one_launch_per_request_one_stream": {"ms": round(ms_s, 3), "GB/s": gbs(ms_s),
                                                                "us_per_request": round(ms_s * 1e3 / len(reqs), 2)},
                          "one_launch_per_call_synchronised": {"ms": round(ms_c, 3), "GB/s": gbs(ms_c),
                                                               "us_per_request": round(ms_c * 1e3 / len(reqs), 2)}},
                "gpu_launches": int(launches), "clocks": clk.summary(), "cpu_baseline": None, "e2e": None}
        print(json.dumps(line), flush=True)
    del pools, ops
    h.close()


# ------------------------------------------------------------------------ precision (TSMTTSM C3)
def spread_operand(n, gen, device):
    """Entries s * 2^e: s uniform in [1, 2), random sign, e uniform integer in [-20, 20]."""
    import torch
    s = torch.rand(n, dtype=torch.float64, device=device, generator=gen) + 1.0
    sign = torch.randint(0, 2, (n,), device=device, generator=gen, dtype=torch.int32) * 2 - 1
    e = torch.randint(-20, 21, (n,), device=device, generator=gen, dtype=torch.int32)
    return torch.ldexp(s * sign, e)


def precision_rows(h, dev, widths, steps_split, warmup_split, rank, world, K=1 << 24):
    """Per width M = N: time native, split and dd TSMTTSM on s*2^e data and their normwise errors
    against the dd result.  Returns (rows, split bytes, split ms)."""
    import torch
    rows = []
    total_bytes, total_ms = 0.0, 0.0
    for M in widths:
        g = torch.Generator(device=dev).manual_seed(4242 + M + 13 * rank)
        A = spread_operand(K * M, g, dev)
        B = spread_operand(K * M, g, dev)
        out = {}
        for meth in ("dd", "native", "split"):
            C = torch.zeros(M * M, dtype=torch.float64, device=dev)
            for _ in range(max(1, warmup_split if meth == "split" else 1)):
                h.tsmttsm(M, M, K, A, M, 1.0, B, M, 0.0, C, M, acc=meth)
            steps = steps_split if meth == "split" else max(1, min(steps_split, 2))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            barrier(world)
            torch.cuda.synchronize()
            e0.record()
            for _ in range(steps):
                h.tsmttsm(M, M, K, A, M, 1.0, B, M, 0.0, C, M, acc=meth)
            e1.record()
            torch.cuda.synchronize()
            ms = max_over_ranks(e0.elapsed_time(e1) / steps, world)
            out[meth] = (C.clone(), ms)
            if meth == "split":
                total_bytes += 2 * M * K * 8 * steps
                total_ms += ms * steps
        A.abs_()
        B.abs_()
        D = torch.zeros(M * M, dtype=torch.float64, device=dev)
        h.tsmttsm(M, M, K, A, M, 1.0, B, M, 0.0, D, M, acc="native")
        den = float(torch.linalg.vector_norm(D))
        ref = out["dd"][0]
        for meth in ("native", "split", "dd"):
            C, ms = out[meth]
            err = float(torch.linalg.vector_norm(C - ref)) / den
            by = 2 * M * K * 8
            rows.append({"M": M, "N": M, "K": K, "method": meth, "ms": round(ms, 3),
                         "GB/s": round(by / (ms * 1e-3) / 1e9, 1),
                         "eff_fp64_tflops": round(2 * M * M * K / (ms * 1e-3) / 1e12, 2),
                         "normwise_err_vs_dd": err if meth != "dd" else 0.0})
        for r in rows[-3:]:
            r["speedup_vs_native"] = round(out["native"][1] / r["ms"], 2)
        del A, B, D, out
        torch.cuda.empty_cache()
    return rows, total_bytes, total_ms


def run_precision(args):
    """FP64 TSMTTSM C = A^T B at M = N in {32, 64, 128}, K = 2^24, entries s * 2^e, three ways:
    CUDA-core FP64 ("native"), split precision on the tensor cores ("split") and double-double
    accumulation ("dd", the reference's PseudoQuad form).  Errors are normwise,
    ||C - C_dd||_F / || |A|^T |B| ||_F, against the double-double result of the same launch data
    (the dd method itself is pinned against the exact super-accumulator by the GPU tests)."""
    import torch
    from skinny_matmul_gb300 import Handle, build, lib
    rank, world, local = dist_setup(args.gpus)
    build.build()
    h = Handle(torch.cuda.current_device())
    L = lib.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    n0 = L.skinny_kernel_launches()
    hbm, peak_kind = peaks()
    with ClockSampler(local) as clk:
        rows, total_bytes, total_ms = precision_rows(h, dev, (32, 64, 128), args.steps, args.warmup, rank, world)
    launches = L.skinny_kernel_launches() - n0
    h.check_device()
    value = total_bytes / (total_ms * 1e-3) / 1e9
    if rank == 0:
        split = {r["M"]: r for r in rows if r["method"] == "split"}
        line = {"metric": METRIC, "value": round(value, 1), "unit": "GB/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": round(total_ms / max(1, args.steps), 3),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic s*2^e (s U[1,2), random sign, e U{-20..20}) from a seeded generator",
                "config": {"workload": "precision-c3", "description": WORKLOADS["precision-c3"][1],
                           "l2": "operands larger than L2 (no flush needed)",
                           "parallelism": "replicas" if world > 1 else "single GPU"},
                "roofline": {"bound": "tensor", "kernel": "split_wide_kernel",
                             "achieved_eff_fp64_tflops": round(sum(split[m]["eff_fp64_tflops"] for m in split) / 3, 2),
                             "hbm_GB/s": round(value, 1), "hbm_peak": hbm, "hbm_frac": round(value / hbm, 4),
                             "note": "value = algorithmic bytes of the split launches / their time"},
                "split_vs_fp64": {str(m): {"speedup": split[m]["speedup_vs_native"],
                                           "err": split[m]["normwise_err_vs_dd"]} for m in split},
                "precision": rows, "gpu_launches": int(launches), "clocks": clk.summary(),
                "cpu_baseline": None, "e2e": None}
        print(json.dumps(line), flush=True)
    h.close()


def measure_e2e(h, items, ops, args, world):
    """Same metric through the public API with HOST buffers: every step copies each shape's inputs
    from pinned host memory to the device, runs the product and copies the result back to pinned
    host memory.  Pipelined as a caller streaming large products would: uploads on one stream,
    products on a second (each waits for its own upload), downloads on a third (each waits for its
    own product); a TSMM shape moves in row chunks of ~128 MB of A (its rows are independent, so
    the products on row slices give the same bits), so that a chunk's upload overlaps the previous
    chunk's product and download and both link directions stay busy (GB300's host link: 211 GB/s
    up, 194 GB/s down, 343 GB/s both ways at once)."""
    import torch
    maxA = max(o["A"][0].numel() * o["A"][0].element_size() for o in ops)
    maxB = max(o["B"][0].numel() * o["B"][0].element_size() for o in ops)
    maxC = max(o["C"].numel() * o["C"].element_size() for o in ops)
    hA = torch.empty(maxA, dtype=torch.uint8, pin_memory=True)
    hB = torch.empty(maxB, dtype=torch.uint8, pin_memory=True)
    hC = torch.empty(maxC, dtype=torch.uint8, pin_memory=True)
    hOut = torch.empty(maxC, dtype=torch.uint8, pin_memory=True)  # downloads never race uploads
    # host values must be finite numbers: fill as uniform doubles
    for t in (hA, hB, hC, hOut):
        d = t.view(torch.float64)
        d.uniform_(-1, 1)
    steps = max(1, min(args.steps, 3))
    s_in, s_cmp, s_out = torch.cuda.Stream(), torch.cuda.Stream(), torch.cuda.Stream()

    def as_bytes(t):
        return (torch.view_as_real(t) if t.is_complex() else t).view(torch.uint8)

    h2d = d2h = 0
    prev_out = [None] * len(items)  # a shape's download in the previous step

    chunk_bytes = 128 << 20

    def tsmm_chunks(i, it, op):
        """A TSMM shape in row chunks; returns the bytes moved up and down."""
        A, B, C = op["A"][0], op["B"][0], op["C"]
        M, N, K = it["M"], it["N"], it["K"]
        es = A.element_size()
        ldc = M if it["inplace"] else N
        acc = args.method if it["dt"] in ("f64", "c64") or args.method == "dd" else "native"
        rows = max(1024, chunk_bytes // (M * es))
        up_b = down_b = 0
        if prev_out[i] is not None:  # this shape's buffers are free once its last download ran
            s_in.wait_event(prev_out[i])
        with torch.cuda.stream(s_in):
            nB = B.numel() * es
            as_bytes(B).view(-1).copy_(hB[:nB], non_blocking=True)
            up_b += nB
        for r0 in range(0, K, rows):
            kc = min(rows, K - r0)
            Ac, Cc = A[r0 * M:(r0 + kc) * M], C[r0 * ldc:(r0 + kc) * ldc]
            a0, na, c0, nc = r0 * M * es, kc * M * es, r0 * ldc * es, kc * ldc * es
            up, done = torch.cuda.Event(), torch.cuda.Event()
            with torch.cuda.stream(s_in):
                as_bytes(Ac).view(-1).copy_(hA[a0:a0 + na], non_blocking=True)
                up_b += na
                if not it["inplace"]:
                    as_bytes(Cc).view(-1).copy_(hC[c0:c0 + nc], non_blocking=True)
                    up_b += nc
                up.record(s_in)
            s_cmp.wait_event(up)
            with torch.cuda.stream(s_cmp):
                h.tsmm(M, N, kc, Ac, M, 1.0, B, M, 0.5, Cc, ldc, acc=acc)
                done.record(s_cmp)
            s_out.wait_event(done)
            with torch.cuda.stream(s_out):
                hOut[c0:c0 + nc].copy_(as_bytes(Cc).view(-1), non_blocking=True)
                down_b += nc
        out = torch.cuda.Event()
        out.record(s_out)
        prev_out[i] = out
        return up_b, down_b

    def one():
        nonlocal h2d, d2h
        h2d = d2h = 0
        for i, (it, op) in enumerate(zip(items, ops)):
            if it["op"] == "tsmm":
                u, d = tsmm_chunks(i, it, op)
                h2d += u
                d2h += d
                continue
            A, B, C = op["A"][0], op["B"][0], op["C"]
            nA, nB, nC = (x.numel() * x.element_size() for x in (A, B, C))
            up, done, out = torch.cuda.Event(), torch.cuda.Event(), torch.cuda.Event()
            if prev_out[i] is not None:  # this shape's buffers are free once its last download ran
                s_in.wait_event(prev_out[i])
            with torch.cuda.stream(s_in):
                as_bytes(A).view(-1).copy_(hA[:nA], non_blocking=True)
                as_bytes(B).view(-1).copy_(hB[:nB], non_blocking=True)
                h2d += nA + nB
                if it["op"] == "tsmm" and not it["inplace"]:
                    as_bytes(C).view(-1).copy_(hC[:nC], non_blocking=True)
                    h2d += nC
                up.record(s_in)
            s_cmp.wait_event(up)
            with torch.cuda.stream(s_cmp):
                call(h, it, op, 0, args.method)
                done.record(s_cmp)
            s_out.wait_event(done)
            with torch.cuda.stream(s_out):
                hOut[:nC].copy_(as_bytes(C).view(-1), non_blocking=True)
                d2h += nC
                out.record(s_out)
            prev_out[i] = out

    def run(n):
        cur = torch.cuda.current_stream()
        for st in (s_in, s_cmp, s_out):
            st.wait_stream(cur)
        for _ in range(n):
            one()
        for st in (s_in, s_cmp, s_out):
            cur.wait_stream(st)

    run(1)
    torch.cuda.synchronize()
    barrier(world)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    run(steps)
    e1.record()
    torch.cuda.synchronize()
    ms = max_over_ranks(e0.elapsed_time(e1), world)
    b = sum_over_ranks(sum(it["bytes"] for it in items) * steps, world)
    return {"value": round(b / (ms * 1e-3) / 1e9, 1), "unit": "GB/s", "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h), "steps": steps,
            "pipeline": "upload / product / download streams, TSMM in row chunks of ~128 MB of A"}

if __name__ == "__main__":
    main()
