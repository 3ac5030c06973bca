"""Benchmark of the out-of-core tiled GEMM on GB300 (one JSON line on rank 0).

Metric: FP64-accurate TFLOP/s (2 m n k / time) of the Ozaki emulated-FP64 path,
reported beside the native FP64 (DMMA) path on the same inputs, with the
componentwise error metric of both against a twice-working-precision oracle.

Default workload (--workload ozaki32768): m = n = k = 32768, NN, entries u * 2^e
with u uniform [-1, 1) and e a uniform integer in [-20, 20] (seeded, synthetic),
alpha = 1, beta = 0, the slice count the smallest that meets the native path's
error on a calibration sub-problem of the same k and distribution; the error at
6..11 slices on the full problem is reported beside it.
  value    device-resident operands (tmm_gemm_device), CUDA-event timed
  e2e      the public host-pointer call (tmm_gemm) with pinned host buffers:
           every step copies A and B to the device and C back
Other workloads: native4096 (m = n = k = 4096 NN, uniform, alpha = beta = 1,
tiles 2048, 2 streams, pinned, copy_c_back), the out-of-core, batched, sweep
and float / complex workloads of the WORKLOADS table.

CPU baselines (rank 0, N = 1): a host dgemm through NumPy's BLAS on all host
cores (cpu_baseline, on a square sub-block of the workload), and the reference
algorithm's CPU restatement (the oracle, cpu_baseline_port).

--impl reference times the reference algorithm's CPU restatement (the oracle;
the reference itself is cuBLAS-backed GPU code whose sources are not present on
the GPU machine) on all host cores: every warm-up and timed step is one bounded
k-slab sample of the same workload.  It imports nothing of this library.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "tiled-mm_gb300"))

PEAKS_FILE = ROOT / "MEASURED_PEAKS.json"
# Instruction-rate ceilings on this machine's GB300, measured with the repository's own probes
# (tiled-mm_gb300/peaks/engine_rates.cu: dmma and imma mma.sync loops; tcgen05 e4m3 M128 N256 K32
# issued back to back from shared memory) and the vendor library's dense e4m3 GEMM
# (tiled-mm_gb300/peaks/cublaslt_e4m3.py, 8192^3).  The tcgen05 pipe retires 16384 e4m3 FLOP per
# clock and SM (512 cycles per 128 x 256 x 128 k-block): the tensor roofline of the slice-product
# kernel is that rate at the SM clock measured during the timed region.
# tcgen05_e4m3_sustained_digits_tflops: the CTA-pair instruction back to back on digit operands
# for about a second, at the power limit (512 cycles per k-block at ~1.71 GHz), the ceiling of
# a kernel that keeps the pipe busy for a whole long launch
MEASURED_ENGINE_PEAKS = {"imma_s8_tops": 157.9, "dmma_f64_tflops": 1.099,
                         "tcgen05_e4m3_tflops": 4847.2, "cublaslt_e4m3_tflops": 3948.0,
                         "tcgen05_e4m3_sustained_digits_tflops": 4262.0}
TCGEN05_E4M3_FLOP_PER_CLK_SM = 16384.0
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one slice-product launch, from one
# ncu capture of a smaller launch with the headline's k tile and slice count (m = n = 8192,
# k = 16384, 11 slices: the same per-tile sequence, 2048 tiles instead of 32768); a launch of
# another shape is scaled by its units (tiles x slice pairs x k-blocks), which assumes the
# traffic per unit does not depend on the number of tiles.  None: no capture for this engine.
ENGINE_DRAM_CAPTURE = {"launch_mnk": (8192, 8192, 16384), "slices": 11, "bytes": 125.42e9 + 11.26e9}

WORKLOADS = {
    "ozaki32768": dict(m=32768, n=32768, k=32768, ta="N", tb="N", alpha=1.0, beta=0.0, kind=2, param=20.0,
                       path="ozaki", tiles=(16384, 16384, 16384), streams=2, policy="autotune",
                       e2e_max_tiles=(32768, 32768, 32768),
                       desc="Ozaki-emulated FP64 GEMM m=n=k=32768 NN, u*2^e, e in [-20,20], k tiles of 16384 "
                            "on the device, autotuned tiles end to end"),
    "ozaki8192": dict(m=8192, n=8192, k=8192, ta="N", tb="N", alpha=1.0, beta=0.0, kind=2, param=20.0,
                      path="ozaki", tiles=(8192, 8192, 8192), streams=2,
                      desc="Ozaki-emulated FP64 GEMM m=n=k=8192 NN, u*2^e, e in [-20,20] (profiling size)"),
    # one engine launch with the headline's k tile and slice count on a sixteenth of its tiles: the
    # size the slice-product kernel is profiled at (a few GB on the device)
    "ozaki8192k16384": dict(m=8192, n=8192, k=16384, ta="N", tb="N", alpha=1.0, beta=0.0, kind=2, param=20.0,
                            path="ozaki", tiles=(8192, 8192, 16384), streams=2,
                            desc="Ozaki-emulated FP64 GEMM m=n=8192, k=16384 NN, u*2^e, e in [-20,20], one k tile "
                                 "(profiling size of the headline's engine launch)"),
    # the out-of-core update m = n = 65536, k = 131072 (NT, alpha = -1, beta = 1) with every dimension
    # halved, so that its host operands fit this host's 199 GB of RAM
    "ooc_ozaki": dict(m=32768, n=32768, k=65536, ta="N", tb="T", alpha=-1.0, beta=1.0, kind=3, param=10.0,
                      path="ozaki", tiles=(65536, 65536, 32768), streams=2, policy="autotune", pageable=True,
                      pin=True, copy_back=False,
                      desc="Out-of-core Ozaki FP64 GEMM m=n=32768, k=65536, NT, alpha=-1, beta=1, N(0,1) x row "
                           "factors 2^U[-10,10], pageable host buffers registered per call, copy_c_back=false, "
                           "autotuned tiles and streams"),
    "sweep": dict(m=20000, n=20000, k=20000, ta="N", tb="N", alpha=1.0, beta=0.0, kind=0, param=0.0,
                  path="sweep", tiles=(5000, 5000, 5000), streams=2,
                  desc="host-pointer FP64 GEMM sweep m=n=k in 4000..20000 step 2000, NN, uniform[-1,1), "
                       "tiles 5000, 2 streams, pinned: the tiled call, the cublasXt-style entry, the vendor "
                       "cublasXt and the Ozaki path"),
    "zgemm8192": dict(m=8192, n=8192, k=8192, ta="N", tb="C", alpha=1.0, beta=0.0, kind=0, param=0.0,
                      path="embedded", dtype="complex128", tiles=(8192, 8192, 8192), streams=2,
                      desc="complex double GEMM m=n=k=8192, op(B) conjugate-transposed, uniform[-1,1) parts, "
                           "device-resident: Ozaki path (real embedding) vs the native complex kernel"),
    "cgemm8192": dict(m=8192, n=8192, k=8192, ta="N", tb="C", alpha=1.0, beta=0.0, kind=0, param=0.0,
                      path="embedded", dtype="complex64", tiles=(8192, 8192, 8192), streams=2,
                      desc="complex float GEMM m=n=k=8192, op(B) conjugate-transposed, uniform[-1,1) parts, "
                           "device-resident: the FP32 tensor-core engine (real embedding) vs the Ozaki path (FP64 "
                           "embedding, 6 slices) and the FFMA kernel"),
    "sgemm16384": dict(m=16384, n=16384, k=16384, ta="N", tb="N", alpha=1.0, beta=0.0, kind=0, param=0.0,
                       path="embedded", dtype="float32", tiles=(16384, 16384, 16384), streams=2,
                       desc="float GEMM m=n=k=16384 NN, uniform[-1,1), device-resident: the FP32 tensor-core "
                            "engine vs the Ozaki path (FP64 embedding, 6 slices) and the FFMA kernel"),
    "batched512": dict(m=4096, n=4096, k=4096, ta="N", tb="N", alpha=1.0, beta=0.0, kind=0, param=0.0,
                       path="batched", tiles=(4096, 4096, 4096), streams=2,
                       desc="512 GEMMs, m,n,k log-uniform [64,4096], half FP64 half FP32, random trans, "
                            "uniform[-1,1), pinned host buffers, one persistent launch in a captured CUDA graph"),
    "batched512_ozaki": dict(m=4096, n=4096, k=4096, ta="N", tb="N", alpha=1.0, beta=0.0, kind=0, param=0.0,
                             path="batched", ozaki=True, tiles=(4096, 4096, 4096), streams=2,
                             desc="512 GEMMs, m,n,k log-uniform [64,4096], half FP64 half FP32, random trans, "
                                  "uniform[-1,1), pinned host buffers, captured CUDA graph; FP64 problems on the Ozaki "
                                  "path at the slice count that meets the native batch's error metric"),
    # the out-of-core update m = n = k = 100000 (TN, ld padded by 64, alpha = 1, beta = 0.5, tiles
    # 8192^3, 3 streams) at a quarter of each dimension (a host-link-to-DMMA ratio the full size
    # shares; a full-size call takes about 30 minutes on the DMMA pipe), with the device memory capped
    # at 6 GiB -- the footprint of 3 streams x 3 tiles of 512 MiB -- so that A and B tiles are evicted
    # and sent again as the C tiles advance
    "ooc_native": dict(m=25000, n=25000, k=25000, ta="T", tb="N", alpha=1.0, beta=0.5, kind=0, param=0.0,
                       path="native", tiles=(8192, 8192, 8192), streams=3, ld_pad=64, mem_limit=6 << 30,
                       desc="Out-of-core native FP64 GEMM m=n=k=25000 TN, ld padded by 64, alpha=1, beta=0.5, "
                            "uniform[-1,1), tiles 8192^3, 3 streams, pinned host buffers, device memory capped at "
                            "6 GiB so that tiles are evicted and streamed"),
    "native4096": dict(m=4096, n=4096, k=4096, ta="N", tb="N", alpha=1.0, beta=1.0, kind=0, param=0.0,
                       path="native", tiles=(2048, 2048, 2048), streams=2,
                       desc="FP64 GEMM m=n=k=4096 NN, uniform[-1,1), alpha=beta=1, tiles 2048, 2 streams"),
}


# ----------------------------------------------------------------------------- helpers
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int = 0):
        self.gpu = gpu
        self.samples: list[list[str]] = []
        self._stop = threading.Event()
        self._t = threading.Thread(target=self._run, daemon=True)

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                for line in out.stdout.strip().splitlines():
                    self.samples.append([x.strip() for x in line.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t.start()
        return self

    def __exit__(self, *exc):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self) -> dict:
        sm = [float(s[1]) for s in self.samples if len(s) > 8 and s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if len(s) > 8 and s[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            if len(s) > 8:
                for nm, v in zip(names, s[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


def dist_setup(n_gpus: int):
    """torchrun ranks (one per GPU) or a single process."""
    if int(os.environ.get("WORLD_SIZE", "1")) > 1:
        import torch
        import torch.distributed as dist

        rank, world, local = int(os.environ["RANK"]), int(os.environ["WORLD_SIZE"]), int(os.environ["LOCAL_RANK"])
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
        return rank, world, local, dist
    return 0, 1, 0, None


def barrier(dist):
    if dist is not None:
        import torch

        dist.barrier()
        torch.cuda.synchronize()


def max_over_ranks(dist, v: float) -> float:
    if dist is None:
        return v
    import torch

    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def measured_peaks() -> dict:
    try:
        return json.loads(PEAKS_FILE.read_text())
    except Exception:
        return {}


# ----------------------------------------------------------------------------- inputs without the library
_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix64(x: np.ndarray) -> np.ndarray:
    """splitmix64 on uint64 arrays (wrapping arithmetic), the generator's hash."""
    with np.errstate(over="ignore"):
        x = x + np.uint64(0x9E3779B97F4A7C15)
        x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return x ^ (x >> np.uint64(31))


def np_generate(kind: int, param: float, seed: int, mat_id: int, rows: int, cols: int, row0: int = 0, col0: int = 0,
                full_rows: int | None = None) -> np.ndarray:
    """The rows x cols block at (row0, col0) of the seeded synthetic matrix (column-major, ld = rows),
    restated in NumPy so that the CPU baselines need nothing of this library: element (i, j) of a
    full_rows-row matrix hashes seed ^ (id << 56) ^ (i + j * full_rows).  Uniform and u * 2^e entries
    are bit-identical to the library's generators; the normal kinds agree to rounding."""
    full_rows = full_rows or rows
    i = np.arange(row0, row0 + rows, dtype=np.uint64)
    j = np.arange(col0, col0 + cols, dtype=np.uint64)
    idx = (i[:, None] + j[None, :] * np.uint64(full_rows)).ravel(order="F")
    key = np.uint64(seed) ^ (np.uint64(mat_id) << np.uint64(56))
    h = _splitmix64(idx ^ key)
    u = (h >> np.uint64(11)).astype(np.float64) * 2.0 ** -52 - 1.0
    if kind == 0:
        return u
    if kind == 2:
        p = int(param)
        he = _splitmix64(idx ^ (np.uint64(seed) ^ (np.uint64(mat_id ^ 0x40) << np.uint64(56))))
        e = (he % np.uint64(2 * p + 1)).astype(np.int64) - p
        return np.ldexp(u, e.astype(np.int32))
    if kind in (3, 4):
        h2 = _splitmix64(idx ^ (np.uint64(seed) ^ (np.uint64(mat_id ^ 0x80) << np.uint64(56))))
        u1 = 1.0 - (h >> np.uint64(11)).astype(np.float64) * 2.0 ** -53
        u2 = (h2 >> np.uint64(11)).astype(np.float64) * 2.0 ** -53
        z = np.sqrt(-2.0 * np.log(u1)) * np.cos(np.pi * 2.0 * u2)
        line = np.broadcast_to(i[:, None] if kind == 3 else j[None, :], (rows, cols))
        hf = _splitmix64(line.ravel(order="F") ^ (np.uint64(seed) ^ (np.uint64(mat_id ^ 0x40) << np.uint64(56))))
        f = (2.0 * (hf >> np.uint64(11)).astype(np.float64) * 2.0 ** -53 - 1.0) * param
        return z * np.exp2(f)
    raise ValueError(f"generator kind {kind} is not restated here")


def host_blas_info() -> str:
    try:
        cfg = np.show_config(mode="dicts")
        blas = cfg.get("Build Dependencies", {}).get("blas", {})
        return f"{blas.get('name', 'unknown')} {blas.get('version', '')}".strip()
    except Exception:
        return "unknown"


def host_blas_baseline(w, seconds_budget: float = 12.0) -> dict:
    """A host dgemm (NumPy's BLAS, all host cores) on a square sub-block of the workload's own
    matrices: the leading min(m, n, k, 8192)^3 product of A and B, timed until the budget."""
    cores = len(os.sched_getaffinity(0))
    d = min(w["m"], w["n"], w["k"], 8192)
    a = np_generate(w["kind"], w["param"], 0, 0, d, d, full_rows=w["m"]).reshape(d, d, order="F")
    b = np_generate(w["kind"], w["param"], 0, 1, d, d, full_rows=w["k"]).reshape(d, d, order="F")
    c = a @ b  # warm-up (BLAS threads start)
    reps, t = 0, 0.0
    t0 = time.perf_counter()
    while t < seconds_budget / 2 or reps < 2:
        np.matmul(a, b, out=c)
        reps += 1
        t = time.perf_counter() - t0
        if reps >= 50:
            break
    return {"value": 2.0 * d ** 3 * reps / t / 1e12, "unit": "TFLOP/s", "cores": cores, "kind": "host_blas",
            "blas": host_blas_info(), "sample": f"dgemm {d}x{d}x{d} (the leading block of the workload's A and B), "
            f"{reps} calls in {t:.1f} s", "seconds": t / reps}


def oracle_sample_setup(w, seconds_target: float):
    """The oracle (the reference algorithm restated on the CPU: tiled GEMM with the reference's
    tile semantics, per-tile plain product) and a k-slab of the workload (full m and n) sized so
    that one sample takes about seconds_target on all host threads.  Inputs come from the NumPy
    restatement of the generator: nothing of this library is loaded."""
    sys.path.insert(0, str(ROOT / "tests"))
    from oracle_lib import load_oracle, oracle_gemm

    oracle = load_oracle()
    cores = len(os.sched_getaffinity(0))
    m, n = w["m"], w["n"]
    c = np.zeros(m * n)

    def make(k):
        a = np_generate(w["kind"], w["param"], 0, 0, m, k, full_rows=m)
        b = np_generate(w["kind"], w["param"], 0, 1, k, n, full_rows=w["k"])
        return a, b

    def sample(a, b, k):
        t0 = time.perf_counter()
        oracle_gemm(oracle, "N", "N", m, n, k, 1.0, a, m, b, k, 0.0, c, m, (min(m, 4096), min(n, 4096), k),
                    nthreads=cores)
        return time.perf_counter() - t0

    k = 8
    a, b = make(k)
    dt = sample(a, b, k)
    k = int(min(w["k"], max(8, k * seconds_target / max(dt, 1e-3))))
    a, b = make(k)
    return (lambda: sample(a, b, k)), m, n, k, cores


def cpu_baseline_port(w, seconds_budget: float = 15.0) -> dict:
    """The oracle port on a k-slab of the workload, all host threads (kind "port")."""
    run, m, n, k, cores = oracle_sample_setup(w, seconds_budget / 2)
    times = [run() for _ in range(2)]
    dt = min(times)
    return {"value": 2.0 * m * n * k / dt / 1e12, "unit": "TFLOP/s", "cores": cores, "kind": "port",
            "sample": f"k-slab m={m} n={n} k={k} of the workload ({dt:.1f} s)", "seconds": dt}


def host_link_bandwidth(torch, nbytes: int = 1 << 30) -> dict:
    """Pinned host <-> device copy bandwidth (GB/s), best of 3, CUDA events: the link term of the
    end-to-end roofline."""
    h = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    d = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    out = {}
    for name, fn in (("h2d_gbs", lambda: d.copy_(h, non_blocking=True)),
                     ("d2h_gbs", lambda: h.copy_(d, non_blocking=True))):
        best = None
        for _ in range(3):
            e0.record()
            fn()
            e1.record()
            e1.synchronize()
            t = e0.elapsed_time(e1) / 1e3
            best = t if best is None else min(best, t)
        out[name] = nbytes / best / 1e9
    del h, d
    return out


# ----------------------------------------------------------------------------- our implementation
def error_metric_dev(tmm, w, a_h, b_h, c_out_h, nsamp=2048) -> float:
    m, n, k = w["m"], w["n"], w["k"]
    return tmm.error_metric(w["ta"], w["tb"], m, n, k, w["alpha"], a_h, m if w["ta"] == "N" else k, b_h,
                            k if w["tb"] == "N" else n, w["beta"], None, m, c_out_h, m, n_samples=nsamp, seed=7)


def calibrate_slices(tmm, torch, w, native_metric_ref: float | None, log) -> tuple[int, dict]:
    """Smallest slice count whose error metric meets the native path's on a sub-problem with the
    workload's k and value distribution (m = n = 2048)."""
    m = n = 2048
    k = w["k"]
    dev = torch.device("cuda")
    a = torch.empty(m * k, dtype=torch.float64, device=dev)
    b = torch.empty(k * n, dtype=torch.float64, device=dev)
    tmm.fill_device(a.data_ptr(), m, k, m, w["kind"], w["param"], seed=101, mat_id=0)
    tmm.fill_device(b.data_ptr(), k, n, k, w["kind"], w["param"], seed=101, mat_id=1)
    a_h, b_h = a.cpu().numpy(), b.cpu().numpy()
    ctx = tmm.make_context(np.float64, 1, 32768, 32768, 32768)
    ctx.set_ozaki_engine(w["engine"])
    c = torch.zeros(m * n, dtype=torch.float64, device=dev)
    tmm.gemm_device(ctx, "N", "N", m, n, k, 1.0, a, m, b, k, 0.0, c, m, stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    sub = dict(w, m=m, n=n)
    e_nat = error_metric_dev(tmm, sub, a_h, b_h, c.cpu().numpy())
    sweep = {}
    chosen = None
    for s in range(6, 21):
        ctx.set_path(tmm.PATH_OZAKI, s)
        tmm.gemm_device(ctx, "N", "N", m, n, k, 1.0, a, m, b, k, 0.0, c, m,
                        stream=torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        e = error_metric_dev(tmm, sub, a_h, b_h, c.cpu().numpy())
        sweep[s] = e
        log(f"calibration: slices={s} metric={e:.3e} (native {e_nat:.3e})")
        if e <= e_nat:
            chosen = s
            break
    ctx.close()
    return (chosen or 20), {"native_metric": e_nat, "sweep": sweep, "m": m, "n": n, "k": k}


def run_ours(args, w, rank, world, dist, log) -> dict:
    import torch

    import tiledmm as tmm

    dev = torch.device("cuda")
    m, n, k = w["m"], w["n"], w["k"]
    a_rows, a_cols = (m, k) if w["ta"] == "N" else (k, m)
    b_rows, b_cols = (k, n) if w["tb"] == "N" else (n, k)
    pad = w.get("ld_pad", 0)  # leading dimensions padded beyond the stored rows
    lda, ldb, ldc = a_rows + pad, b_rows + pad, m + pad
    flops = 2.0 * m * n * k
    stream = torch.cuda.current_stream()
    sid = stream.cuda_stream
    result: dict = {}

    # ---- slice count
    slices = None
    calib = None
    if w["path"] == "ozaki":
        if args.slices:
            slices = args.slices
        else:
            slices, calib = calibrate_slices(tmm, torch, w, None, log)
        log(f"slices = {slices}")

    # ---- device-resident operands
    A = torch.zeros(lda * a_cols, dtype=torch.float64, device=dev)
    B = torch.zeros(ldb * b_cols, dtype=torch.float64, device=dev)
    Cd = torch.zeros(ldc * n, dtype=torch.float64, device=dev)
    # (the row-factor kinds scale the rows of the stored A and of the stored B)
    tmm.fill_device(A.data_ptr(), a_rows, a_cols, lda, w["kind"], w["param"], seed=rank, mat_id=0, stream=sid)
    tmm.fill_device(B.data_ptr(), b_rows, b_cols, ldb, w["kind"], w["param"], seed=rank, mat_id=1, stream=sid)
    tmm.fill_device(Cd.data_ptr(), m, n, ldc, w.get("kind_c", w["kind"]), w["param"], seed=rank, mat_id=2, stream=sid)
    C0 = Cd.clone()
    ctx = tmm.make_context(np.float64, w["streams"], *w["tiles"])
    if slices:
        ctx.set_path(tmm.PATH_OZAKI, slices)
        ctx.set_ozaki_engine(w["engine"])
    eng = ctx.ozaki_engine()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]

    def dev_step():
        tmm.gemm_device(ctx, w["ta"], w["tb"], m, n, k, w["alpha"], A, lda, B, ldb, w["beta"], Cd, ldc, stream=sid)

    for _ in range(args.warmup):
        Cd.copy_(C0)
        dev_step()
    torch.cuda.synchronize()
    launches_per_step = ctx.stats()["kernels"]
    # inputs (8.6 GB per operand at the default workload) are far larger than the 126 MB L2
    times = []
    barrier(dist)
    ctx.set_kernel_timing(True)  # events on the engine's stream around each engine launch
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        for _ in range(args.steps):
            Cd.copy_(C0)  # restore C (also evicts L2); outside the event-timed region
            ev[0].record(stream)
            dev_step()
            ev[1].record(stream)
            ev[1].synchronize()
            times.append(ev[0].elapsed_time(ev[1]) / 1e3)
    kernel_seconds, kernel_launches = ctx.kernel_time()
    ctx.set_kernel_timing(False)
    # a tensor-core wait that gave up (after ~1 s) inside the timed steps would leave C incomplete
    # and the timing meaningless: the line says so
    result["device_status"] = "ok" if ctx.device_status(sid) == 0 else "timeout"
    barrier(dist)
    t_step = max_over_ranks(dist, float(np.mean(times)))
    result["value"] = world * flops / t_step / 1e12
    result["ms_per_step"] = t_step * 1e3
    result["clocks"] = clk.summary()
    result["gpu_launches"] = launches_per_step * args.steps

    # ---- dominant kernel: the engine launches of the timed steps, each bracketed by CUDA events
    result["device_step_seconds"] = t_step
    result["engine_kernel"] = {"launches": kernel_launches, "ms_per_launch": 1e3 * kernel_seconds / max(kernel_launches, 1),
                               "share_of_step": kernel_seconds / (t_step * args.steps)}

    # ---- error metric of this path's result (sampled entries, compensated dot products on the host)
    Cd.copy_(C0)
    dev_step()
    torch.cuda.synchronize()
    a_h, b_h = A.cpu().numpy(), B.cpu().numpy()
    c_out = Cd.cpu().numpy()
    c0_h = C0.cpu().numpy() if w["beta"] != 0 else None
    e_ours = tmm.error_metric(w["ta"], w["tb"], m, n, k, w["alpha"], a_h, lda, b_h, ldb, w["beta"], c0_h, ldc, c_out,
                              ldc, n_samples=args.samples, seed=11)
    result["error_metric"] = e_ours

    # ---- the error at each slice count on the full problem (one untimed-for-the-value call each,
    # event-timed for reference), beside the native path's error below
    if w["path"] == "ozaki" and args.sweep_slices:
        c_pin = torch.empty(ldc * n, dtype=torch.float64).pin_memory()
        sweep = {}
        for s_try in [int(x) for x in args.sweep_slices.split(",")]:
            ctx.set_path(tmm.PATH_OZAKI, s_try)
            Cd.copy_(C0)
            ev[0].record(stream)
            dev_step()
            ev[1].record(stream)
            ev[1].synchronize()
            t_s = ev[0].elapsed_time(ev[1]) / 1e3
            c_pin.copy_(Cd)
            e_s = tmm.error_metric(w["ta"], w["tb"], m, n, k, w["alpha"], a_h, lda, b_h, ldb, w["beta"], c0_h, ldc,
                                   c_pin.numpy(), ldc, n_samples=args.samples, seed=11)
            sweep[s_try] = {"error_metric": e_s, "tflops": flops / t_s / 1e12, "slice_pairs": s_try * (s_try + 1) // 2}
            log(f"full-size sweep: slices={s_try} metric={e_s:.3e} {flops / t_s / 1e12:.1f} TFLOP/s")
        ctx.set_path(tmm.PATH_OZAKI, slices)
        result["slice_sweep_full_size"] = sweep
        del c_pin

    # ---- native path on the same device-resident inputs (for the "vs native" comparison)
    if w["path"] == "ozaki" and not args.skip_native:
        nctx = tmm.make_context(np.float64, 1, *w["tiles"])
        Cd.copy_(C0)
        ev[0].record(stream)
        tmm.gemm_device(nctx, w["ta"], w["tb"], m, n, k, w["alpha"], A, lda, B, ldb, w["beta"], Cd, ldc, stream=sid)
        ev[1].record(stream)
        ev[1].synchronize()
        t_nat = ev[0].elapsed_time(ev[1]) / 1e3
        c_nat = Cd.cpu().numpy()
        e_nat = tmm.error_metric(w["ta"], w["tb"], m, n, k, w["alpha"], a_h, lda, b_h, ldb, w["beta"], c0_h, ldc, c_nat,
                                 ldc, n_samples=args.samples, seed=11)
        result["native"] = {"tflops": flops / t_nat / 1e12, "seconds": t_nat, "error_metric": e_nat,
                            "kernel": "DMMA mma.sync m16n8k4 f64"}
        nctx.close()
    del C0
    torch.cuda.empty_cache()

    # ---- end to end through the public host-pointer call
    pageable = w.get("pageable", False)
    if pageable:  # ordinary (pageable) host memory; registered by the call itself when w["pin"]
        ha, hb, hc = a_h, b_h, c0_h.copy() if c0_h is not None else np.zeros(ldc * n)
        keep = []
    else:
        pa = tmm.PinnedArray((lda * a_cols,))
        pb = tmm.PinnedArray((ldb * b_cols,))
        pc = tmm.PinnedArray((ldc * n,))
        pa.array[:] = a_h
        pb.array[:] = b_h
        ha, hb, hc = pa.array, pb.array, pc.array
        keep = [pa, pb, pc]
        del a_h, b_h
    c_init = hc.copy() if w["beta"] != 0 else None
    del A, B, Cd
    torch.cuda.empty_cache()
    hctx = tmm.make_context(np.float64, w["streams"], *w.get("e2e_max_tiles", w["tiles"]))
    autotune = w.get("policy") == "autotune" and not args.tiles
    if autotune:
        hctx.set_tile_policy(tmm.TILE_POLICY_AUTOTUNE)
    if w.get("mem_limit"):  # a device-memory cap that makes the tiles stream (evicted and sent again)
        hctx.set_memory_limit(w["mem_limit"])
    if slices:
        hctx.set_path(tmm.PATH_OZAKI, slices)
        hctx.set_ozaki_engine(w["engine"])
    copy_back = w.get("copy_back", True)
    e2e_times = []

    def e2e_call():
        tmm.gemm(hctx, w["ta"], w["tb"], m, n, k, w["alpha"], ha, lda, hb, ldb, w["beta"], hc, ldc,
                 pin_host_buffers=w.get("pin", False), copy_c_back=copy_back)

    # warm-up; with the autotuner, until it has timed its candidates (each warm-up call runs one)
    for i in range(max(1, args.e2e_warmup) + (8 if autotune else 0)):
        if c_init is not None:
            hc[:] = c_init
        e2e_call()
        if i + 1 >= max(1, args.e2e_warmup) and (not autotune or hctx.stats()["autotune_state"] >= 2):
            break
    hctx.set_kernel_timing(True)
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as e2e_clk:
        for _ in range(args.e2e_steps):
            if c_init is not None:
                hc[:] = c_init
            t0 = time.perf_counter()
            e2e_call()
            e2e_times.append(time.perf_counter() - t0)
    e2e_kernel_s, _ = hctx.kernel_time()
    e2e_busy_s, e2e_span_s = hctx.kernel_busy_time()
    e2e_error = None
    if copy_back:  # the last call's C, sampled against compensated dot products on the host
        e2e_error = tmm.error_metric(w["ta"], w["tb"], m, n, k, w["alpha"], ha, lda, hb, ldb, w["beta"], c_init, ldc,
                                     hc, ldc, n_samples=min(args.samples, 256), seed=11)
    hctx.set_kernel_timing(False)
    st = hctx.stats()
    t_e2e = max_over_ranks(dist, float(np.mean(e2e_times)))
    result["e2e"] = {"value": world * flops / t_e2e / 1e12, "unit": "TFLOP/s", "h2d_bytes_per_step": st["h2d_bytes"],
                     "d2h_bytes_per_step": st["d2h_bytes"], "seconds_per_step": t_e2e,
                     "host_buffers": ("pageable, registered inside each call" if w.get("pin") else
                                      "pageable, not registered (copy kernels when the GPU reads host memory "
                                      "through the host page tables)")
                     if pageable else "pinned (cudaHostAlloc)",
                     "copy_c_back": copy_back, "steps": args.e2e_steps,
                     "step_seconds": [round(x, 4) for x in e2e_times],
                     # the union of the engine launches' device intervals (launches on the two
                     # compute streams overlap) and their sum, per step
                     "engine_busy_seconds_per_step": e2e_busy_s / max(1, args.e2e_steps),
                     "engine_launch_seconds_sum_per_step": e2e_kernel_s / max(1, args.e2e_steps),
                     "clocks": e2e_clk.summary()}
    if e2e_error is not None:
        result["e2e"]["error_metric"] = e2e_error
    if w.get("mem_limit"):
        result["e2e"]["device_memory_limit_bytes"] = w["mem_limit"]
    result["e2e"]["direct_bytes_per_step"] = st["direct_bytes"]
    result["tiles"] = [st["tile_m"], st["tile_n"], st["tile_k"], st["n_streams"]]
    if autotune:
        result["e2e"]["autotune"] = {"state": st["autotune_state"], "report": hctx.autotune_report()}
    result["e2e_tiles_loaded"] = st["tiles_loaded"]
    hctx.close()
    ctx.close()
    for p in keep:
        p.free()

    if w["path"] == "ozaki":
        pairs = slices * (slices + 1) // 2
        lowp_ops = pairs * flops
        sms = torch.cuda.get_device_properties(0).multi_processor_count
        max_mhz = measured_peaks().get("sm_max_mhz") or 2070.0

        def pipe_peak(clocks: dict) -> tuple[float, float]:
            mhz = (clocks or {}).get("sm_mhz") or max_mhz
            return TCGEN05_E4M3_FLOP_PER_CLK_SM * sms * mhz * 1e6 / 1e12, mhz

        if eng["engine"] == "imma":
            peak, mhz = MEASURED_ENGINE_PEAKS["imma_s8_tops"], None
            src = "mma.sync m16n8k32 s8 issue rate measured on this GPU (engine_rates probe)"
        else:
            peak, mhz = pipe_peak(result["clocks"])
            src = (f"tcgen05.mma kind::f8f6f4 pipe rate, {TCGEN05_E4M3_FLOP_PER_CLK_SM:.0f} FLOP/clk/SM (measured "
                   f"back to back on this GPU) x {sms} SMs x the median SM clock of the timed region ({mhz:.0f} MHz)")
        # algorithmic low-precision operations per launch over the average launch duration
        achieved = lowp_ops * args.steps / kernel_seconds / 1e12
        # the device-resident path launches the engine on all of C per k tile
        launch = (m, n, min(k, w["tiles"][2]))
        traffic = None
        cap = ENGINE_DRAM_CAPTURE
        if eng["engine"] == "tcgen05" and cap["bytes"]:
            def units(mm, nn, kk, s_):
                return -(-mm // 128) * -(-nn // 256) * (s_ * (s_ + 1) // 2) * -(-kk // 128)
            traffic = cap["bytes"] * units(*launch, slices) / units(*cap["launch_mnk"], cap["slices"])
        result["roofline"] = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                              "frac": achieved / peak, "traffic": traffic,
                              "kernel": "oz_gemm_tc" if eng["engine"] == "tcgen05" else "oz_gemm_imma",
                              "launch_mnk": list(launch),
                              "ops": f"{pairs} slice-pair products x 2mnk per step, over the engine launches' "
                                     "event-timed durations",
                              "peak_source": src}
        if traffic:
            algo = slices * (launch[0] + launch[1]) * launch[2] + 8 * launch[0] * launch[1]
            result["roofline"]["traffic_source"] = (
                f"ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch m={cap['launch_mnk'][0]} "
                f"n={cap['launch_mnk'][1]} k={cap['launch_mnk'][2]} at {cap['slices']} slices, scaled by tiles x "
                f"pairs x k-blocks")
            result["roofline"]["algorithmic_bytes_per_launch"] = algo
            result["roofline"]["traffic_over_algorithmic"] = traffic / algo
        if eng["engine"] == "tcgen05":
            bf16 = measured_peaks().get("bf16_tflops") or 1910.1
            result["roofline"]["frac_of_other_ceilings"] = {
                "cublaslt_e4m3_gemm": achieved / MEASURED_ENGINE_PEAKS["cublaslt_e4m3_tflops"],
                "tcgen05_pipe_sustained_at_power_limit":
                    achieved / MEASURED_ENGINE_PEAKS["tcgen05_e4m3_sustained_digits_tflops"],
                "two_x_bf16_burst": achieved / (2.0 * bf16),
                "tcgen05_pipe_at_max_clock": achieved / pipe_peak({"sm_mhz": max_mhz})[0]}
            # spec roofline of the host-pointer call: the slower of the slice products at the
            # pipe rate (at the e2e run's clock) and the host-link traffic at the measured bandwidth
            link = host_link_bandwidth(torch)
            p_e2e, mhz_e2e = pipe_peak(result["e2e"]["clocks"])
            t_compute = lowp_ops / (p_e2e * 1e12)
            t_h2d = result["e2e"]["h2d_bytes_per_step"] / (link["h2d_gbs"] * 1e9)
            t_d2h = result["e2e"]["d2h_bytes_per_step"] / (link["d2h_gbs"] * 1e9)
            t_roof = max(t_compute, t_h2d, t_d2h)
            result["e2e"]["roofline"] = {
                "t_roof_seconds": t_roof, "t_measured_seconds": result["e2e"]["seconds_per_step"],
                "frac": t_roof / result["e2e"]["seconds_per_step"],
                "terms_seconds": {"compute": t_compute, "h2d": t_h2d, "d2h": t_d2h},
                "link_gbs": link, "pipe_tflops_at_clock": p_e2e, "sm_mhz": mhz_e2e}
        result["slices"] = slices
        result["slice_pairs"] = pairs
        result["engine"] = eng
        if calib:
            result["calibration"] = calib
    else:
        peak = MEASURED_ENGINE_PEAKS["dmma_f64_tflops"]
        achieved = flops * args.steps / kernel_seconds / 1e12
        result["roofline"] = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                              "frac": achieved / peak, "traffic": None, "kernel": "gemm_f64_dmma",
                              "peak_source": "mma.sync m16n8k4 f64 issue rate measured on this GPU (engine_rates "
                                             "probe)"}
        # the host-pointer call's bound: the slower of the products at the DMMA issue rate and the
        # host-link traffic it moved (tiles sent again after eviction included) at the measured bandwidth
        link = host_link_bandwidth(torch)
        t_compute = flops / (peak * 1e12)
        t_h2d = result["e2e"]["h2d_bytes_per_step"] / (link["h2d_gbs"] * 1e9)
        t_d2h = result["e2e"]["d2h_bytes_per_step"] / (link["d2h_gbs"] * 1e9)
        t_roof = max(t_compute, t_h2d, t_d2h)
        result["e2e"]["roofline"] = {"t_roof_seconds": t_roof, "t_measured_seconds": result["e2e"]["seconds_per_step"],
                                     "frac": t_roof / result["e2e"]["seconds_per_step"],
                                     "terms_seconds": {"compute": t_compute, "h2d": t_h2d, "d2h": t_d2h},
                                     "link_gbs": link}
    return result


def run_batched(args, rank, world, dist, log, ozaki: bool = False) -> dict:
    """512 GEMMs, m, n, k log-uniform in [64, 4096], half FP64 / half FP32, random trans flags,
    uniform[-1,1) entries, page-locked host buffers: one persistent launch per call, captured
    (with its copies) into a CUDA graph on the first call and replayed; against a loop of the
    plain per-problem path on the same problems.  With ozaki, the FP64 problems run on the Ozaki
    path at the smallest slice count whose error metric (max over the FP64 problems, sampled
    entries) meets the native batch's, and the native batch is timed beside it."""
    import tiledmm as tmm

    rng = np.random.default_rng(1234 + rank)
    count = args.batch_count
    keep, probs = [], []
    flops = 0.0
    for i in range(count):
        dt = np.float64 if i % 2 == 0 else np.float32
        if args.batch_dtypes != "mixed":
            dt = np.float64 if args.batch_dtypes == "f64" else np.float32
        m, n, k = (int(round(np.exp(rng.uniform(np.log(64), np.log(4096))))) for _ in range(3))
        ta, tb = rng.choice(["N", "T"]), rng.choice(["N", "T"])
        ar, ac = (m, k) if ta == "N" else (k, m)
        br, bc = (k, n) if tb == "N" else (n, k)
        arrs = []
        for size in (ar * ac, br * bc, m * n):
            pa = tmm.PinnedArray((size,), dt)
            pa.array[:] = rng.uniform(-1, 1, size).astype(dt)
            keep.append(pa)
            arrs.append(pa.array)
        probs.append(dict(trans_a=ta, trans_b=tb, m=m, n=n, k=k, alpha=1.0, a=arrs[0], ld_a=ar, b=arrs[1], ld_b=br,
                          beta=0.0, c=arrs[2], ld_c=m))
        flops += 2.0 * m * n * k
    f64 = [p for p in probs if p["a"].dtype == np.float64]
    f64_flops = sum(2.0 * p["m"] * p["n"] * p["k"] for p in f64)
    # error metric of the FP64 results: max over the 24 largest FP64 problems, 256 sampled entries each
    err_probs = sorted(f64, key=lambda p: -p["m"] * p["n"] * p["k"])[:24]

    def f64_error():
        if not err_probs:  # an FP32-only batch (--batch-dtypes f32) has no FP64 result to check
            return float("nan")
        return max(tmm.error_metric(p["trans_a"], p["trans_b"], p["m"], p["n"], p["k"], 1.0, p["a"], p["ld_a"],
                                    p["b"], p["ld_b"], 0.0, None, p["m"], p["c"], p["ld_c"], n_samples=256, seed=5)
                   for p in err_probs)

    def timed_batch(ctx):
        times = []
        for it in range(args.warmup + args.steps):
            barrier(dist)
            t0 = time.perf_counter()
            tmm.gemm_batched(ctx, probs)
            t1 = time.perf_counter()
            if it >= args.warmup:
                times.append(t1 - t0)
        return max_over_ranks(dist, float(np.mean(times)))

    ctx = tmm.make_context(np.float64, 2, 4096, 4096, 4096)
    t_native = timed_batch(ctx)
    st_native = ctx.stats()
    e_native = f64_error()
    log(f"batched native: {t_native * 1e3:.1f} ms per call, graph={st_native['batch_graph']}, error {e_native:.3g}")
    out = {}
    t_batch, st = t_native, st_native
    if ozaki:
        octx = tmm.make_context(np.float64, 2, 4096, 4096, 4096)
        octx.set_ozaki_engine(args.engine)
        calib = {}
        slices = args.slices
        if not slices and not err_probs:
            slices = 11
        if not slices:
            for s_try in range(7, 14):
                octx.set_path(tmm.PATH_OZAKI, s_try)
                tmm.gemm_batched(octx, probs)
                calib[s_try] = f64_error()
                if calib[s_try] <= e_native:
                    slices = s_try
                    break
            slices = slices or 13
        octx.set_path(tmm.PATH_OZAKI, slices)
        t_batch = timed_batch(octx)
        st = octx.stats()
        e_oz = f64_error()
        log(f"batched ozaki ({slices} slices): {t_batch * 1e3:.1f} ms per call, error {e_oz:.3g}")
        out["ozaki"] = {"slices": slices, "calibration_error_metric": calib, "error_metric": e_oz,
                        "seconds": t_batch, "engine": args.engine}
        out["native_batch"] = {"tflops": world * flops / t_native / 1e12, "seconds": t_native, "error_metric": e_native,
                               "graph": st_native["batch_graph"]}
    else:
        out["error_metric"] = e_native
    # the plain path, one call per problem (contexts per dtype, default tile policy)
    c64 = tmm.make_context(np.float64, 2, 4096, 4096, 4096)
    c32 = tmm.make_context(np.float32, 2, 4096, 4096, 4096)
    t0 = time.perf_counter()
    for p in probs:
        ctxp = c64 if p["a"].dtype == np.float64 else c32
        tmm.gemm(ctxp, p["trans_a"], p["trans_b"], p["m"], p["n"], p["k"], p["alpha"], p["a"], p["ld_a"], p["b"],
                 p["ld_b"], p["beta"], p["c"], p["ld_c"], pin_host_buffers=False, copy_c_back=True)
    t_loop = max_over_ranks(dist, time.perf_counter() - t0)
    log(f"loop of the plain path: {t_loop * 1e3:.1f} ms")
    for pa in keep:
        pa.free()
    if ozaki:
        pairs = out["ozaki"]["slices"] * (out["ozaki"]["slices"] + 1) // 2
        lowp = pairs * f64_flops / t_batch / 1e12  # e4m3 slice-product rate, whole call (copies, FP32 half included)
        roof = {"bound": "tensor", "achieved": lowp, "peak": MEASURED_ENGINE_PEAKS["tcgen05_e4m3_tflops"],
                "unit": "TFLOP/s", "frac": lowp / MEASURED_ENGINE_PEAKS["tcgen05_e4m3_tflops"], "traffic": None,
                "kernel": "oz_gemm_tc<true> (the FP64 problems of a chunk in one grouped launch, four chunks "
                          "pipelined with their copies); FP32 problems in one grouped f32tc launch beside them",
                "peak_source": "measured tcgen05 e4m3 issue rate on this pool's GB300",
                "fp64_accurate_tflops_of_fp64_half": f64_flops / t_batch / 1e12}
    else:
        roof = {"bound": "tensor", "achieved": f64_flops / t_batch / 1e12,
                "peak": MEASURED_ENGINE_PEAKS["dmma_f64_tflops"], "unit": "TFLOP/s",
                "frac": f64_flops / t_batch / 1e12 / MEASURED_ENGINE_PEAKS["dmma_f64_tflops"],
                "traffic": None, "kernel": "grouped_kernel (FP64 DMMA items dominate)",
                "peak_source": "measured DMMA issue rate on this pool's GB300"}
    res = {"value": world * flops / t_batch / 1e12, "ms_per_step": t_batch * 1e3, "gpu_launches": st["kernels"],
           "e2e": {"value": world * flops / t_batch / 1e12, "unit": "TFLOP/s", "h2d_bytes_per_step": st["h2d_bytes"],
                   "d2h_bytes_per_step": st["d2h_bytes"], "note": "the batched call is host-to-host"},
           "loop_of_plain_path": {"tflops": world * flops / t_loop / 1e12, "seconds": t_loop,
                                  "speedup_of_batched": t_loop / t_batch},
           "batch": {"problems": count, "flops": flops, "fp64_flops": f64_flops, "graph": st["batch_graph"]},
           "roofline": roof}
    res.update(out)
    return res


def _vendor_cublasxt():
    """The vendor's cublasXt (comparison only; the library never links cuBLAS)."""
    import ctypes as C

    for name in ("libcublas.so", "libcublas.so.13", "/usr/local/cuda/lib64/libcublas.so"):
        try:
            return C.CDLL(name)
        except OSError:
            pass
    return None


def run_sweep(args, rank, world, dist, log) -> dict:
    """The reference's compare.sh sweep (examples/compare.sh: m = n = k = 4000..20000, tile 5000,
    2 streams, Tiled-MM's multiply example beside cublasXt-multiply) on this GPU: per size, one
    warm-up call and args.steps timed calls, host wall time, pinned host buffers, FP64."""
    import ctypes as C

    import tiledmm as tmm

    sizes = [int(x) for x in args.sweep_sizes.split(",")]
    reps = max(1, args.steps)
    vendor = _vendor_cublasxt()
    rows = []

    def timed(fn):
        fn()
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        return (time.perf_counter() - t0) / reps

    for size in sizes:
        m = n = k = size
        pa, pb, pc = (tmm.PinnedArray((size * size,)) for _ in range(3))
        tmm.fill_host(pa.array, m, k, m, 0, 0.0, seed=rank, mat_id=0)
        tmm.fill_host(pb.array, k, n, k, 0, 0.0, seed=rank, mat_id=1)
        a, b, c = pa.array, pb.array, pc.array
        flops = 2.0 * m * n * k
        row = {"size": size}
        ctx = tmm.make_context(np.float64, 2, 5000, 5000, 5000)
        row["tiled_tflops"] = flops / timed(lambda: tmm.gemm(ctx, "N", "N", m, n, k, 1.0, a, m, b, k, 0.0, c, m)) / 1e12
        ours = c.copy()
        ctx.close()
        xt = tmm.XtHandle(block_dim=5000)
        row["xt_entry_tflops"] = flops / timed(lambda: xt.gemm(np.float64, 0, 0, m, n, k, 1.0, a, m, b, k, 0.0, c,
                                                               m)) / 1e12
        xt.set_path(tmm.PATH_OZAKI, 11)
        row["xt_entry_ozaki11_tflops"] = flops / timed(lambda: xt.gemm(np.float64, 0, 0, m, n, k, 1.0, a, m, b, k,
                                                                       0.0, c, m)) / 1e12
        xt.close()
        if vendor is not None:
            h = C.c_void_p()
            if vendor.cublasXtCreate(C.byref(h)) == 0:
                devs = (C.c_int * 1)(0)
                vendor.cublasXtDeviceSelect(h, 1, devs)
                vendor.cublasXtSetBlockDim(h, 5000)
                al, be = C.c_double(1.0), C.c_double(0.0)
                sz = C.c_size_t

                def vendor_call():
                    st = vendor.cublasXtDgemm(h, 0, 0, sz(m), sz(n), sz(k), C.byref(al), C.c_void_p(a.ctypes.data),
                                              sz(m), C.c_void_p(b.ctypes.data), sz(k), C.byref(be),
                                              C.c_void_p(c.ctypes.data), sz(m))
                    if st != 0:
                        raise RuntimeError(f"cublasXtDgemm status {st}")

                row["cublasxt_tflops"] = flops / timed(vendor_call) / 1e12
                row["max_rel_diff_vs_cublasxt"] = float(np.abs(ours - c).max() / max(np.abs(c).max(), 1e-300))
                vendor.cublasXtDestroy(h)
        log(json.dumps(row))
        rows.append(row)
        for p in (pa, pb, pc):
            p.free()
    last = rows[-1]
    return {"value": last["tiled_tflops"], "ms_per_step": 2.0 * last["size"] ** 3 / last["tiled_tflops"] / 1e9,
            "sweep": rows, "reps": reps, "warmup": 1,
            "e2e": {"value": last["tiled_tflops"], "unit": "TFLOP/s", "h2d_bytes_per_step": 16 * last["size"] ** 2,
                    "d2h_bytes_per_step": 8 * last["size"] ** 2, "note": "every call is host to host"},
            "vendor_cublasxt": vendor is not None}


def run_embedded(args, w, rank, world, dist, log) -> dict:
    """Float, complex float or complex double on the device: the Ozaki path (real FP64 embedding,
    tcgen05 engine) against the native kernel of the type, TFLOP/s = 2mnk (real) or 8mnk
    (complex) / time, CUDA events.  Componentwise error of both results on 256 sampled rows,
    |C - C*| / (|op(A)| |op(B)|) with C* the FP64 (complex128) product of the same inputs."""
    import torch

    import tiledmm as tmm

    m, n, k = w["m"], w["n"], w["k"]
    npdt = np.dtype(w["dtype"])
    cplx = npdt.kind == "c"
    tdt = {np.float32: torch.float32, np.complex64: torch.complex64, np.complex128: torch.complex128}[npdt.type]
    part = torch.float64 if npdt.type == np.complex128 else torch.float32
    g = torch.Generator(device="cuda").manual_seed(rank)

    def rnd(count):
        x = torch.rand(count, dtype=part, device="cuda", generator=g) * 2 - 1
        if not cplx:
            return x
        return torch.complex(x, torch.rand(count, dtype=part, device="cuda", generator=g) * 2 - 1)

    a, b = rnd(m * k), rnd(k * n)
    slices = args.slices or (11 if npdt.type == np.complex128 else 6)
    flops = (8.0 if cplx else 2.0) * m * n * k
    # op(A) is N (m x k, ld m); op(B) is tb of a stored n x k (ld n) matrix
    ldb = n if w["tb"] != "N" else k
    rows = torch.randperm(m, generator=torch.Generator().manual_seed(7))[:256].cuda()
    wide = torch.complex128 if cplx else torch.float64
    A = a.view(k, m).t()[rows].to(wide)  # sampled rows of op(A)
    Bs = b.view(-1, ldb).t() if w["tb"] == "N" else b.view(-1, ldb)  # op(B) before conjugation: k x n
    if w["tb"] == "C":
        Bs = Bs.conj()
    exact = A @ Bs.to(wide)
    den = A.abs() @ Bs.to(wide).abs()
    out = {}
    names = ("ozaki", "native") if npdt.type == np.complex128 else ("native", "ozaki", "native_simt")
    for name in names:
        # float and complex float: the native path is the FP32 tensor-core engine; the FFMA tile
        # kernel it replaced (TMM_F32_KERNEL=simt) is timed beside it
        if name == "native_simt":
            os.environ["TMM_F32_KERNEL"] = "simt"
        ctx = tmm.make_context(npdt.type, w["streams"], *w["tiles"])
        os.environ.pop("TMM_F32_KERNEL", None)
        if name == "ozaki":
            ctx.set_path(tmm.PATH_OZAKI, slices)
            ctx.set_ozaki_engine(w["engine"])
        c = torch.zeros(m * n, dtype=tdt, device="cuda")
        stream = torch.cuda.current_stream()
        call = lambda: tmm.gemm_device(ctx, w["ta"], w["tb"], m, n, k, 1.0, a, m, b, ldb, 0.0, c, m,
                                       stream=stream.cuda_stream)
        timed_path = "ozaki" if npdt.type == np.complex128 else "native"
        for _ in range(args.warmup if name == timed_path else 1):
            call()
        torch.cuda.synchronize()
        reps = args.steps if name == timed_path else 1
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            call()
        e1.record(stream)
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) / reps / 1e3
        got = c.view(n, m).t()[rows].to(wide)
        err = ((got - exact).abs() / den).max().item()
        out[name] = {"tflops": flops / t / 1e12, "ms": t * 1e3, "max_componentwise_error": err}
        ctx.close()
    out["slices"] = slices
    head = "ozaki" if npdt.type == np.complex128 else "native"
    return {"value": out[head]["tflops"], "ms_per_step": out[head]["ms"], "path_timed": head, "embedded": out,
            "e2e": None, "gpu_launches": None}


def run_reference_arm(args, w, base: dict) -> dict:
    """The reference algorithm's CPU restatement on all host threads: each warm-up and timed step
    is one k-slab sample of the workload (full m and n), sized for about a second and a half, so
    that the whole run ends within a few minutes."""
    run, m, n, k, cores = oracle_sample_setup(w, 1.5)
    for _ in range(args.warmup):
        run()
    times = [run() for _ in range(args.steps)]
    t = float(np.mean(times))
    value = 2.0 * m * n * k / t / 1e12
    sample = f"k-slab m={m} n={n} k={k} of the workload per step"
    return dict(base, impl="reference", value=value, ms_per_step=t * 1e3,
                cpu_baseline={"value": value, "unit": "TFLOP/s", "cores": cores, "kind": "port", "sample": sample},
                e2e={"value": value, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                reference_note="the reference's per-tile arithmetic is cuBLAS on a GPU and its sources are not on "
                               "the GPU machine; its algorithm (tiled GEMM, the reference's tile semantics) is timed "
                               "as the oracle's CPU restatement on the host cores, one k-slab sample per step")


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="ozaki32768", choices=sorted(WORKLOADS))
    ap.add_argument("--slices", type=int, default=0)
    ap.add_argument("--engine", default="tcgen05", choices=["tcgen05", "imma"])
    ap.add_argument("--batch-count", type=int, default=512)
    ap.add_argument("--batch-dtypes", default="mixed", choices=["mixed", "f64", "f32"])
    ap.add_argument("--samples", type=int, default=1024)
    ap.add_argument("--skip-native", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--e2e-warmup", type=int, default=1)
    ap.add_argument("--tiles", default="", help="tile_m,tile_n,tile_k of the context (overrides the workload's)")
    ap.add_argument("--pin", default="workload", choices=["workload", "on", "off"],
                    help="pin_host_buffers of the end-to-end call (default: the workload's)")
    ap.add_argument("--sweep-sizes", default="4000,6000,8000,10000,12000,14000,16000,18000,20000")
    ap.add_argument("--sweep-slices", default="6,7,8,9,10,11",
                    help="slice counts whose error is measured on the full problem (empty: none)")
    args = ap.parse_args()
    w = dict(WORKLOADS[args.workload], engine=args.engine)
    if args.tiles:
        w["tiles"] = tuple(int(x) for x in args.tiles.split(","))
    if args.pin != "workload":
        w["pin"] = args.pin == "on"
    rank, world, local, dist = dist_setup(args.gpus)
    log = (lambda s: print(s, file=sys.stderr, flush=True)) if rank == 0 else (lambda s: None)
    config = {"workload": w["desc"], "m": w["m"], "n": w["n"], "k": w["k"], "trans": w["ta"] + w["tb"],
              "alpha": w["alpha"], "beta": w["beta"], "path": w["path"], "parallelism": f"replicas{world}",
              "l2": "inputs larger than L2 (C restored between steps)"}
    base = {"metric": "FP64-accurate TFLOP/s (Ozaki emulated FP64 vs native DGEMM, same GB300 and error bound)",
            "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded counter-based generator)", "config": config}

    if args.impl == "reference":
        if rank != 0:
            return
        print(json.dumps(run_reference_arm(args, w, base)), flush=True)
        return

    if w["path"] == "embedded":
        res = run_embedded(args, w, rank, world, dist, log)
        if rank == 0:
            line = dict(base)
            kind = {"complex128": "complex FP64", "complex64": "complex FP32", "float32": "FP32"}[w["dtype"]]
            line["metric"] = (f"{kind} TFLOP/s ({'8' if 'complex' in w['dtype'] else '2'}mnk / time) of the default "
                              "path, beside the other paths of the type")
            line["dtype"] = {"complex128": "c128", "complex64": "c64", "float32": "f32"}[w["dtype"]]
            line.update(res)
            print(json.dumps(line), flush=True)
        if dist is not None:
            dist.destroy_process_group()
        return
    if w["path"] == "sweep":
        res = run_sweep(args, rank, world, dist, log)
        if rank == 0:
            line = dict(base)
            line["metric"] = "FP64 TFLOP/s of the host-pointer tiled GEMM at the largest sweep size"
            line.update(res)
            print(json.dumps(line), flush=True)
        if dist is not None:
            dist.destroy_process_group()
        return
    if w["path"] == "batched":
        res = run_batched(args, rank, world, dist, log, ozaki=w.get("ozaki", False))
        if rank == 0:
            line = dict(base)
            line["metric"] = ("FP64-accurate TFLOP/s of 512 uneven FP64/FP32 GEMMs (FP64 problems on the Ozaki path, "
                              "graph replay)" if w.get("ozaki") else
                              "TFLOP/s of 512 uneven FP64/FP32 GEMMs (one persistent launch, graph replay)")
            line["dtype"] = "f64+f32"
            line.update(res)
            print(json.dumps(line), flush=True)
        if dist is not None:
            dist.destroy_process_group()
        return
    res = run_ours(args, w, rank, world, dist, log)
    if rank == 0:
        line = dict(base)
        line.update(res)
        if not args.skip_cpu and world == 1:
            line["cpu_baseline"] = host_blas_baseline(w)
            line["cpu_baseline_port"] = cpu_baseline_port(w)
        peaks = measured_peaks()
        if peaks:
            line["measured_peaks_file"] = {k: peaks.get(k) for k in ("hbm_gbs", "bf16_tflops", "bf16_tflops_sustained")}
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
