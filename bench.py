"""Benchmark of the out-of-core tiled GEMM on GB300 (one JSON line on rank 0).

Metric: FP64-accurate TFLOP/s (2 m n k / time) of the Ozaki emulated-FP64 path,
reported beside the native FP64 (DMMA) path on the same inputs, with the
componentwise error metric of both against a twice-working-precision oracle.

Default workload (--workload ozaki32768): m = n = k = 32768, NN, entries u * 2^e
with u uniform [-1, 1) and e a uniform integer in [-20, 20] (seeded, synthetic),
alpha = 1, beta = 0, the slice count the smallest that meets the native path's
error on a calibration sub-problem of the same k and distribution.
  value    device-resident operands (tmm_gemm_device), CUDA-event timed
  e2e      the public host-pointer call (tmm_gemm) with pinned host buffers:
           every step copies A and B to the device and C back
Other workloads: native4096 (m = n = k = 4096 NN, uniform, alpha = beta = 1,
tiles 2048, 2 streams, pinned, copy_c_back).

--impl reference times the reference algorithm's CPU restatement (the oracle;
the reference itself is cuBLAS-backed GPU code that is not present on the GPU
box) on the host cores, on a bounded k-slab of the same workload.
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
# measured on this machine's GB300 with the repository's own probes (mma.sync loops, CUDA events)
# Instruction-rate ceilings on this machine's GB300, measured by tiled-mm_gb300/peaks/engine_rates.cu
# (dmma, imma; tcgen05 e4m3 M128 N256 K32 back to back from shared memory) and the vendor library's
# dense e4m3 GEMM (tiled-mm_gb300/peaks/cublaslt_e4m3.py, 8192^3); summarised in
# profiles/engine_rates.md.
MEASURED_ENGINE_PEAKS = {"imma_s8_tops": 157.9, "dmma_f64_tflops": 1.099,
                         "tcgen05_e4m3_tflops": 4847.2, "cublaslt_e4m3_tflops": 3948.0}
# DRAM bytes (read + write) per launch of the slice-product kernel on the device-resident path,
# from one ncu capture of the workload's own command (profiles/oz_gemm_tc_ozaki32768.md):
# (workload, launch m, n, k tile, slices) -> bytes
MEASURED_TRAFFIC = {("ozaki32768", (32768, 32768, 16384), 11): 2.605e12}

WORKLOADS = {
    "ozaki32768": dict(m=32768, n=32768, k=32768, ta="N", tb="N", alpha=1.0, beta=0.0, kind=2, param=20.0,
                       path="ozaki", tiles=(16384, 16384, 16384), streams=2,
                       desc="Ozaki-emulated FP64 GEMM m=n=k=32768 NN, u*2^e, e in [-20,20], tiles 16384^3"),
    "ozaki8192": dict(m=8192, n=8192, k=8192, ta="N", tb="N", alpha=1.0, beta=0.0, kind=2, param=20.0,
                      path="ozaki", tiles=(8192, 8192, 8192), streams=2,
                      desc="Ozaki-emulated FP64 GEMM m=n=k=8192 NN, u*2^e, e in [-20,20] (profiling size)"),
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
                           "device-resident: Ozaki path (real FP64 embedding, 6 slices) vs the native kernel"),
    "sgemm16384": dict(m=16384, n=16384, k=16384, ta="N", tb="N", alpha=1.0, beta=0.0, kind=0, param=0.0,
                       path="embedded", dtype="float32", tiles=(16384, 16384, 16384), streams=2,
                       desc="float GEMM m=n=k=16384 NN, uniform[-1,1), device-resident: Ozaki path (FP64 "
                            "embedding, 6 slices) vs the native FP32 kernel"),
    "batched512": dict(m=4096, n=4096, k=4096, ta="N", tb="N", alpha=1.0, beta=0.0, kind=0, param=0.0,
                       path="batched", tiles=(4096, 4096, 4096), streams=2,
                       desc="512 GEMMs, m,n,k log-uniform [64,4096], half FP64 half FP32, random trans, "
                            "uniform[-1,1), pinned host buffers, one persistent launch in a captured CUDA graph"),
    "batched512_ozaki": dict(m=4096, n=4096, k=4096, ta="N", tb="N", alpha=1.0, beta=0.0, kind=0, param=0.0,
                             path="batched", ozaki=True, tiles=(4096, 4096, 4096), streams=2,
                             desc="512 GEMMs, m,n,k log-uniform [64,4096], half FP64 half FP32, random trans, "
                                  "uniform[-1,1), pinned host buffers, captured CUDA graph; FP64 problems on the Ozaki "
                                  "path at the slice count that meets the native batch's error metric"),
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
    lda = m if w["ta"] == "N" else k
    ldb = k if w["tb"] == "N" else n
    a_rows, a_cols = (m, k) if w["ta"] == "N" else (k, m)
    b_rows, b_cols = (k, n) if w["tb"] == "N" else (n, k)
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
    A = torch.empty(a_rows * a_cols, dtype=torch.float64, device=dev)
    B = torch.empty(b_rows * b_cols, dtype=torch.float64, device=dev)
    Cd = torch.empty(m * n, dtype=torch.float64, device=dev)
    # (the row-factor kinds scale the rows of the stored A and of the stored B)
    tmm.fill_device(A.data_ptr(), a_rows, a_cols, a_rows, w["kind"], w["param"], seed=rank, mat_id=0, stream=sid)
    tmm.fill_device(B.data_ptr(), b_rows, b_cols, b_rows, w["kind"], w["param"], seed=rank, mat_id=1, stream=sid)
    tmm.fill_device(Cd.data_ptr(), m, n, m, w.get("kind_c", w["kind"]), w["param"], seed=rank, mat_id=2, stream=sid)
    C0 = Cd.clone()
    ctx = tmm.make_context(np.float64, w["streams"], *w["tiles"])
    if slices:
        ctx.set_path(tmm.PATH_OZAKI, slices)
        ctx.set_ozaki_engine(w["engine"])
    eng = ctx.ozaki_engine()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]

    def dev_step():
        tmm.gemm_device(ctx, w["ta"], w["tb"], m, n, k, w["alpha"], A, lda, B, ldb, w["beta"], Cd, m, stream=sid)

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
    e_ours = tmm.error_metric(w["ta"], w["tb"], m, n, k, w["alpha"], a_h, lda, b_h, ldb, w["beta"], c0_h, m, c_out, m,
                              n_samples=args.samples, seed=11)
    result["error_metric"] = e_ours

    # ---- native path on the same device-resident inputs (for the "vs native" comparison)
    if w["path"] == "ozaki" and not args.skip_native:
        nctx = tmm.make_context(np.float64, 1, *w["tiles"])
        Cd.copy_(C0)
        ev[0].record(stream)
        tmm.gemm_device(nctx, w["ta"], w["tb"], m, n, k, w["alpha"], A, lda, B, ldb, w["beta"], Cd, m, stream=sid)
        ev[1].record(stream)
        ev[1].synchronize()
        t_nat = ev[0].elapsed_time(ev[1]) / 1e3
        c_nat = Cd.cpu().numpy()
        e_nat = tmm.error_metric(w["ta"], w["tb"], m, n, k, w["alpha"], a_h, lda, b_h, ldb, w["beta"], c0_h, m, c_nat,
                                 m, n_samples=args.samples, seed=11)
        result["native"] = {"tflops": flops / t_nat / 1e12, "seconds": t_nat, "error_metric": e_nat,
                            "kernel": "DMMA mma.sync m16n8k4 f64"}
        nctx.close()
    del C0
    torch.cuda.empty_cache()

    # ---- end to end through the public host-pointer call
    pageable = w.get("pageable", False)
    if pageable:  # ordinary (pageable) host memory; registered by the call itself when w["pin"]
        ha, hb, hc = a_h, b_h, c0_h.copy() if c0_h is not None else np.zeros(m * n)
        keep = []
    else:
        pa = tmm.PinnedArray((a_rows * a_cols,))
        pb = tmm.PinnedArray((b_rows * b_cols,))
        pc = tmm.PinnedArray((m * n,))
        pa.array[:] = a_h
        pb.array[:] = b_h
        ha, hb, hc = pa.array, pb.array, pc.array
        keep = [pa, pb, pc]
        del a_h, b_h
    c_init = hc.copy() if w["beta"] != 0 else None
    del A, B, Cd
    torch.cuda.empty_cache()
    hctx = tmm.make_context(np.float64, w["streams"], *w["tiles"])
    if w.get("policy") == "autotune":
        hctx.set_tile_policy(tmm.TILE_POLICY_AUTOTUNE)
    if slices:
        hctx.set_path(tmm.PATH_OZAKI, slices)
        hctx.set_ozaki_engine(w["engine"])
    copy_back = w.get("copy_back", True)
    e2e_times = []

    def e2e_call():
        tmm.gemm(hctx, w["ta"], w["tb"], m, n, k, w["alpha"], ha, lda, hb, ldb, w["beta"], hc, m,
                 pin_host_buffers=w.get("pin", False), copy_c_back=copy_back)

    for _ in range(max(1, args.e2e_warmup)):
        if c_init is not None:
            hc[:] = c_init
        e2e_call()
    hctx.set_kernel_timing(True)
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as e2e_clk:
        for _ in range(args.e2e_steps):
            if c_init is not None:
                hc[:] = c_init
            t0 = time.perf_counter()
            e2e_call()
            e2e_times.append(time.perf_counter() - t0)
    e2e_kernel_s, _ = hctx.kernel_time()
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
                     "engine_kernel_seconds_per_step": e2e_kernel_s / max(1, args.e2e_steps),
                     "clocks": e2e_clk.summary()}
    result["e2e"]["direct_bytes_per_step"] = st["direct_bytes"]
    result["tiles"] = [st["tile_m"], st["tile_n"], st["tile_k"], st["n_streams"]]
    result["e2e_tiles_loaded"] = st["tiles_loaded"]
    hctx.close()
    ctx.close()
    for p in keep:
        p.free()

    if w["path"] == "ozaki":
        pairs = slices * (slices + 1) // 2
        lowp_ops = pairs * flops
        if eng["engine"] == "imma":
            peak = MEASURED_ENGINE_PEAKS["imma_s8_tops"]
            src = "mma.sync m16n8k32 s8 issue rate, tiled-mm_gb300/peaks/engine_rates.cu"
        else:
            bf16 = measured_peaks().get("bf16_tflops") or 1910.1
            peak = 2.0 * bf16
            src = "2 x the measured dense bf16 cuBLAS burst rate in MEASURED_PEAKS.json (e4m3 issues at twice bf16)"
        # algorithmic low-precision operations per launch over the average launch duration
        achieved = lowp_ops * args.steps / kernel_seconds / 1e12
        # the device-resident path launches the engine on all of C per k tile
        launch = (m, n, min(k, w["tiles"][2]))
        traffic = MEASURED_TRAFFIC.get((args.workload, launch, slices))
        result["roofline"] = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                              "frac": achieved / peak, "traffic": traffic,
                              "kernel": "oz_gemm_tc" if eng["engine"] == "tcgen05" else "oz_gemm_imma",
                              "launch_mnk": list(launch),
                              "ops": f"{pairs} slice-pair products x 2mnk per step, over the engine launches' "
                                     "event-timed durations",
                              "peak_source": src}
        if eng["engine"] == "tcgen05":
            result["roofline"]["frac_of_other_ceilings"] = {
                "cublaslt_e4m3_gemm": achieved / MEASURED_ENGINE_PEAKS["cublaslt_e4m3_tflops"],
                "tcgen05_pipe_back_to_back": achieved / MEASURED_ENGINE_PEAKS["tcgen05_e4m3_tflops"]}
        if traffic:
            result["roofline"]["traffic_source"] = "ncu dram__bytes_read.sum + dram__bytes_write.sum per launch, " \
                                                   "profiles/oz_gemm_tc_ozaki32768.md"
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
                              "peak_source": "mma.sync m16n8k4 f64 issue rate, tiled-mm_gb300/peaks/engine_rates.cu"}
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
                "kernel": "oz_gemm_tc (FP64 problems: one launch per problem and k tile, a branch stream per problem)",
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
    for name in ("ozaki", "native"):
        ctx = tmm.make_context(npdt.type, w["streams"], *w["tiles"])
        if name == "ozaki":
            ctx.set_path(tmm.PATH_OZAKI, slices)
            ctx.set_ozaki_engine(w["engine"])
        c = torch.zeros(m * n, dtype=tdt, device="cuda")
        stream = torch.cuda.current_stream()
        call = lambda: tmm.gemm_device(ctx, w["ta"], w["tb"], m, n, k, 1.0, a, m, b, ldb, 0.0, c, m,
                                       stream=stream.cuda_stream)
        for _ in range(args.warmup if name == "ozaki" else 1):
            call()
        torch.cuda.synchronize()
        reps = args.steps if name == "ozaki" else 1
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
    return {"value": out["ozaki"]["tflops"], "ms_per_step": out["ozaki"]["ms"], "embedded": out,
            "e2e": None, "gpu_launches": None}


def cpu_baseline(w, seconds_budget: float = 20.0) -> dict:
    """The reference algorithm's CPU restatement (the oracle: tiled GEMM with the reference's tile
    semantics, per-tile plain GEMM) on a k-slab of the workload, all host threads."""
    sys.path.insert(0, str(ROOT / "tests"))
    from oracle_lib import load_oracle, oracle_gemm

    import tiledmm as tmm

    oracle = load_oracle()
    cores = len(os.sched_getaffinity(0))
    m, n = w["m"], w["n"]
    k = 64
    while True:
        a = np.zeros(m * k)
        b = np.zeros(k * n)
        tmm.fill_host(a, m, k, m, w["kind"], w["param"], seed=0, mat_id=0)
        tmm.fill_host(b, k, n, k, w["kind"], w["param"], seed=0, mat_id=1)
        c = np.zeros(m * n)
        t0 = time.perf_counter()
        oracle_gemm(oracle, "N", "N", m, n, k, 1.0, a, m, b, k, 0.0, c, m, (min(m, 4096), min(n, 4096), k),
                    nthreads=cores)
        dt = time.perf_counter() - t0
        if dt * 4 > seconds_budget or k >= w["k"]:
            break
        k = min(w["k"], k * 4)
    return {"value": 2.0 * m * n * k / dt / 1e12, "unit": "TFLOP/s", "cores": cores, "kind": "port",
            "sample": f"k-slab m={m} n={n} k={k} of the workload ({dt:.1f} s)", "seconds": dt}


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
        cb = cpu_baseline(w)
        line = dict(base, impl="reference", value=cb["value"], ms_per_step=cb["seconds"] * 1e3,
                    cpu_baseline=cb, e2e={"value": cb["value"], "unit": "TFLOP/s", "h2d_bytes_per_step": 0,
                                          "d2h_bytes_per_step": 0})
        line["config"] = dict(config, reference_note="the reference's per-tile arithmetic is cuBLAS on a GPU; "
                              "its algorithm is timed here as the oracle's CPU restatement on the host cores")
        print(json.dumps(line), flush=True)
        return

    if w["path"] == "embedded":
        res = run_embedded(args, w, rank, world, dist, log)
        if rank == 0:
            line = dict(base)
            kind = {"complex128": "complex FP64", "complex64": "complex FP32", "float32": "FP32"}[w["dtype"]]
            line["metric"] = (f"{kind} TFLOP/s ({'8' if 'complex' in w['dtype'] else '2'}mnk / time), Ozaki path vs "
                              "the native kernel of the type")
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
        if not args.skip_cpu:
            line["cpu_baseline"] = cpu_baseline(w)
        peaks = measured_peaks()
        if peaks:
            line["measured_peaks_file"] = {k: peaks.get(k) for k in ("hbm_gbs", "bf16_tflops", "bf16_tflops_sustained")}
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
