"""Host-link copy bandwidth while a tensor-core kernel runs on one GB300: a 4 GiB page-locked
copy host to device, then device to host, on one stream, started 50 ms after a background
launch on another stream (none; one Ozaki engine launch m = n = 32768, k = 16384, 11 slices;
sixty cuBLAS bf16 GEMMs of 16384^3 through torch.matmul).  One JSON line per case, with the
SM clock sampled meanwhile and how long the background outlasted the copies.

    python tiled-mm_gb300/peaks/link_under_engine.py
"""
import sys, json, time
from pathlib import Path
ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "tiled-mm_gb300")); sys.path.insert(0, str(ROOT))
import numpy as np, torch
import tiledmm as tmm, bench
nb = 4 << 30
hsrc = torch.empty(nb // 4, dtype=torch.float32).pin_memory(); hsrc.fill_(1.0)
hdst = torch.empty(nb // 4, dtype=torch.float32).pin_memory()
dbuf = torch.empty(nb // 4, dtype=torch.float32, device="cuda")
cs = torch.cuda.Stream(); ks = torch.cuda.Stream()
ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
def copies():
    with torch.cuda.stream(cs):
        ev[0].record(cs); dbuf.copy_(hsrc, non_blocking=True); ev[1].record(cs)
        hdst.copy_(dbuf, non_blocking=True); ev[2].record(cs)
# backgrounds
m = n = 32768; k = 16384
A = torch.empty(m * k, dtype=torch.float64, device="cuda"); B = torch.empty(k * n, dtype=torch.float64, device="cuda")
C = torch.zeros(m * n, dtype=torch.float64, device="cuda")
tmm.fill_device(A.data_ptr(), m, k, m, 2, 20.0, seed=0, mat_id=0); tmm.fill_device(B.data_ptr(), k, n, k, 2, 20.0, seed=0, mat_id=1)
ctx = tmm.make_context(np.float64, 2, m, n, k); ctx.set_path(tmm.PATH_OZAKI, 11)
xb = torch.randn(16384, 16384, device="cuda", dtype=torch.bfloat16); yb = torch.randn(16384, 16384, device="cuda", dtype=torch.bfloat16)
def bg_ozaki():
    tmm.gemm_device(ctx, "N", "N", m, n, k, 1.0, A, m, B, k, 0.0, C, m, stream=ks.cuda_stream)
def bg_bf16():
    with torch.cuda.stream(ks):
        for _ in range(60): torch.matmul(xb, yb)
def bg_none(): pass
torch.cuda.synchronize()
bg_ozaki(); bg_bf16(); torch.cuda.synchronize()   # warm
for name, fn in (("none", bg_none), ("ozaki_engine", bg_ozaki), ("cublas_bf16_16384", bg_bf16), ("none", bg_none), ("ozaki_engine", bg_ozaki)):
    torch.cuda.synchronize()
    k0 = torch.cuda.Event(enable_timing=True); k1 = torch.cuda.Event(enable_timing=True)
    with bench.ClockSampler(0) as clk:
        k0.record(ks); fn(); k1.record(ks)
        time.sleep(0.05)
        copies()
        torch.cuda.synchronize()
    h2d = ev[0].elapsed_time(ev[1]); d2h = ev[1].elapsed_time(ev[2]); kern = k0.elapsed_time(k1)
    print(json.dumps({"background": name, "h2d_gbs": round(nb / h2d / 1e6, 1), "d2h_gbs": round(nb / d2h / 1e6, 1),
                      "kernel_ms": round(kern, 1), "copy_started_ms_after_kernel": round(k0.elapsed_time(ev[0]), 1),
                      "copy_ended_ms_before_kernel_end": round(ev[2].elapsed_time(k1), 1), "clocks": clk.summary()}), flush=True)
