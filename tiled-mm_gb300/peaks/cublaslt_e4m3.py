"""Dense e4m3 GEMM rate of the vendor library (cuBLASLt through torch._scaled_mm, fp32 or bf16 out),
the practical ceiling for an e4m3 tensor-core kernel on this GPU.

    python tiled-mm_gb300/peaks/cublaslt_e4m3.py      # one JSON line
"""
import json

import torch


def rate(m, n, k, out_dtype, reps=20):
    a = torch.randn(m, k, device="cuda").to(torch.float8_e4m3fn)
    b = torch.randn(n, k, device="cuda").to(torch.float8_e4m3fn)
    one = torch.tensor(1.0, device="cuda")
    f = lambda: torch._scaled_mm(a, b.t(), scale_a=one, scale_b=one, out_dtype=out_dtype)
    for _ in range(5):
        f()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        f()
    e1.record()
    torch.cuda.synchronize()
    return 2.0 * m * n * k / (e0.elapsed_time(e1) / reps / 1e3) / 1e12


if __name__ == "__main__":
    res = {}
    for size in (8192, 16384):
        for od in (torch.bfloat16, torch.float32):
            res[f"{size}^3 {str(od).split('.')[-1]} out"] = round(rate(size, size, size, od), 1)
    print(json.dumps({"probe": "cublaslt_e4m3_gemm_tflops", **res}))
