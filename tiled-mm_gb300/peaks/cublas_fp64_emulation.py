"""The vendor's FP64 GEMM on the benchmark's inputs, native and with cuBLAS's fixed-point FP64
emulation (CUBLAS_FP64_EMULATED_FIXEDPOINT_MATH, emulation strategy "eager" so that it is used
whenever possible, mantissa bits chosen by cuBLAS): rate and the bench's componentwise error
metric, beside the library's Ozaki path.  Comparison only; the library never links cuBLAS.

    python tiled-mm_gb300/peaks/cublas_fp64_emulation.py [--size 32768] [--reps 3]
"""
import argparse
import ctypes as C
import json
import sys
from pathlib import Path

import numpy as np
import torch

sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
import tiledmm as tmm  # noqa: E402

MATH_DEFAULT, MATH_FP64_EMULATED_FIXEDPOINT = 0, 8
STRATEGY_EAGER = 2


def load_cublas():
    for name in ("libcublas.so", "libcublas.so.13", "/usr/local/cuda/lib64/libcublas.so"):
        try:
            return C.CDLL(name)
        except OSError:
            pass
    raise RuntimeError("libcublas not found")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", type=int, default=32768)
    ap.add_argument("--reps", type=int, default=1)
    ap.add_argument("--samples", type=int, default=1024)
    args = ap.parse_args()
    n = args.size
    lib = load_cublas()
    h = C.c_void_p()
    assert lib.cublasCreate_v2(C.byref(h)) == 0
    # the bench's default workload: u * 2^e, e in [-20, 20], seed 0, matrix ids 0 and 1, NN, alpha 1, beta 0
    A = torch.empty(n * n, dtype=torch.float64, device="cuda")
    B = torch.empty(n * n, dtype=torch.float64, device="cuda")
    Cd = torch.zeros(n * n, dtype=torch.float64, device="cuda")
    tmm.fill_device(A.data_ptr(), n, n, n, tmm.GEN_UEXP, 20.0, seed=0, mat_id=0)
    tmm.fill_device(B.data_ptr(), n, n, n, tmm.GEN_UEXP, 20.0, seed=0, mat_id=1)
    torch.cuda.synchronize()
    a_h, b_h = A.cpu().numpy(), B.cpu().numpy()
    al, be = C.c_double(1.0), C.c_double(0.0)

    def dgemm():
        st = lib.cublasDgemm_v2(h, 0, 0, n, n, n, C.byref(al), C.c_void_p(A.data_ptr()), n, C.c_void_p(B.data_ptr()),
                                n, C.byref(be), C.c_void_p(Cd.data_ptr()), n)
        if st != 0:
            raise RuntimeError(f"cublasDgemm status {st}")

    out = {"probe": "cublas_dgemm_fp64_emulation", "m": n, "n": n, "k": n, "inputs": "u*2^e, e in [-20,20]"}
    for name, mode in (("native", MATH_DEFAULT), ("fixedpoint_emulation_eager", MATH_FP64_EMULATED_FIXEDPOINT)):
        row = {"set_math_mode": lib.cublasSetMathMode(h, mode)}
        if mode == MATH_FP64_EMULATED_FIXEDPOINT:
            row["set_strategy"] = lib.cublasSetEmulationStrategy(h, STRATEGY_EAGER)
        dgemm()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.reps):
            dgemm()
        e1.record()
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) / args.reps / 1e3
        row["tflops"] = 2.0 * n ** 3 / t / 1e12
        row["error_metric"] = tmm.error_metric("N", "N", n, n, n, 1.0, a_h, n, b_h, n, 0.0, None, n, Cd.cpu().numpy(),
                                               n, n_samples=args.samples, seed=11)
        bits = C.c_int(-1)
        if lib.cublasGetFixedPointEmulationMaxMantissaBitCount(h, C.byref(bits)) == 0:
            row["max_mantissa_bits"] = bits.value
        out[name] = row
    lib.cublasDestroy_v2(h)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
