"""Drives host-pointer GEMM calls under the CUPTI timeline probe (overlap_trace.cpp) with a
marker around each timed call, for overlap_summary.py.

    CUDA_INJECTION64_PATH=tiled-mm_gb300/peaks/_build/liboverlap_trace.so \
    OVERLAP_TRACE_OUT=gpurun_out/trace_native4096.csv \
    python tiled-mm_gb300/peaks/overlap_run.py --workload native4096 --calls 3

Workloads are bench.py's (inputs from the same seeded generator, pinned host buffers, the
workload's tiles, streams and path; the Ozaki workloads at 11 slices)."""
from __future__ import annotations

import argparse
import ctypes
import os
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "tiled-mm_gb300"))
sys.path.insert(0, str(ROOT))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="native4096")
    ap.add_argument("--calls", type=int, default=3)
    ap.add_argument("--tiles", default="", help="tile_m,tile_n,tile_k (default: the workload's)")
    args = ap.parse_args()
    import tiledmm as tmm
    from bench import WORKLOADS

    probe = ctypes.CDLL(os.environ["CUDA_INJECTION64_PATH"])
    probe.overlap_trace_mark.argtypes = [ctypes.c_char_p]
    w = WORKLOADS[args.workload]
    m, n, k = w["m"], w["n"], w["k"]
    tiles = tuple(int(x) for x in args.tiles.split(",")) if args.tiles else w["tiles"]
    a_rows, a_cols = (m, k) if w["ta"] == "N" else (k, m)
    b_rows, b_cols = (k, n) if w["tb"] == "N" else (n, k)
    pa, pb, pc = tmm.PinnedArray((a_rows * a_cols,)), tmm.PinnedArray((b_rows * b_cols,)), tmm.PinnedArray((m * n,))
    tmm.fill_host(pa.array, a_rows, a_cols, a_rows, w["kind"], w["param"], seed=0, mat_id=0)
    tmm.fill_host(pb.array, b_rows, b_cols, b_rows, w["kind"], w["param"], seed=0, mat_id=1)
    tmm.fill_host(pc.array, m, n, m, 0, 0.0, seed=0, mat_id=2)
    ctx = tmm.make_context(np.float64, w["streams"], *tiles)
    if w["path"] == "ozaki":
        ctx.set_path(tmm.PATH_OZAKI, 11)
    call = lambda: tmm.gemm(ctx, w["ta"], w["tb"], m, n, k, w["alpha"], pa.array, a_rows, pb.array, b_rows, w["beta"],
                            pc.array, m, pin_host_buffers=True, copy_c_back=w.get("copy_back", True))
    call()  # warm-up: buffers sized, kernels loaded
    for i in range(args.calls):
        probe.overlap_trace_mark(f"begin {i}".encode())
        call()
        probe.overlap_trace_mark(f"end {i}".encode())
    st = ctx.stats()
    print(f"{args.workload}: tiles {st['tile_m']}x{st['tile_n']}x{st['tile_k']}, {st['n_streams']} streams, "
          f"last call {st['seconds']:.3f} s, H2D {st['h2d_bytes']} B, D2H {st['d2h_bytes']} B")
    ctx.close()
    for p in (pa, pb, pc):
        p.free()


if __name__ == "__main__":
    main()
