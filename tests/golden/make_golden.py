"""Generates tests/golden/reference_host_golden.npz from the reference itself.

The reference's own host code (src/Tiled-MM/*.cpp: tile policy, tile
geometry, round-robin schedule, gemm driver) is compiled unmodified against
the host stand-in for the CUDA runtime and cuBLAS (oracle/fake_cuda, recipe in
oracle/Makefile) and run on the known-answer inputs of its own test
(tests/test-multiply.cpp:58-66: std::mt19937(42), integers 0..9, drawn A, B,
C) at the shapes its CI and ctest use.  Needs the reference sources
(the environment variable TMM_REFERENCE_DIR names the checkout; required) and
g++; run from the repo root:

    TMM_REFERENCE_DIR=<reference checkout> python tests/golden/make_golden.py
"""
from __future__ import annotations

import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
from oracle_lib import load_ref_host, ref_gemm  # noqa: E402

# (name, m, n, k, trans, tile_m, tile_n, tile_k, streams, alpha, beta, ld_pad)
CASES = [
    ("ci_small_tiles", 50, 200, 21, "NN", 4, 4, 4, 2, 1.0, 0.0, 0),   # ci/daint-alps.yml:48-56
    ("ci_smaller_than_tile", 5, 2, 2, "NN", 4, 4, 4, 2, 1.0, 0.0, 0),  # ci/daint-alps.yml:58-64
    ("beta_one", 37, 23, 19, "NN", 8, 8, 8, 3, 1.0, 1.0, 0),
    ("beta_alpha", 33, 41, 24, "NN", 16, 8, 8, 2, -2.0, 0.5, 3),
    ("tn", 30, 20, 24, "TN", 8, 8, 8, 2, 1.0, 1.0, 0),
    ("nt", 30, 20, 21, "NT", 8, 8, 8, 2, 1.0, 1.0, 2),
    ("tt", 17, 26, 32, "TT", 8, 8, 8, 2, 1.0, 0.0, 0),
    ("default_tiles", 120, 90, 70, "NN", 5000, 5000, 5000, 2, 1.0, 1.0, 0),
    # transposed A with a short k tile: the reference computes the tile's k extent at the
    # m tile index (src/Tiled-MM/tiled_mm.cpp:148-165), so its result differs from the product
    ("tn_short_k_tile", 50, 12, 23, "TN", 4, 4, 4, 2, 1.0, 0.0, 0),
]


def kat_inputs(na: int, nb: int, nc: int) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    with tempfile.TemporaryDirectory() as d:
        exe = Path(d) / "kat_inputs"
        subprocess.run(["g++", "-O1", "-o", str(exe), str(HERE / "kat_inputs.cpp")], check=True)
        raw = subprocess.run([str(exe), str(na), str(nb), str(nc)], check=True, capture_output=True).stdout
    v = np.frombuffer(raw, dtype=np.uint8)
    return v[:na], v[na:na + nb], v[na + nb:]


def main() -> None:
    ref = load_ref_host()
    if ref is None:
        raise SystemExit("reference sources not found: set TMM_REFERENCE_DIR to the reference checkout")
    out: dict[str, np.ndarray] = {}
    for (name, m, n, k, tr, tm, tn, tk, streams, alpha, beta, pad) in CASES:
        ta, tb = tr[0], tr[1]
        a_rows, a_cols = (m, k) if ta == "N" else (k, m)
        b_rows, b_cols = (k, n) if tb == "N" else (n, k)
        lda, ldb, ldc = a_rows + pad, b_rows + pad, m + pad
        a8, b8, c8 = kat_inputs(lda * a_cols, ldb * b_cols, ldc * n)
        a, b, c = a8.astype(np.float64), b8.astype(np.float64), c8.astype(np.float64)
        c_back = c.copy()
        _, _, tiles = ref_gemm(ref, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c_back, ldc, streams,
                               (tm, tn, tk), copy_c_back=True)
        c_dev = c.copy()
        _, full, _ = ref_gemm(ref, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c_dev, ldc, streams,
                              (tm, tn, tk), copy_c_back=False)
        out[f"{name}/params"] = np.array([m, n, k, ord(ta), ord(tb), tm, tn, tk, streams, lda, ldb, ldc] + list(tiles),
                                         dtype=np.int64)
        out[f"{name}/scalars"] = np.array([alpha, beta])
        out[f"{name}/a"], out[f"{name}/b"], out[f"{name}/c"] = a8, b8, c8
        out[f"{name}/c_copy_back"] = c_back
        out[f"{name}/full_c"] = full
    # tile policy table (src/Tiled-MM/mm_handle.cpp:89-110)
    rows = []
    for dim in [1, 2, 3, 4, 5, 7, 12, 100, 997, 1000, 1024, 1357, 4096, 4567, 5000, 10000, 12345, 23456, 32768,
                65536, 67891, 100000, 131072]:
        for cur in [0, 2048, 5000, 8192]:
            for mx in [4, 1000, 2048, 5000, 8192]:
                rows.append((dim, cur, mx, ref.ref_optimal_tile_size(dim, cur, mx)))
    out["tile_policy"] = np.array(rows, dtype=np.int64)
    # tile geometry (src/Tiled-MM/tiled_matrix.cpp:8-80)
    geo = []
    info = np.zeros(5, dtype=np.int64)
    for rows_, cols_, ld, tr_, tc_ in [(50, 21, 50, 4, 4), (21, 200, 23, 4, 4), (5, 2, 5, 4, 4), (1000, 1000, 1000, 300, 700),
                                       (1234, 1357, 1300, 5000, 5000), (4096, 4096, 4096, 2048, 2048)]:
        for ci in range(0, (rows_ + min(tr_, rows_) - 1) // min(tr_, rows_)):
            for cj in range(0, (cols_ + min(tc_, cols_) - 1) // min(tc_, cols_)):
                ref.ref_tiled_matrix_info(rows_, cols_, ld, tr_, tc_, ci, cj, info.ctypes.data)
                geo.append((rows_, cols_, ld, tr_, tc_, ci, cj, *info.tolist()))
    out["tile_geometry"] = np.array(geo, dtype=np.int64)
    np.savez_compressed(HERE / "reference_host_golden.npz", **out)
    print(f"wrote {HERE / 'reference_host_golden.npz'} ({len(CASES)} gemm cases, {len(rows)} policy rows, {len(geo)} tiles)")


if __name__ == "__main__":
    main()
