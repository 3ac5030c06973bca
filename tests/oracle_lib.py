"""ctypes bindings of the oracle (oracle/tmm_oracle.c, oracle/tmm_ozaki_oracle.c) and of the
reference's own host code built against the CUDA stand-in (oracle/_ref).  Test infrastructure:
only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this module."""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
ORACLE = ROOT / "oracle"
ORACLE_SO = ORACLE / "_build" / "libtmm_oracle.so"
REF_SO = ORACLE / "_ref" / "libtiledmm_ref_host.so"
# the reference checkout, where one exists (set by the build step that compiles oracle/_ref)
_REF_ENV = os.environ.get("TMM_REFERENCE_DIR", "")
REFERENCE_DIR = Path(_REF_ENV) if _REF_ENV else None

_p, _i64, _ci, _d = C.c_void_p, C.c_int64, C.c_int, C.c_double
DT = {np.dtype(np.float32): 0, np.dtype(np.float64): 1, np.dtype(np.complex64): 2, np.dtype(np.complex128): 3}


def _make(target: str | None = None) -> None:
    cmd = ["make", "-s", "-C", str(ORACLE)] + ([target, f"REF={REFERENCE_DIR}"] if target else [])
    subprocess.run(cmd, check=True, capture_output=True)


def load_oracle() -> C.CDLL:
    srcs = [ORACLE / "tmm_oracle.c", ORACLE / "tmm_ozaki_oracle.c"]
    if not ORACLE_SO.exists() or any(s.stat().st_mtime > ORACLE_SO.stat().st_mtime for s in srcs):
        _make()
    lib = C.CDLL(str(ORACLE_SO))
    lib.tmmo_optimal_tile_size.restype = _ci
    lib.tmmo_optimal_tile_size.argtypes = [_ci, _ci, _ci]
    lib.tmmo_num_tiles.restype = _i64
    lib.tmmo_num_tiles.argtypes = [_i64, _i64]
    lib.tmmo_tile_extent.restype = _i64
    lib.tmmo_tile_extent.argtypes = [_i64, _i64, _i64]
    lib.tmmo_gemm.restype = _ci
    lib.tmmo_gemm.argtypes = [_ci, C.c_char, C.c_char, _i64, _i64, _i64, _p, _p, _i64, _p, _i64, _p, _p, _i64, _ci,
                              _p, _i64, _i64, _i64, _ci]
    lib.tmmo_dd_entries.restype = None
    lib.tmmo_dd_entries.argtypes = [C.c_char, C.c_char, _i64, _i64, _i64, _d, _p, _i64, _p, _i64, _d, _p, _i64,
                                    _i64, _p, _p, _p, _p]
    lib.tmmo_error_metric.restype = _d
    lib.tmmo_error_metric.argtypes = [_i64, _p, _p, _p, _i64]
    lib.tmmo_ozaki_split.restype = None
    lib.tmmo_ozaki_split.argtypes = [_p, _i64, C.c_char, _i64, _i64, _i64, _ci, _ci, _p, _p]
    lib.tmmo_ozaki_gemm.restype = _ci
    lib.tmmo_ozaki_gemm.argtypes = [C.c_char, C.c_char, _i64, _i64, _i64, _d, _p, _i64, _p, _i64, _d, _p, _i64, _ci,
                                    _ci, _i64, _i64, _i64]
    return lib


def load_ref_host() -> C.CDLL | None:
    """The reference's host code (tile policy, geometry, schedule) compiled from its own sources
    against oracle/fake_cuda; None where the reference sources are absent."""
    if not REF_SO.exists():
        if REFERENCE_DIR is None or not (REFERENCE_DIR / "src" / "Tiled-MM" / "tiled_mm.cpp").exists():
            return None
        _make("ref")
    try:
        lib = C.CDLL(str(REF_SO))
    except OSError:
        return None
    lib.ref_optimal_tile_size.restype = _ci
    lib.ref_optimal_tile_size.argtypes = [_ci, _ci, _ci]
    lib.ref_tiled_matrix_info.restype = None
    lib.ref_tiled_matrix_info.argtypes = [_ci, _ci, _ci, _ci, _ci, _ci, _ci, _p]
    lib.ref_gemm.restype = _ci
    lib.ref_gemm.argtypes = [_ci, C.c_char, C.c_char, _ci, _ci, _ci, _p, _p, _ci, _p, _ci, _p, _p, _ci, _ci, _ci,
                             _ci, _ci, _ci, _ci, _p, _p]
    lib.fake_trace_reset.restype = None
    lib.fake_trace_get.restype = None
    lib.fake_trace_get.argtypes = [_p]
    return lib


def _sc(dtype, v) -> np.ndarray:
    return np.asarray([v], dtype=dtype)


def oracle_gemm(lib, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, tiles, copy_c_back=True, nthreads=8):
    """Runs the oracle; returns (c (in place when copy_c_back), full_c or None)."""
    dt = a.dtype
    full = None if copy_c_back else np.zeros(m * n, dtype=dt)
    al, be = _sc(dt, alpha), _sc(dt, beta)
    st = lib.tmmo_gemm(DT[dt], ta.encode(), tb.encode(), m, n, k, al.ctypes.data, a.ctypes.data, lda, b.ctypes.data,
                       ldb, be.ctypes.data, c.ctypes.data, ldc, int(copy_c_back),
                       None if full is None else full.ctypes.data, tiles[0], tiles[1], tiles[2], nthreads)
    if st != 0:
        raise ValueError("oracle rejected arguments")
    return c, full


def ref_gemm(lib, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, streams, tiles, copy_c_back=True, pin=False):
    dt = a.dtype
    full = None if copy_c_back else np.zeros(m * n, dtype=dt)
    al, be = _sc(dt, alpha), _sc(dt, beta)
    used = np.zeros(3, dtype=np.int32)
    st = lib.ref_gemm(DT[dt], ta.encode(), tb.encode(), m, n, k, al.ctypes.data, a.ctypes.data, lda, b.ctypes.data,
                      ldb, be.ctypes.data, c.ctypes.data, ldc, streams, tiles[0], tiles[1], tiles[2], int(pin),
                      int(copy_c_back), None if full is None else full.ctypes.data, used.ctypes.data)
    if st != 0:
        raise RuntimeError("reference gemm threw")
    return c, full, tuple(int(x) for x in used)


def reference_tiles(oracle, m, n, k, max_tiles, cur=(0, 0, 0)):
    """The tile sizes the reference driver picks (src/Tiled-MM/mm_handle.cpp:117-133)."""
    return (oracle.tmmo_optimal_tile_size(m, cur[0], max_tiles[0]),
            oracle.tmmo_optimal_tile_size(n, cur[1], max_tiles[1]),
            oracle.tmmo_optimal_tile_size(k, cur[2], max_tiles[2]))


def dd_entries(oracle, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c0, ldc, ii, jj):
    ii = np.ascontiguousarray(ii, dtype=np.int64)
    jj = np.ascontiguousarray(jj, dtype=np.int64)
    out = np.zeros(len(ii))
    mag = np.zeros(len(ii))
    oracle.tmmo_dd_entries(ta.encode(), tb.encode(), m, n, k, alpha, a.ctypes.data, lda, b.ctypes.data, ldb, beta,
                           None if c0 is None else c0.ctypes.data, ldc, len(ii), ii.ctypes.data, jj.ctypes.data,
                           out.ctypes.data, mag.ctypes.data)
    return out, mag


def ozaki_oracle(oracle, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, slices, tk, kb, pass_blocks, w=5):
    st = oracle.tmmo_ozaki_gemm(ta.encode(), tb.encode(), m, n, k, alpha, a.ctypes.data, lda, b.ctypes.data, ldb,
                                beta, c.ctypes.data, ldc, slices, w, tk, kb, pass_blocks)
    if st != 0:
        raise ValueError("ozaki oracle rejected arguments")
    return c
