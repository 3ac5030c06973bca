"""Python mirror of Tiled-MM's public API over the GB300 C ABI (include/tmm_c_api.h).

Same names and argument meaning as the reference's C++ API:

    ctx = tiledmm.make_context(np.float64, n_streams=2, tile_m=5000, tile_n=5000, tile_k=5000)
    tiledmm.gemm(ctx, 'N', 'N', m, n, k, alpha, a, ld_a, b, ld_b, beta, c, ld_c,
                 pin_host_buffers=True, copy_c_back=True)
    c_dev_ptr = ctx.get_full_device_buffer_c().data()

(src/Tiled-MM/mm_handle.hpp:60-76, src/Tiled-MM/tiled_mm.hpp:69-79).
Matrices are NumPy arrays holding column-major data (any array whose memory
is the column-major matrix: a Fortran-ordered 2-D array or a flat buffer).
Failures raise RuntimeError("GPU ERROR: ...") as the reference throws
std::runtime_error("GPU ERROR") (src/Tiled-MM/util.hpp:13-27).

There is no CPU fallback: importing this module fails if the CUDA library
has not been built (python tiled-mm_gb300/build.py).
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "lib" / "libtiledmm_gb300.so"

if not LIB_PATH.exists():
    raise ImportError(f"tiledmm: CUDA library {LIB_PATH} is missing; build it with "
                      f"`python tiled-mm_gb300/build.py` (no CPU fallback exists)")

_lib = C.CDLL(str(LIB_PATH))

FLOAT, DOUBLE, COMPLEX_FLOAT, COMPLEX_DOUBLE = 0, 1, 2, 3
PATH_NATIVE, PATH_OZAKI = 0, 1
OZAKI_IMMA, OZAKI_TCGEN05 = 0, 1
TILE_POLICY_REFERENCE, TILE_POLICY_FIXED, TILE_POLICY_AUTOTUNE = 0, 1, 2
STATUS = {0: "success", 1: "invalid argument", 2: "CUDA error", 3: "out of device memory",
          4: "not supported", 5: "internal error", 6: "device wait timed out"}

_DTYPES = {np.dtype(np.float32): FLOAT, np.dtype(np.float64): DOUBLE,
           np.dtype(np.complex64): COMPLEX_FLOAT, np.dtype(np.complex128): COMPLEX_DOUBLE}
_NP = {v: k for k, v in _DTYPES.items()}

_p = C.c_void_p
_i64 = C.c_int64
_ci = C.c_int
_sz = C.c_size_t

# exported symbols and signatures (the same list include/tmm_c_api.h declares)
SIGNATURES = {
    "tmm_create": (_ci, [_ci, _ci, _ci, _ci, _ci, C.POINTER(_p)]),
    "tmm_destroy": (_ci, [_p]),
    "tmm_gemm": (_ci, [_p, C.c_char, C.c_char, _i64, _i64, _i64, _p, _p, _i64, _p, _i64, _p, _p, _i64, _ci, _ci]),
    "tmm_gemm_device": (_ci, [_p, C.c_char, C.c_char, _i64, _i64, _i64, _p, _p, _i64, _p, _i64, _p, _p, _i64, _p]),
    "tmm_ozaki_gemm_device_noalloc": (_ci, [C.c_char, C.c_char, _i64, _i64, _i64, C.c_double, _p, _i64, _p, _i64,
                                            C.c_double, _p, _i64, _ci, _i64, _p]),
    "tmm_ozaki_noalloc_status": (_ci, [_p]),
    "tmm_gemm_batched": (_ci, [_p, _ci, _p, _ci]),
    "tmm_device_status": (_ci, [_p, _p]),
    "tmm_xt_create": (_ci, [C.POINTER(_p)]),
    "tmm_xt_destroy": (_ci, [_p]),
    "tmm_xt_set_block_dim": (_ci, [_p, _ci]),
    "tmm_xt_get_block_dim": (_ci, [_p, C.POINTER(_ci)]),
    "tmm_xt_set_path": (_ci, [_p, _ci, _ci]),
    "tmm_xt_last_error": (C.c_char_p, [_p]),
    "tmm_xt_sgemm": (_ci, [_p, _ci, _ci, _i64, _i64, _i64, _p, _p, _i64, _p, _i64, _p, _p, _i64]),
    "tmm_xt_dgemm": (_ci, [_p, _ci, _ci, _i64, _i64, _i64, _p, _p, _i64, _p, _i64, _p, _p, _i64]),
    "tmm_xt_cgemm": (_ci, [_p, _ci, _ci, _i64, _i64, _i64, _p, _p, _i64, _p, _i64, _p, _p, _i64]),
    "tmm_xt_zgemm": (_ci, [_p, _ci, _ci, _i64, _i64, _i64, _p, _p, _i64, _p, _i64, _p, _p, _i64]),
    "tmm_get_full_c": (_ci, [_p, C.POINTER(_p), C.POINTER(_sz), C.POINTER(_sz)]),
    "tmm_get_stream": (_ci, [_p, _ci, C.POINTER(_p)]),
    "tmm_get_result_stream": (_ci, [_p, C.POINTER(_p)]),
    "tmm_get_device_buffer": (_ci, [_p, C.c_char, _ci, C.POINTER(_p)]),
    "tmm_stream_create": (_ci, [C.POINTER(_p)]),
    "tmm_stream_destroy": (_ci, [_p]),
    "tmm_event_create": (_ci, [C.POINTER(_p)]),
    "tmm_event_destroy": (_ci, [_p]),
    "tmm_event_record": (_ci, [_p, _p]),
    "tmm_event_synchronize": (_ci, [_p]),
    "tmm_event_elapsed": (_ci, [_p, _p, C.POINTER(C.c_double)]),
    "tmm_stream_wait_event": (_ci, [_p, _p]),
    "tmm_set_num_streams": (_ci, [_p, _ci]),
    "tmm_get_num_streams": (_ci, [_p, C.POINTER(_ci)]),
    "tmm_set_tile_sizes": (_ci, [_p, _ci, _ci, _ci]),
    "tmm_get_tile_sizes": (_ci, [_p, C.POINTER(_ci), C.POINTER(_ci), C.POINTER(_ci)]),
    "tmm_set_full_sizes": (_ci, [_p, _i64, _i64, _i64]),
    "tmm_optimal_tile_sizes": (_ci, [_p, _i64, _i64, _i64, C.POINTER(_ci), C.POINTER(_ci), C.POINTER(_ci)]),
    "tmm_get_max_tile_sizes": (_ci, [_p, C.POINTER(_ci), C.POINTER(_ci), C.POINTER(_ci)]),
    "tmm_set_streams_and_tiles": (_ci, [_p, _ci, _ci, _ci, _ci]),
    "tmm_set_path": (_ci, [_p, _ci, _ci]),
    "tmm_get_path": (_ci, [_p, C.POINTER(_ci), C.POINTER(_ci)]),
    "tmm_set_ozaki_engine": (_ci, [_p, _ci]),
    "tmm_get_ozaki_engine": (_ci, [_p, C.POINTER(_ci), C.POINTER(_ci), C.POINTER(_i64)]),
    "tmm_set_tile_policy": (_ci, [_p, _ci]),
    "tmm_get_autotune_report": (_ci, [_p, C.c_char_p, _sz]),
    "tmm_set_memory_limit": (_ci, [_p, _sz]),
    "tmm_get_stats": (_ci, [_p, _p]),
    "tmm_set_kernel_timing": (_ci, [_p, _ci]),
    "tmm_get_kernel_time": (_ci, [_p, _p, _p]),
    "tmm_get_kernel_busy_time": (_ci, [_p, _p, _p]),
    "tmm_last_error": (C.c_char_p, [_p]),
    "tmm_status_string": (C.c_char_p, [_ci]),
    "tmm_malloc_pinned": (_ci, [_sz, C.POINTER(_p)]),
    "tmm_free_pinned": (_ci, [_p]),
    "tmm_copy_to_device": (_ci, [_p, _p, _sz]),
    "tmm_copy_to_host": (_ci, [_p, _p, _sz]),
    "tmm_memcpy_async": (_ci, [_p, _p, _sz, _p]),
    "tmm_malloc_device": (_ci, [_sz, C.POINTER(_p)]),
    "tmm_free_device": (_ci, [_p]),
    "tmm_fill_host_f64": (_ci, [_p, _i64, _i64, _i64, _ci, C.c_double, C.c_uint64, C.c_uint64, _ci]),
    "tmm_fill_device_f64": (_ci, [_p, _i64, _i64, _i64, _ci, C.c_double, C.c_uint64, C.c_uint64, _p]),
    "tmm_error_metric_f64": (_ci, [C.c_char, C.c_char, _i64, _i64, _i64, C.c_double, _p, _i64, _p, _i64,
                                   C.c_double, _p, _i64, _p, _i64, _i64, C.c_uint64, _ci, C.POINTER(C.c_double)]),
}

for _name, (_res, _args) in SIGNATURES.items():
    _f = getattr(_lib, _name, None)
    if _f is not None:
        _f.restype = _res
        _f.argtypes = _args


class Stats(C.Structure):
    _fields_ = [("h2d_bytes", C.c_uint64), ("d2h_bytes", C.c_uint64), ("kernels", C.c_uint64),
                ("tiles_loaded", C.c_uint64), ("tiles_reused", C.c_uint64), ("tile_m", _ci), ("tile_n", _ci),
                ("tile_k", _ci), ("n_streams", _ci), ("path", _ci), ("ozaki_slices", _ci), ("seconds", C.c_double),
                ("batch_graph", _ci), ("direct_host", _ci), ("direct_bytes", C.c_uint64), ("autotune_state", _ci)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


def lib() -> C.CDLL:
    return _lib


def _check(status: int, ctx_ptr=None) -> None:
    if status != 0:
        msg = _lib.tmm_last_error(ctx_ptr).decode(errors="replace")
        raise RuntimeError(f"GPU ERROR: {STATUS.get(status, status)}: {msg}")


def _ptr(x) -> int | None:
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if isinstance(x, np.ndarray):
        return x.ctypes.data
    if hasattr(x, "data_ptr"):  # torch tensors (device pointers for gemm_device)
        return x.data_ptr()
    raise TypeError(f"cannot take the address of {type(x)}")


def _scalar(dtype: int, v) -> C.Array:
    arr = np.asarray([v], dtype=_NP[dtype])
    return arr


class DeviceVector:
    """View of mm_handle::get_full_device_buffer_c() (src/Tiled-MM/device_vector.hpp:26-28)."""

    def __init__(self, ctx: "MMHandle"):
        self._ctx = ctx

    def _query(self):
        p, size, cap = _p(), _sz(), _sz()
        _check(_lib.tmm_get_full_c(self._ctx._h, C.byref(p), C.byref(size), C.byref(cap)), self._ctx._h)
        return p.value or 0, size.value, cap.value

    def data(self) -> int:
        return self._query()[0]

    def size(self) -> int:
        return self._query()[1]

    def capacity(self) -> int:
        return self._query()[2]

    def to_host(self, out: np.ndarray) -> np.ndarray:
        """Copy size() elements to `out` (copy_to_host, src/Tiled-MM/util.hpp:85-88)."""
        ptr, size, _ = self._query()
        nbytes = min(size * self._ctx.itemsize, out.nbytes)
        _check(_lib.tmm_copy_to_host(ptr, out.ctypes.data, nbytes))
        return out


class MMHandle:
    """mm_handle<Scalar> (src/Tiled-MM/mm_handle.hpp:11-55)."""

    def __init__(self, dtype, n_streams: int = 2, tile_m: int = 5000, tile_n: int = 5000, tile_k: int = 5000):
        self.dtype = _DTYPES[np.dtype(dtype)] if not isinstance(dtype, int) else dtype
        self.np_dtype = _NP[self.dtype]
        self.itemsize = self.np_dtype.itemsize
        h = _p()
        _check(_lib.tmm_create(self.dtype, n_streams, tile_m, tile_n, tile_k, C.byref(h)))
        self._h = h
        self._full_c = DeviceVector(self)

    def close(self) -> None:
        if getattr(self, "_h", None):
            _lib.tmm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- reference mm_handle methods
    def set_num_streams(self, n: int) -> None:
        _check(_lib.tmm_set_num_streams(self._h, n), self._h)

    def get_num_streams(self) -> int:
        v = _ci()
        _check(_lib.tmm_get_num_streams(self._h, C.byref(v)), self._h)
        return v.value

    def set_tile_sizes(self, tile_m: int, tile_n: int | None = None, tile_k: int | None = None) -> None:
        tile_n = tile_m if tile_n is None else tile_n
        tile_k = tile_m if tile_k is None else tile_k
        _check(_lib.tmm_set_tile_sizes(self._h, tile_m, tile_n, tile_k), self._h)

    def get_tile_sizes(self) -> tuple[int, int, int]:
        a, b, c = _ci(), _ci(), _ci()
        _check(_lib.tmm_get_tile_sizes(self._h, C.byref(a), C.byref(b), C.byref(c)), self._h)
        return a.value, b.value, c.value

    def set_full_sizes(self, m: int, n: int, k: int) -> None:
        _check(_lib.tmm_set_full_sizes(self._h, m, n, k), self._h)

    def optimal_tile_sizes(self, m: int, n: int, k: int) -> tuple[int, int, int]:
        a, b, c = _ci(), _ci(), _ci()
        _check(_lib.tmm_optimal_tile_sizes(self._h, m, n, k, C.byref(a), C.byref(b), C.byref(c)), self._h)
        return a.value, b.value, c.value

    def get_max_tile_sizes(self) -> tuple[int, int, int]:
        a, b, c = _ci(), _ci(), _ci()
        _check(_lib.tmm_get_max_tile_sizes(self._h, C.byref(a), C.byref(b), C.byref(c)), self._h)
        return a.value, b.value, c.value

    def set_streams_and_tiles(self, n_streams: int, tile_m: int, tile_n: int, tile_k: int) -> None:
        _check(_lib.tmm_set_streams_and_tiles(self._h, n_streams, tile_m, tile_n, tile_k), self._h)

    def get_full_device_buffer_c(self) -> DeviceVector:
        return self._full_c

    # ---- additions
    def set_path(self, path: int, slices: int = 0) -> None:
        _check(_lib.tmm_set_path(self._h, path, slices), self._h)

    def get_path(self) -> tuple[int, int]:
        a, b = _ci(), _ci()
        _check(_lib.tmm_get_path(self._h, C.byref(a), C.byref(b)), self._h)
        return a.value, b.value

    def set_ozaki_engine(self, engine) -> None:
        e = {"imma": OZAKI_IMMA, "tcgen05": OZAKI_TCGEN05}.get(engine, engine)
        _check(_lib.tmm_set_ozaki_engine(self._h, e), self._h)

    def ozaki_engine(self) -> dict:
        """Which engine runs the Ozaki slice products, its k-block and exactness pass length."""
        e, kb, pb = _ci(), _ci(), _i64()
        _check(_lib.tmm_get_ozaki_engine(self._h, C.byref(e), C.byref(kb), C.byref(pb)), self._h)
        return {"engine": ["imma", "tcgen05"][e.value], "k_block": kb.value, "pass_blocks": pb.value}

    def set_tile_policy(self, policy: int) -> None:
        _check(_lib.tmm_set_tile_policy(self._h, policy), self._h)

    def autotune_report(self) -> str:
        """The autotuner's measured candidates and choice for this context's last autotuned call."""
        buf = C.create_string_buffer(4096)
        _check(_lib.tmm_get_autotune_report(self._h, buf, len(buf)), self._h)
        return buf.value.decode()

    def set_memory_limit(self, nbytes: int) -> None:
        _check(_lib.tmm_set_memory_limit(self._h, nbytes), self._h)

    def set_kernel_timing(self, on: bool = True) -> None:
        """Bracket every engine kernel launch with CUDA events on its stream (clears the totals)."""
        _check(_lib.tmm_set_kernel_timing(self._h, int(bool(on))), self._h)

    def kernel_time(self) -> tuple[float, int]:
        """(device seconds, launches) of the engine kernels since set_kernel_timing(True)."""
        sec, n = C.c_double(), C.c_uint64()
        _check(_lib.tmm_get_kernel_time(self._h, C.byref(sec), C.byref(n)), self._h)
        return sec.value, n.value

    def kernel_busy_time(self) -> tuple[float, float]:
        """(busy seconds, span seconds) of the same launches: the union of their device
        intervals (overlapping launches on several streams count once) and first start to
        last end."""
        busy, span = C.c_double(), C.c_double()
        _check(_lib.tmm_get_kernel_busy_time(self._h, C.byref(busy), C.byref(span)), self._h)
        return busy.value, span.value

    def device_status(self, stream: int | None = None) -> int:
        """Waits for `stream`; TMM_ERROR_TIMEOUT (6) if a kernel of this context gave up a pipeline
        wait since the last check, else 0."""
        return _lib.tmm_device_status(self._h, stream)

    def stats(self) -> dict:
        s = Stats()
        _check(_lib.tmm_get_stats(self._h, C.byref(s)), self._h)
        return s.as_dict()

    def last_error(self) -> str:
        return _lib.tmm_last_error(self._h).decode(errors="replace")


def make_context(dtype=np.float64, n_streams: int = 2, tile_m: int = 5000, tile_n: int = 5000,
                 tile_k: int = 5000) -> MMHandle:
    """gpu::make_context<Scalar>(streams, tile_m, tile_n, tile_k) (src/Tiled-MM/mm_handle.hpp:60-76)."""
    return MMHandle(dtype, n_streams, tile_m, tile_n, tile_k)


def gemm(ctx: MMHandle, trans_a: str, trans_b: str, m: int, n: int, k: int, alpha, a, ld_a: int, b, ld_b: int,
         beta, c, ld_c: int, pin_host_buffers: bool = True, copy_c_back: bool = True) -> None:
    """gpu::gemm(ctx, trans_a, trans_b, m, n, k, alpha, a, ld_a, b, ld_b, beta, c, ld_c, pin, copy_c_back)
    (src/Tiled-MM/tiled_mm.hpp:69-79).  a, b, c: host arrays of ctx's dtype holding column-major data."""
    for name, x in (("a", a), ("b", b), ("c", c)):
        if isinstance(x, np.ndarray) and x.dtype != ctx.np_dtype:
            raise TypeError(f"{name} has dtype {x.dtype}, context is {ctx.np_dtype}")
    al, be = _scalar(ctx.dtype, alpha), _scalar(ctx.dtype, beta)
    st = _lib.tmm_gemm(ctx._h, trans_a.encode()[:1], trans_b.encode()[:1], m, n, k, al.ctypes.data, _ptr(a), ld_a,
                       _ptr(b), ld_b, be.ctypes.data, _ptr(c), ld_c, int(bool(pin_host_buffers)), int(bool(copy_c_back)))
    _check(st, ctx._h)


def gemm_device(ctx: MMHandle, trans_a: str, trans_b: str, m: int, n: int, k: int, alpha, a_dev, ld_a: int, b_dev,
                ld_b: int, beta, c_dev, ld_c: int, stream: int | None = None) -> None:
    """Device-resident operands (pointers or torch CUDA tensors); enqueued on `stream` (cudaStream_t as int)."""
    al, be = _scalar(ctx.dtype, alpha), _scalar(ctx.dtype, beta)
    st = _lib.tmm_gemm_device(ctx._h, trans_a.encode()[:1], trans_b.encode()[:1], m, n, k, al.ctypes.data, _ptr(a_dev),
                              ld_a, _ptr(b_dev), ld_b, be.ctypes.data, _ptr(c_dev), ld_c, stream)
    _check(st, ctx._h)


class BatchProblem(C.Structure):
    """tmm_batch_problem (include/tmm_c_api.h)."""
    _fields_ = [("dtype", _ci), ("trans_a", C.c_char), ("trans_b", C.c_char), ("m", _i64), ("n", _i64), ("k", _i64),
                ("alpha", C.c_double), ("beta", C.c_double), ("a", _p), ("ld_a", _i64), ("b", _p), ("ld_b", _i64),
                ("c", _p), ("ld_c", _i64)]


class XtHandle:
    """cublasXt-style handle (include/tmm_c_api.h, tmm_xt_*): one block dimension for all tile
    sizes, ?gemm with trans as cublasOperation_t values (0 N, 1 T, 2 C) on host or device
    pointers, page-locking for the call, synchronous."""

    _FN = {np.float32: "tmm_xt_sgemm", np.float64: "tmm_xt_dgemm", np.complex64: "tmm_xt_cgemm",
           np.complex128: "tmm_xt_zgemm"}
    _DT = {np.float32: FLOAT, np.float64: DOUBLE, np.complex64: COMPLEX_FLOAT, np.complex128: COMPLEX_DOUBLE}

    def __init__(self, block_dim: int | None = None):
        self._h = _p()
        _check(_lib.tmm_xt_create(C.byref(self._h)))
        if block_dim is not None:
            self.set_block_dim(block_dim)

    def _check(self, status: int) -> None:
        if status != 0:
            msg = _lib.tmm_xt_last_error(self._h).decode(errors="replace")
            raise RuntimeError(f"GPU ERROR: {STATUS.get(status, status)}: {msg}")

    def set_block_dim(self, block_dim: int) -> None:
        self._check(_lib.tmm_xt_set_block_dim(self._h, block_dim))

    def block_dim(self) -> int:
        v = _ci()
        self._check(_lib.tmm_xt_get_block_dim(self._h, C.byref(v)))
        return v.value

    def set_path(self, path: int, slices: int = 0) -> None:
        self._check(_lib.tmm_xt_set_path(self._h, path, slices))

    def gemm(self, dtype, transa: int, transb: int, m: int, n: int, k: int, alpha, a, lda: int, b, ldb: int, beta,
             c, ldc: int) -> None:
        dt = np.dtype(dtype).type
        al, be = _scalar(self._DT[dt], alpha), _scalar(self._DT[dt], beta)
        fn = getattr(_lib, self._FN[dt])
        self._check(fn(self._h, transa, transb, m, n, k, al.ctypes.data, _ptr(a), lda, _ptr(b), ldb, be.ctypes.data,
                       _ptr(c), ldc))

    def close(self) -> None:
        if self._h:
            _lib.tmm_xt_destroy(self._h)
            self._h = _p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def gemm_batched(ctx: MMHandle, problems: list[dict], device_operands: bool = False) -> None:
    """Many GEMMs (FP64 and FP32 mixed) in one persistent launch; each dict has the keys
    trans_a, trans_b, m, n, k, alpha, a, ld_a, b, ld_b, beta, c, ld_c (arrays of float32 or
    float64, host or, with device_operands, device)."""
    arr = (BatchProblem * max(1, len(problems)))()
    for i, p in enumerate(problems):
        dt = p["a"].dtype if isinstance(p["a"], np.ndarray) else np.dtype(p.get("dtype", np.float64))
        arr[i] = BatchProblem(_DTYPES[np.dtype(dt)], p["trans_a"].encode()[:1], p["trans_b"].encode()[:1], p["m"],
                              p["n"], p["k"], float(p["alpha"]), float(p["beta"]), _ptr(p["a"]), p["ld_a"],
                              _ptr(p["b"]), p["ld_b"], _ptr(p["c"]), p["ld_c"])
    _check(_lib.tmm_gemm_batched(ctx._h, len(problems), C.cast(arr, C.c_void_p), int(bool(device_operands))), ctx._h)


class PinnedArray:
    """Page-locked host array (gpu::malloc_pinned, src/Tiled-MM/util.hpp:64-72)."""

    def __init__(self, shape, dtype=np.float64, order: str = "F"):
        dt = np.dtype(dtype)
        count = int(np.prod(shape))
        p = _p()
        _check(_lib.tmm_malloc_pinned(max(1, count * dt.itemsize), C.byref(p)))
        self._p = p.value
        buf = (C.c_char * max(1, count * dt.itemsize)).from_address(self._p)
        self.array = np.ndarray(shape, dtype=dt, buffer=buf, order=order)

    def free(self) -> None:
        if getattr(self, "_p", None):
            self.array = None
            _lib.tmm_free_pinned(self._p)
            self._p = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def fill_host(x: np.ndarray, rows: int, cols: int, ld: int, kind: int = 0, param: float = 0.0, seed: int = 0,
              mat_id: int = 0, n_threads: int | None = None) -> np.ndarray:
    """Seeded synthetic FP64 matrix (tiled-mm_gb300/csrc/tmm_datagen.h) into host memory."""
    if x.dtype != np.float64:
        raise TypeError("fill_host fills float64 arrays")
    nt = n_threads or min(32, len(os.sched_getaffinity(0)))
    _check(_lib.tmm_fill_host_f64(x.ctypes.data, rows, cols, ld, kind, param, seed, mat_id, nt))
    return x


def fill_device(ptr: int, rows: int, cols: int, ld: int, kind: int = 0, param: float = 0.0, seed: int = 0,
                mat_id: int = 0, stream: int | None = None) -> None:
    _check(_lib.tmm_fill_device_f64(ptr, rows, cols, ld, kind, param, seed, mat_id, stream))


def error_metric(trans_a, trans_b, m, n, k, alpha, a, ld_a, b, ld_b, beta, c0, ld_c0, c, ld_c, n_samples=4096,
                 seed=1, n_threads=None) -> float:
    """max |C - C*| / (k u (|alpha||A||B| + |beta||C0|)) over sampled entries, C* in twice-working precision."""
    out = C.c_double()
    nt = n_threads or min(32, len(os.sched_getaffinity(0)))
    _check(_lib.tmm_error_metric_f64(trans_a.encode()[:1], trans_b.encode()[:1], m, n, k, float(alpha), _ptr(a),
                                     ld_a, _ptr(b), ld_b, float(beta), _ptr(c0), ld_c0, _ptr(c), ld_c, n_samples,
                                     seed, nt, C.byref(out)))
    return out.value


GEN_UNIFORM, GEN_INT09, GEN_UEXP, GEN_NORMAL_ROWEXP, GEN_NORMAL_COLEXP, GEN_SMALLINT = range(6)
