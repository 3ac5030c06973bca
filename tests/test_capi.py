"""CPU-side checks of the C-ABI library: it loads, exports every entry point include/tmm_c_api.h
declares, its host-only helpers (seeded generator, error metric) agree with independent
restatements, and the headers compile as C and as the drop-in C++ API.  No GPU compute."""
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import HAS_GPU, ROOT
from oracle_lib import dd_entries

HEADER = ROOT / "include" / "tmm_c_api.h"


def declared_symbols():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(tmm_\w+)\s*\(", text, re.M)))


def test_exports_every_declared_symbol(tmm):
    syms = declared_symbols()
    assert len(syms) >= 30
    out = subprocess.run(["nm", "-D", "--defined-only", str(tmm.LIB_PATH)], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r" T (tmm_\w+)", out))
    missing = [s for s in syms if s not in exported]
    assert not missing, missing
    # and the Python binding knows each of them
    assert set(syms) <= set(tmm.SIGNATURES), set(syms) - set(tmm.SIGNATURES)


def test_library_links_no_cublas(tmm):
    out = subprocess.run(["readelf", "-d", str(tmm.LIB_PATH)], capture_output=True, text=True, check=True).stdout
    assert "cublas" not in out  # every FLOP is this library's own kernels


def test_status_strings(tmm):
    lib = tmm.lib()
    assert lib.tmm_status_string(0) == b"success"
    assert lib.tmm_status_string(1) == b"invalid argument"
    assert lib.tmm_last_error(None) is not None


def test_null_context_is_rejected(tmm):
    lib = tmm.lib()
    one = np.ones(1)
    st = lib.tmm_gemm(None, b"N", b"N", 1, 1, 1, one.ctypes.data, one.ctypes.data, 1, one.ctypes.data, 1,
                      one.ctypes.data, one.ctypes.data, 1, 0, 1)
    assert st == 1


@pytest.mark.skipif(HAS_GPU, reason="checks the no-device error path")
def test_create_without_gpu_fails_cleanly(tmm):
    with pytest.raises(RuntimeError, match="GPU ERROR"):
        tmm.make_context(np.float64)


# ---------------------------------------------------------------- seeded generator
M64 = (1 << 64) - 1


def splitmix64(x):
    x = (x + 0x9E3779B97F4A7C15) & M64
    x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & M64
    x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & M64
    return x ^ (x >> 31)


def gen_value(kind, param, seed, mid, row, col, rows):
    idx = row + col * rows
    h = splitmix64(seed ^ (mid << 56) ^ idx)
    u = float(h >> 11) * 2.0 ** -52 - 1.0
    if kind == 0:
        return u
    if kind == 1:
        return float(h % 10)
    if kind == 2:
        p = int(param)
        he = splitmix64(seed ^ ((mid ^ 0x40) << 56) ^ idx)
        e = int(he % (2 * p + 1)) - p
        return u * 2.0 ** e
    raise ValueError(kind)


@pytest.mark.parametrize("kind,param", [(0, 0.0), (1, 0.0), (2, 20.0)])
def test_host_generator_matches_restatement(tmm, kind, param):
    rows, cols, ld = 13, 7, 16
    x = np.full(ld * cols, -7.0)
    tmm.fill_host(x, rows, cols, ld, kind, param, seed=123, mat_id=2, n_threads=3)
    X = x.reshape(cols, ld).T
    for j in range(cols):
        for i in range(rows):
            assert X[i, j] == gen_value(kind, param, 123, 2, i, j, rows)
    assert np.all(X[rows:] == -7.0)  # padding rows untouched


def test_uniform_generator_range_and_mean(tmm):
    x = np.zeros(200000)
    tmm.fill_host(x, 200000, 1, 200000, 0, 0.0, seed=0, mat_id=0)
    assert x.min() >= -1.0 and x.max() < 1.0
    assert abs(x.mean()) < 0.01


# ---------------------------------------------------------------- error metric
def test_error_metric_agrees_with_oracle(tmm, oracle):
    rng = np.random.default_rng(9)
    m, n, k = 31, 17, 64
    a, b, c0 = rng.uniform(-1, 1, m * k), rng.uniform(-1, 1, k * n), rng.uniform(-1, 1, m * n)
    exact = 1.25 * (a.reshape(k, m).T @ b.reshape(n, k).T) - 0.5 * c0.reshape(n, m).T
    c = np.asfortranarray(exact).reshape(-1, order="F").copy()
    c[5] += 1e-12  # a known error
    got = tmm.error_metric("N", "N", m, n, k, 1.25, a, m, b, k, -0.5, c0, m, c, m, n_samples=m * n * 4, seed=3)
    ii, jj = np.repeat(np.arange(m), n), np.tile(np.arange(n), m)
    ref, mag = dd_entries(oracle, "N", "N", m, n, k, 1.25, a, m, b, k, -0.5, c0, m, ii, jj)
    vals = c.reshape(n, m).T[ii, jj].copy()
    want = oracle.tmmo_error_metric(len(ii), vals.ctypes.data, ref.ctypes.data, mag.ctypes.data, k)
    assert got <= want * (1 + 1e-9) and got > 0.5 * want  # samples cover most entries


# ---------------------------------------------------------------- headers
def test_c_header_is_plain_c(tmp_path):
    src = tmp_path / "t.c"
    src.write_text('#include "tmm_c_api.h"\nint main(void){ tmm_context* c = 0; return tmm_destroy(c); }\n')
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-fsyntax-only", "-I", str(ROOT / "include"), str(src)],
                   check=True)


def test_cpp_dropin_headers_compile():
    subprocess.run(["g++", "-std=c++14", "-Wall", "-fsyntax-only", "-I", str(ROOT / "include"),
                    str(ROOT / "tests" / "cpp" / "test_multiply_gb300.cpp")], check=True)


def test_noalloc_argument_checks_need_no_gpu(tmm):
    """The allocation-free entry rejects bad arguments and oversized requests before it
    touches a device (the pointers below are never dereferenced)."""
    lib = tmm.lib()
    fake = 256  # a non-null stand-in pointer
    assert lib.tmm_ozaki_gemm_device_noalloc(b"X", b"N", 8, 8, 8, 1.0, fake, 8, fake, 8, 0.0, fake, 8, 4, 0, None) == 1
    assert lib.tmm_ozaki_gemm_device_noalloc(b"N", b"N", 8, 8, 8, 1.0, fake, 8, fake, 8, 0.0, fake, 8, 0, 0, None) == 1
    # m near 2^62: rejected before any byte count could overflow
    big = 1 << 62
    st = lib.tmm_ozaki_gemm_device_noalloc(b"N", b"N", big, 8, 128, 1.0, fake, big, fake, 128, 0.0, fake, big, 4, 0,
                                           None)
    assert st == 1 and b"scratch" in lib.tmm_last_error(None)
    # 20 slices of two 200000-line operands cannot fit one 128-wide k step
    st = lib.tmm_ozaki_gemm_device_noalloc(b"N", b"N", 200000, 200000, 128, 1.0, fake, 200000, fake, 128, 0.0, fake,
                                           200000, 20, 0, None)
    assert st == 1 and b"scratch" in lib.tmm_last_error(None)
    # a k_tile no larger than k that the scratch cannot hold
    st = lib.tmm_ozaki_gemm_device_noalloc(b"N", b"N", 2048, 2048, 8192, 1.0, fake, 2048, fake, 8192, 0.0, fake, 2048,
                                           13, 8192, None)
    assert st == 1 and b"k_tile" in lib.tmm_last_error(None)


def test_library_exports_the_four_gemm_instantiations(tmm):
    """gpu::gemm<S> is compiled into the library for the reference's four scalar types
    (src/Tiled-MM/tiled_mm.cpp:626-668), so programs link against it as against the reference."""
    out = subprocess.run(["nm", "-D", "--defined-only", "-C", str(tmm.LIB_PATH)], capture_output=True, text=True,
                         check=True).stdout
    for s in ("float", "double", "std::complex<float>", "std::complex<double>"):
        assert f"void gpu::gemm<{s}" in out.replace("> >", ">>").replace("<float >", "<float>").replace(
            "<double >", "<double>"), s


def test_cmake_consumer_links_against_the_package(tmm, tmp_path):
    """A downstream CMake project does find_package(Tiled-MM) and links Tiled-MM::Tiled-MM,
    exactly as against the reference's package (CMakeLists.txt:42-63); it builds here (it runs on
    a GPU only)."""
    import shutil

    if shutil.which("cmake") is None:
        pytest.skip("cmake is not installed on this machine")
    build = tmp_path / "build"
    cfg = subprocess.run(["cmake", "-S", str(ROOT / "tests" / "cpp" / "consumer"), "-B", str(build),
                          f"-DCMAKE_PREFIX_PATH={ROOT / 'tiled-mm_gb300' / 'tiledmm'}"], capture_output=True,
                         text=True)
    assert cfg.returncode == 0, cfg.stdout + cfg.stderr
    bld = subprocess.run(["cmake", "--build", str(build)], capture_output=True, text=True)
    assert bld.returncode == 0, bld.stdout + bld.stderr
    exe = build / "consumer"
    assert exe.exists()
    needed = subprocess.run(["readelf", "-d", str(exe)], capture_output=True, text=True, check=True).stdout
    assert "libtiledmm_gb300.so" in needed
