"""Build the GB300 (sm_103a) shared library in-tree.

    python tiled-mm_gb300/build.py            # -> tiled-mm_gb300/tiledmm/lib/libtiledmm_gb300.so

Every translation unit is compiled by nvcc for sm_103a only, in parallel, then
linked into one shared library with the CUDA runtime linked statically (the
library needs no LD_LIBRARY_PATH and no cuBLAS).
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "tiledmm" / "lib"
BUILD = PKG / "_build"
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
          "--expt-relaxed-constexpr", "-I", str(PKG.parent / "include"), "-I", str(CSRC)]

SOURCES = ["tmm_core.cpp", "tmm_native.cu", "tmm_ozaki.cu", "tmm_tcgen05.cu", "tmm_batched.cu", "tmm_autotune.cpp",
           "tmm_noalloc.cu", "tmm_xt.cpp", "tmm_ozaki_embed.cu", "tmm_dropin.cpp",
           "tmm_f32tc.cu"]
LIB = OUT / "libtiledmm_gb300.so"


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        raise RuntimeError(f"build step failed: {cmd[-1]}")
    if r.stderr.strip() and os.environ.get("TMM_BUILD_VERBOSE"):
        sys.stderr.write(r.stderr)


def _newer(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return False
    t = target.stat().st_mtime
    return all(d.stat().st_mtime <= t for d in deps if d.exists())


def build(verbose: bool = False, force: bool = False) -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    OUT.mkdir(parents=True, exist_ok=True)
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted((PKG.parent / "include").glob("*.h"))
    srcs = [CSRC / s for s in SOURCES if (CSRC / s).exists()]
    objs = []
    jobs = []
    for s in srcs:
        o = BUILD / (s.stem + ".o")
        objs.append(o)
        if force or not _newer(o, [s] + headers):
            jobs.append([NVCC, *ARCH, *COMMON, "-c", str(s), "-o", str(o)])
    with ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for f in [ex.submit(_run, j) for j in jobs]:
            f.result()
    if force or jobs or not LIB.exists():
        _run([NVCC, *ARCH, "-shared", "-cudart", "static", "-Xlinker", f"-soname={LIB.name}", "-o", str(LIB),
              *map(str, objs), "-lpthread", "-ldl", "-lrt"])
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
