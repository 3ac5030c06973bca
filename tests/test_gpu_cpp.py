"""The drop-in C++ API (include/Tiled-MM/*.hpp) compiled against the library and run with the
reference test program's semantics (tests/test-multiply.cpp) at its CI and ctest shapes."""
import subprocess

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def driver(tmm, tmp_path_factory):
    exe = tmp_path_factory.mktemp("cpp") / "test_multiply_gb300"
    libdir = tmm.LIB_PATH.parent
    subprocess.run(["g++", "-std=c++14", "-O2", "-I", str(ROOT / "include"), str(ROOT / "tests" / "cpp" / "test_multiply_gb300.cpp"),
                    "-o", str(exe), "-L", str(libdir), "-ltiledmm_gb300", f"-Wl,-rpath,{libdir}"], check=True)
    return exe


@pytest.mark.parametrize("args", [
    "50 200 21 4 4 4 2 NN 1 0",        # ci/daint-alps.yml:48-56
    "5 2 2 4 4 4 2 NN 1 0",            # ci/daint-alps.yml:58-64
    "1000 1000 1000 5000 5000 5000 2 NN 1 0",  # tests/CMakeLists.txt:11
    "1234 4567 1357 5000 5000 5000 2 NN 1 0",  # tests/CMakeLists.txt:13
    "300 200 100 64 64 64 3 TN 1 1 7",
    "300 200 101 64 64 64 2 nt -1 0.5 0",
    "257 129 300 128 128 128 2 TT 2 1 1",
    "300 200 100 64 64 64 3 TN 1 1 7 6",   # Ozaki path, 6 slices
])
def test_cpp_driver(driver, args):
    r = subprocess.run([str(driver), *args.split()], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "The result is CORRECT" in r.stdout


def test_consumer_program_runs(tmm, tmp_path):
    """The downstream program of tests/cpp/consumer (gpu::gemm from the library's explicit
    instantiations for all four scalar types, the context's streams, events and device buffers),
    built the way its CMake target would build it."""
    exe = tmp_path / "consumer"
    libdir = tmm.LIB_PATH.parent
    subprocess.run(["g++", "-std=c++14", "-O2", "-DTILED_MM_CUDA", "-I", str(ROOT / "include"),
                    str(ROOT / "tests" / "cpp" / "consumer" / "main.cpp"), "-o", str(exe), "-L", str(libdir),
                    "-ltiledmm_gb300", f"-Wl,-rpath,{libdir}"], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "consumer OK" in r.stdout, r.stdout + r.stderr
