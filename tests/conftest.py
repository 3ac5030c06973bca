import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "tiled-mm_gb300"
sys.path.insert(0, str(PKG))
sys.path.insert(0, str(ROOT / "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running case")


def _gpu_available() -> bool:
    try:
        r = subprocess.run(["nvidia-smi", "-L"], capture_output=True, text=True, timeout=30)
        return r.returncode == 0 and "GPU" in r.stdout
    except Exception:
        return False


HAS_GPU = _gpu_available()


def pytest_collection_modifyitems(config, items):
    if HAS_GPU:
        return
    skip = pytest.mark.skip(reason="no GPU on this machine")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def tmm():
    """The product library (built in-tree); import fails loudly when it is missing."""
    lib = PKG / "tiledmm" / "lib" / "libtiledmm_gb300.so"
    if not lib.exists():
        subprocess.run([sys.executable, str(PKG / "build.py")], check=True)
    import tiledmm

    return tiledmm


@pytest.fixture(scope="session")
def oracle():
    from oracle_lib import load_oracle

    return load_oracle()


@pytest.fixture(scope="session")
def refhost():
    from oracle_lib import load_ref_host

    lib = load_ref_host()
    if lib is None:
        pytest.skip("reference sources not present on this machine (the reference host build is made where they are)")
    return lib
