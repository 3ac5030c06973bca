"""bench.py's output contract, checked on the CPU through its reference arm (the oracle's CPU
restatement timed on the host cores): one JSON line with the keys the harness reads."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_json_line():
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup",
                          "3"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["n_gpus"] == 1 and d["steps"] == 1 and d["warmup"] == 3
    assert d["unit"] == "TFLOP/s" and d["higher_is_better"] is True and d["value"] > 0
    assert "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"] and cb["value"] == d["value"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    # the config is the GPU arm's, key for key (notes sit beside it), and the line's steps are the
    # samples actually timed: steps x ms_per_step fits the run's own wall time
    assert set(d["config"]) == {"workload", "m", "n", "k", "trans", "alpha", "beta", "path", "parallelism", "l2"}
    assert d["steps"] * d["ms_per_step"] / 1e3 < 600
    # the reference arm loads the oracle only, never this library
    assert "reference_note" in d


def test_reference_arm_loads_no_product_library():
    code = ("import runpy, sys; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '0'];"
            "runpy.run_path('bench.py', run_name='__main__');"
            "maps = open('/proc/self/maps').read();"
            "assert 'libtiledmm_gb300' not in maps, 'product library mapped';"
            "assert 'tiledmm' not in sys.modules")
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]


def test_numpy_generator_matches_library(tmm):
    """The CPU baselines draw their inputs from a NumPy restatement of the generator, bit for bit
    the library's for the uniform and u * 2^e kinds, including a block at an offset."""
    sys.path.insert(0, str(ROOT))
    import numpy as np

    from bench import np_generate

    rows, cols = 37, 23
    for kind, param in ((0, 0.0), (2, 20.0)):
        x = np.zeros(rows * cols)
        tmm.fill_host(x, rows, cols, rows, kind, param, seed=5, mat_id=1)
        np.testing.assert_array_equal(np_generate(kind, param, 5, 1, rows, cols), x)
        blk = np_generate(kind, param, 5, 1, 10, 6, row0=20, col0=11, full_rows=rows).reshape(10, 6, order="F")
        np.testing.assert_array_equal(blk, x.reshape(cols, rows).T[20:30, 11:17])
    # normal kind with row factors: same values to rounding
    x = np.zeros(rows * cols)
    tmm.fill_host(x, rows, cols, rows, 3, 10.0, seed=5, mat_id=0)
    np.testing.assert_allclose(np_generate(3, 10.0, 5, 0, rows, cols), x, rtol=1e-12)


def test_workloads_listed_in_help():
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--help"], capture_output=True, text=True,
                         timeout=120, cwd=ROOT)
    assert out.returncode == 0
    for name in ("ozaki32768", "batched512_ozaki", "ooc_ozaki", "sweep", "sgemm16384", "zgemm8192"):
        assert name in out.stdout
