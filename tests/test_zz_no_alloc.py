"""The allocation-free Ozaki entry point, through the C ABI.

tmm_ozaki_gemm_device_noalloc serves callers that cannot call cudaMalloc while
they run (a framework whose caching allocator owns the GPU's memory, a
latency-critical caller that cannot take cudaFree's device-wide sync): its
scratch is a fixed array inside the library.  Its result must equal the regular
device entry point's (tcgen05 engine, same slices, max_tile_k = k_tile) -- the
tolerance of the Ozaki tests, i.e. bit for bit -- on two calls in a row, which
also shows that the contents the first call leaves in the shared scratch do not
leak into the second.  This file is collected last so a run that stops at the
first failure has run every other test before it.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(tmm, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, slices, k_tile, stream):
    lib = tmm.lib()
    return lib.tmm_ozaki_gemm_device_noalloc(ta.encode(), tb.encode(), m, n, k, alpha, a.data_ptr(), lda,
                                             b.data_ptr(), ldb, beta, c.data_ptr(), ldc, slices, k_tile, stream)


def test_no_alloc_matches_regular_entry_twice(tmm):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda")
    slices, k_tile = 9, 384
    stream = torch.cuda.current_stream()
    problems = [("N", "T", 700, 530, 1100, 1.5, -0.5, 11), ("T", "N", 333, 900, 777, -1.0, 2.0, 12)]
    for ta, tb, m, n, k, alpha, beta, seed in problems:
        rng = np.random.default_rng(seed)
        a_rows, a_cols = (m, k) if ta == "N" else (k, m)
        b_rows, b_cols = (k, n) if tb == "N" else (n, k)
        lda, ldb, ldc = a_rows + 3, b_rows + 1, m + 2
        a = rng.uniform(-1, 1, lda * a_cols) * 2.0 ** rng.integers(-20, 21, lda * a_cols)
        b = rng.uniform(-1, 1, ldb * b_cols) * 2.0 ** rng.integers(-20, 21, ldb * b_cols)
        c = rng.uniform(-1, 1, ldc * n)
        da, db = torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev)
        c_ref, c_new = torch.from_numpy(c).to(dev), torch.from_numpy(c).to(dev)

        ctx = tmm.make_context(np.float64, 1, 65536, 65536, k_tile)
        ctx.set_path(tmm.PATH_OZAKI, slices)
        ctx.set_ozaki_engine("tcgen05")
        tmm.gemm_device(ctx, ta, tb, m, n, k, alpha, da, lda, db, ldb, beta, c_ref, ldc, stream=stream.cuda_stream)
        st = _noalloc(tmm, ta, tb, m, n, k, alpha, da, lda, db, ldb, beta, c_new, ldc, slices, k_tile,
                      stream.cuda_stream)
        assert st == 0, tmm.lib().tmm_last_error(None)
        # no tensor-core wait gave up on the GPU (the status call waits for the stream)
        assert tmm.lib().tmm_ozaki_noalloc_status(stream.cuda_stream) == 0, tmm.lib().tmm_last_error(None)
        np.testing.assert_array_equal(c_new.cpu().numpy(), c_ref.cpu().numpy())
        ctx.close()


def test_no_alloc_rejects_oversized_requests(tmm):
    torch = pytest.importorskip("torch")
    x = torch.zeros(16, dtype=torch.float64, device="cuda")
    lib = tmm.lib()
    # 20 slices of two 200000-line operands cannot fit even one 128-wide k step
    st = lib.tmm_ozaki_gemm_device_noalloc(b"N", b"N", 200000, 200000, 128, 1.0, x.data_ptr(), 200000, x.data_ptr(),
                                           128, 0.0, x.data_ptr(), 200000, 20, 0, None)
    assert st == 1
    assert b"scratch" in lib.tmm_last_error(None)
    # a k_tile (no larger than k) beyond what the scratch holds for 2048-line operands at 13 slices
    st = lib.tmm_ozaki_gemm_device_noalloc(b"N", b"N", 2048, 2048, 8192, 1.0, x.data_ptr(), 2048, x.data_ptr(),
                                           8192, 0.0, x.data_ptr(), 2048, 13, 8192, None)
    assert st == 1
    assert b"k_tile" in lib.tmm_last_error(None)
    # a k_tile beyond k is an upper bound, not an error: k = 128 with a huge k_tile runs
    y = torch.ones(256 * 128, dtype=torch.float64, device="cuda")
    out = torch.zeros(256 * 256, dtype=torch.float64, device="cuda")
    st = lib.tmm_ozaki_gemm_device_noalloc(b"N", b"N", 256, 256, 128, 1.0, y.data_ptr(), 256, y.data_ptr(), 128,
                                           0.0, out.data_ptr(), 256, 4, 1 << 40, None)
    assert st == 0, lib.tmm_last_error(None)
    assert lib.tmm_ozaki_noalloc_status(None) == 0
    assert torch.all(out == 128.0)  # all-ones operands: every entry of C is k
