"""GPU parity of the native path (FP64 DMMA tile kernel, FP32/complex SIMT kernels) and of the
out-of-core pipeline, through the C ABI, against the oracle and the reference's golden vectors."""
from pathlib import Path

import numpy as np
import pytest

from gpu_helpers import dense, exact_product, make_problem, op, tol_for
from oracle_lib import oracle_gemm, reference_tiles

pytestmark = pytest.mark.gpu

GOLDEN = np.load(Path(__file__).parent / "golden" / "reference_host_golden.npz")
CASES = sorted({k.split("/")[0] for k in GOLDEN.files if "/" in k})


def run(tmm, ctx, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, pin=True, copy_c_back=True):
    tmm.gemm(ctx, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc, pin, copy_c_back)
    if copy_c_back:
        return c
    full = np.zeros(m * n, dtype=a.dtype)
    ctx.get_full_device_buffer_c().to_host(full)
    return full


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("copy_c_back", [True, False])
def test_reference_golden_bit_exact(tmm, name, copy_c_back):
    """The reference's own known-answer runs (integer inputs: every correct GEMM is bit-equal)."""
    p = GOLDEN[f"{name}/params"]
    m, n, k, ta, tb = int(p[0]), int(p[1]), int(p[2]), chr(p[3]), chr(p[4])
    tm, tn, tk, streams = (int(x) for x in p[5:9])
    lda, ldb, ldc = (int(x) for x in p[9:12])
    ref_tiles = tuple(int(x) for x in p[12:15])
    alpha, beta = (float(x) for x in GOLDEN[f"{name}/scalars"])
    a = GOLDEN[f"{name}/a"].astype(np.float64)
    b = GOLDEN[f"{name}/b"].astype(np.float64)
    c = GOLDEN[f"{name}/c"].astype(np.float64)
    ctx = tmm.make_context(np.float64, streams, tm, tn, tk)
    out = run(tmm, ctx, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c.copy(), ldc, True, copy_c_back)
    assert ctx.get_tile_sizes() == ref_tiles  # same tile policy decision as the reference
    exact = exact_product(ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc)
    if copy_c_back:
        want = GOLDEN[f"{name}/c_copy_back"] if name != "tn_short_k_tile" else None
        if want is not None:
            np.testing.assert_array_equal(out, want)
        np.testing.assert_array_equal(dense(out, ldc, m, n), exact)
    else:
        if ldc == m and name != "tn_short_k_tile":
            np.testing.assert_array_equal(out, GOLDEN[f"{name}/full_c"])
        np.testing.assert_array_equal(out.reshape(n, m).T, exact)


DTYPES = [np.float32, np.float64, np.complex64, np.complex128]


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("trans", ["NN", "NT", "TN", "TT", "CN", "NC", "CC"])
@pytest.mark.parametrize("copy_c_back", [True, False])
def test_all_types_and_transposes_vs_oracle(tmm, oracle, dtype, trans, copy_c_back):
    rng = np.random.default_rng(hash((trans, np.dtype(dtype).str)) % 2**32)
    m, n, k = 97, 75, 131
    ta, tb = trans
    a, lda, b, ldb, c, ldc = make_problem(rng, ta, tb, m, n, k, dtype, pad=0 if not copy_c_back else 5)
    if np.dtype(dtype).kind == "c":
        alpha, beta = dtype(0.5 - 1.25j), dtype(-0.75 + 0.5j)
    else:
        alpha, beta = dtype(1.5), dtype(-0.5)
    ctx = tmm.make_context(dtype, 2, 48, 40, 64)
    out = run(tmm, ctx, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c.copy(), ldc, True, copy_c_back)
    tiles = reference_tiles(oracle, m, n, k, (48, 40, 64))
    assert ctx.get_tile_sizes() == tiles
    cc = c.copy()
    _, full = oracle_gemm(oracle, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, cc, ldc, tiles, copy_c_back)
    want = cc if copy_c_back else full
    scale = np.abs(want).max()
    np.testing.assert_allclose(out, want, rtol=0, atol=tol_for(dtype, k) * max(scale, 1))


def test_beta_zero_never_reads_c(tmm):
    rng = np.random.default_rng(1)
    m, n, k = 70, 90, 50
    a, lda, b, ldb, _, ldc = make_problem(rng, "N", "N", m, n, k)
    c = np.full(ldc * n, np.nan)
    ctx = tmm.make_context(np.float64, 2, 32, 32, 32)
    run(tmm, ctx, "N", "N", m, n, k, 1.0, a, lda, b, ldb, 0.0, c, ldc)
    assert np.isfinite(c).all()
    np.testing.assert_allclose(dense(c, ldc, m, n), exact_product("N", "N", m, n, k, 1.0, a, lda, b, ldb, 0.0, c, ldc),
                               rtol=1e-13, atol=1e-13)


def test_lowercase_trans_and_k_zero(tmm):
    rng = np.random.default_rng(2)
    m, n = 20, 30
    c = rng.uniform(-1, 1, m * n)
    c0 = c.copy()
    ctx = tmm.make_context(np.float64, 2, 16, 16, 16)
    a = np.zeros(1)
    tmm.gemm(ctx, "n", "t", m, n, 0, 1.0, a, m, a, n, 2.0, c, m)
    np.testing.assert_array_equal(c, 2.0 * c0)  # k == 0: C = beta C


def test_invalid_arguments_raise(tmm):
    ctx = tmm.make_context(np.float64, 2, 16, 16, 16)
    a = np.zeros(100)
    with pytest.raises(RuntimeError, match="GPU ERROR"):
        tmm.gemm(ctx, "X", "N", 4, 4, 4, 1.0, a, 4, a, 4, 0.0, a, 4)
    with pytest.raises(RuntimeError, match="GPU ERROR"):
        tmm.gemm(ctx, "N", "N", 4, 4, 4, 1.0, a, 3, a, 4, 0.0, a, 4)  # ld_a < m
    with pytest.raises(RuntimeError, match="GPU ERROR"):
        ctx.set_tile_sizes(17, 1, 1)  # above the context's maximum (mm_handle.cpp:58-61)


@pytest.mark.parametrize("streams", [1, 2, 3, 5])
def test_stream_count_does_not_change_results(tmm, streams):
    rng = np.random.default_rng(3)
    m, n, k = 300, 260, 200
    a, lda, b, ldb, c, ldc = make_problem(rng, "T", "N", m, n, k)
    ctx1 = tmm.make_context(np.float64, 1, 64, 64, 64)
    ctxs = tmm.make_context(np.float64, streams, 64, 64, 64)
    o1 = run(tmm, ctx1, "T", "N", m, n, k, 1.0, a, lda, b, ldb, 0.5, c.copy(), ldc)
    os_ = run(tmm, ctxs, "T", "N", m, n, k, 1.0, a, lda, b, ldb, 0.5, c.copy(), ldc)
    np.testing.assert_array_equal(o1, os_)


def test_resident_operands_cross_the_link_once(tmm):
    rng = np.random.default_rng(4)
    m, n, k = 512, 384, 640
    a, lda, b, ldb, c, ldc = make_problem(rng, "N", "N", m, n, k)
    ctx = tmm.make_context(np.float64, 2, 128, 128, 128)
    run(tmm, ctx, "N", "N", m, n, k, 1.0, a, lda, b, ldb, 1.0, c.copy(), ldc)
    st = ctx.stats()
    assert st["h2d_bytes"] == 8 * (m * k + k * n + m * n)  # compulsory traffic only
    assert st["d2h_bytes"] == 8 * m * n
    assert st["tiles_loaded"] == (m // 128) * (k // 128) + (k // 128) * (n // 128)


def test_out_of_core_eviction_matches_in_core(tmm):
    rng = np.random.default_rng(5)
    m, n, k = 640, 512, 768
    a, lda, b, ldb, c, ldc = make_problem(rng, "N", "T", m, n, k)
    big = tmm.make_context(np.float64, 2, 128, 128, 128)
    small = tmm.make_context(np.float64, 2, 128, 128, 128)
    tile = 128 * 128 * 8
    small.set_memory_limit(4 * 2 * tile + 12 * tile)  # C slots + a few A/B tiles: forces eviction
    o1 = run(tmm, big, "N", "T", m, n, k, 1.0, a, lda, b, ldb, 1.0, c.copy(), ldc)
    o2 = run(tmm, small, "N", "T", m, n, k, 1.0, a, lda, b, ldb, 1.0, c.copy(), ldc)
    np.testing.assert_array_equal(o1, o2)
    assert small.stats()["tiles_loaded"] > big.stats()["tiles_loaded"]


def test_pinned_and_pageable_host_buffers(tmm):
    rng = np.random.default_rng(6)
    m, n, k = 200, 100, 150
    pa = tmm.PinnedArray((m * k,))
    pa.array[:] = rng.uniform(-1, 1, m * k)
    b = rng.uniform(-1, 1, k * n)
    c1, c2 = np.zeros(m * n), np.zeros(m * n)
    ctx = tmm.make_context(np.float64, 2, 64, 64, 64)
    run(tmm, ctx, "N", "N", m, n, k, 1.0, pa.array, m, b, k, 0.0, c1, m, pin=True)  # already registered: used as is
    run(tmm, ctx, "N", "N", m, n, k, 1.0, pa.array.copy(), m, b, k, 0.0, c2, m, pin=False)  # pageable
    np.testing.assert_array_equal(c1, c2)
    pa.free()


@pytest.mark.parametrize("ozaki", [False, True])
@pytest.mark.parametrize("copy_c_back", [True, False])
def test_pageable_buffers_copied_by_kernel(tmm, monkeypatch, ozaki, copy_c_back):
    """Unregistered (pageable) host buffers with pin_host_buffers == false and TMM_DIRECT_HOST=1:
    on a GPU that reads host memory through the host page tables, A, B and C tiles move by copy
    kernels (uneven tiles, padded leading dimensions, beta != 0); the result equals the
    copy-engine path's (the default) bit for bit."""
    rng = np.random.default_rng(61)
    m, n, k = 333, 210, 275
    a, lda, b, ldb, c, ldc = make_problem(rng, "T", "N", m, n, k, pad=3)

    def call():
        ctx = tmm.make_context(np.float64, 2, 128, 96, 100)
        if ozaki:
            ctx.set_path(tmm.PATH_OZAKI, 7)
        out = run(tmm, ctx, "T", "N", m, n, k, 0.5, a, lda, b, ldb, -1.5, c.copy(), ldc, pin=False,
                  copy_c_back=copy_c_back)
        return out, ctx.stats()

    monkeypatch.setenv("TMM_DIRECT_HOST", "1")
    got, st = call()
    monkeypatch.delenv("TMM_DIRECT_HOST")
    want, st0 = call()
    np.testing.assert_array_equal(got, want)
    assert st0["direct_bytes"] == 0 and st0["direct_host"] == 0
    if st["direct_host"]:
        moved = st["h2d_bytes"] + (st["d2h_bytes"] if copy_c_back else 0)
        assert st["direct_bytes"] == moved > 0


def test_repeated_calls_are_deterministic_and_buffers_grow_only(tmm):
    rng = np.random.default_rng(7)
    ctx = tmm.make_context(np.float64, 2, 256, 256, 256)
    caps = []
    outs = []
    for (m, n, k) in [(300, 300, 300), (100, 100, 100), (300, 300, 300)]:
        a, lda, b, ldb, c, ldc = make_problem(np.random.default_rng(m), "N", "N", m, n, k)
        outs.append(run(tmm, ctx, "N", "N", m, n, k, 1.0, a, lda, b, ldb, 0.0, c, ldc, copy_c_back=False))
        caps.append(ctx.get_full_device_buffer_c().capacity())
    np.testing.assert_array_equal(outs[0], outs[2])
    assert caps[1] == caps[0] == caps[2]  # never shrinks (device_vector.hpp:93-107)


@pytest.mark.parametrize("shape", [(1000, 1000, 1000), (1234, 4567, 1357)])
def test_ctest_shapes_vs_oracle(tmm, oracle, shape):
    """tests/CMakeLists.txt:11-14 shapes (default context: 2 streams, tiles 5000), integer inputs."""
    m, n, k = shape
    rng = np.random.default_rng(8)
    a, lda, b, ldb, c, ldc = make_problem(rng, "N", "N", m, n, k, kind="int09")
    ctx = tmm.make_context(np.float64)
    out = run(tmm, ctx, "N", "N", m, n, k, 1.0, a, lda, b, ldb, 0.0, c.copy(), ldc)
    tiles = reference_tiles(oracle, m, n, k, (5000, 5000, 5000))
    cc = c.copy()
    oracle_gemm(oracle, "N", "N", m, n, k, 1.0, a, lda, b, ldb, 0.0, cc, ldc, tiles, nthreads=16)
    np.testing.assert_array_equal(out, cc)


def test_ctest_square_large_sampled(tmm):
    """10000^3 (tests/CMakeLists.txt:12) with integer inputs: exact on sampled rows."""
    m = n = k = 10000
    rng = np.random.default_rng(9)
    a = rng.integers(0, 10, m * k).astype(np.float64)
    b = rng.integers(0, 10, k * n).astype(np.float64)
    c = np.zeros(m * n)
    ctx = tmm.make_context(np.float64)
    tmm.gemm(ctx, "N", "N", m, n, k, 1.0, a, m, b, k, 0.0, c, m)
    rows = rng.integers(0, m, 16)
    A = a.reshape(k, m).T[rows].astype(np.int64)
    B = b.reshape(n, k).T.astype(np.int64)
    want = (A @ B).astype(np.float64)
    np.testing.assert_array_equal(c.reshape(n, m).T[rows], want)


def test_device_entry_matches_host_entry(tmm):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(10)
    m, n, k = 333, 222, 111
    a, lda, b, ldb, c, ldc = make_problem(rng, "N", "T", m, n, k)
    ctx = tmm.make_context(np.float64, 2, 4096, 4096, 4096)
    host = run(tmm, ctx, "N", "T", m, n, k, 0.5, a, lda, b, ldb, 2.0, c.copy(), ldc)
    da, db, dc = (torch.from_numpy(x.copy()).cuda() for x in (a, b, c))
    s = torch.cuda.current_stream()
    tmm.gemm_device(ctx, "N", "T", m, n, k, 0.5, da, lda, db, ldb, 2.0, dc, ldc, stream=s.cuda_stream)
    s.synchronize()
    np.testing.assert_array_equal(dc.cpu().numpy(), host)


def test_kernel_timing_counts_engine_launches(tmm):
    """tmm_set_kernel_timing / tmm_get_kernel_time: one event-timed interval per engine launch
    while on (native tile GEMMs here: 2 x 2 C tiles x 2 k-tiles), none while off, and no effect
    on results."""
    rng = np.random.default_rng(12)
    m, n, k = 300, 260, 200
    a, lda, b, ldb, c, ldc = make_problem(rng, "N", "N", m, n, k)
    ctx = tmm.make_context(np.float64, 2, 150, 130, 100)
    ctx.set_tile_policy(tmm.TILE_POLICY_FIXED)
    plain = run(tmm, ctx, "N", "N", m, n, k, 1.0, a, lda, b, ldb, 0.5, c.copy(), ldc)
    ctx.set_kernel_timing(True)
    timed = run(tmm, ctx, "N", "N", m, n, k, 1.0, a, lda, b, ldb, 0.5, c.copy(), ldc)
    sec, launches = ctx.kernel_time()
    assert launches == 8 and sec > 0
    # launches of two compute streams may overlap: their union is at most their sum and at
    # most the span from the first start to the last end
    busy, span = ctx.kernel_busy_time()
    assert 0 < busy <= sec * (1 + 1e-6) + 1e-6 and busy <= span * (1 + 1e-6) + 1e-6
    np.testing.assert_array_equal(timed, plain)
    ctx.set_kernel_timing(False)
    run(tmm, ctx, "N", "N", m, n, k, 1.0, a, lda, b, ldb, 0.5, c.copy(), ldc)
    assert ctx.kernel_time() == (0.0, 0)


@pytest.mark.parametrize("copy_c_back", [True, False])
def test_device_operands_through_tmm_gemm(tmm, oracle, copy_c_back):
    """tmm_gemm with device pointers (cudaPointerGetAttributes: device memory) runs on the
    device without the host link: same product as the oracle, nothing copied in or out; with
    copy_c_back == false the result lands in the full-C buffer and C is left untouched."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(31)
    m, n, k = 290, 170, 130
    a, lda, b, ldb, c, ldc = make_problem(rng, "T", "N", m, n, k, pad=3)
    want, _ = oracle_gemm(oracle, "T", "N", m, n, k, 1.5, a, lda, b, ldb, -0.5, c.copy(), ldc, (m, n, k))
    da, db, dc = (torch.from_numpy(x.copy()).cuda() for x in (a, b, c))
    ctx = tmm.make_context(np.float64, 2, 128, 128, 64)
    tmm.gemm(ctx, "T", "N", m, n, k, 1.5, da, lda, db, ldb, -0.5, dc, ldc, True, copy_c_back)
    st = ctx.stats()
    assert st["h2d_bytes"] == 0 and st["d2h_bytes"] == 0
    tol = tol_for(np.float64, k)
    if copy_c_back:
        got = dc.cpu().numpy()
    else:
        np.testing.assert_array_equal(dc.cpu().numpy(), c)
        full = np.zeros(m * n)
        ctx.get_full_device_buffer_c().to_host(full)
        got = c.copy()
        got.reshape(n, ldc)[:, :m] = full.reshape(n, m)
    np.testing.assert_allclose(got, want, rtol=tol, atol=tol)


def test_mixed_host_and_device_operands(tmm):
    """A in device memory, B and C in host memory: the tiled host path copies A's tiles
    device to device and gives the bits of the all-host call."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(32)
    m, n, k = 300, 220, 260
    a, lda, b, ldb, c, ldc = make_problem(rng, "N", "T", m, n, k, pad=1)
    ctx = tmm.make_context(np.float64, 2, 128, 96, 100)
    host = run(tmm, ctx, "N", "T", m, n, k, 0.75, a, lda, b, ldb, 1.25, c.copy(), ldc)
    da = torch.from_numpy(a.copy()).cuda()
    mixed = c.copy()
    tmm.gemm(ctx, "N", "T", m, n, k, 0.75, da, lda, b, ldb, 1.25, mixed, ldc)
    np.testing.assert_array_equal(mixed, host)


@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.complex64, np.complex128])
@pytest.mark.parametrize("ops", [(0, 0), (1, 2), (2, 1)])
def test_xt_entry_matches_fixed_tile_call(tmm, dtype, ops):
    """tmm_xt_?gemm (cublasXt call shape; trans as cublasOperation_t 0/1/2) equals tmm_gemm on
    a context with fixed tiles of the block dimension, bit for bit; changing the block
    dimension changes the tiles, not the product beyond rounding."""
    rng = np.random.default_rng(41)
    m, n, k = 260, 190, 230
    ta, tb = ("N", "T", "C")[ops[0]], ("N", "T", "C")[ops[1]]
    if np.dtype(dtype).kind != "c":
        ta, tb = ta.replace("C", "T"), tb.replace("C", "T")
    a, lda, b, ldb, c, ldc = make_problem(rng, ta, tb, m, n, k, dtype=dtype, pad=2)
    xt = tmm.XtHandle(block_dim=96)
    assert xt.block_dim() == 96
    got = c.copy()
    xt.gemm(dtype, ops[0], ops[1], m, n, k, 0.5, a, lda, b, ldb, 1.5, got, ldc)
    ctx = tmm.make_context(dtype, 2, 96, 96, 96)
    ctx.set_tile_policy(tmm.TILE_POLICY_FIXED)
    want = run(tmm, ctx, ta, tb, m, n, k, 0.5, a, lda, b, ldb, 1.5, c.copy(), ldc)
    np.testing.assert_array_equal(got, want)
    xt.set_block_dim(4096)
    other = c.copy()
    xt.gemm(dtype, ops[0], ops[1], m, n, k, 0.5, a, lda, b, ldb, 1.5, other, ldc)
    tol = tol_for(dtype, k)
    np.testing.assert_allclose(other, want, rtol=tol, atol=tol * np.abs(want).max())
    with pytest.raises(RuntimeError):
        xt.gemm(dtype, 7, 0, m, n, k, 0.5, a, lda, b, ldb, 1.5, other, ldc)
    xt.close()


def test_device_generator_matches_host(tmm):
    torch = pytest.importorskip("torch")
    rows, cols, ld = 257, 33, 300
    for kind, param in [(0, 0.0), (1, 0.0), (2, 20.0), (5, 16.0)]:
        h = np.zeros(ld * cols)
        tmm.fill_host(h, rows, cols, ld, kind, param, seed=5, mat_id=1)
        d = torch.zeros(ld * cols, dtype=torch.float64, device="cuda")
        tmm.fill_device(d.data_ptr(), rows, cols, ld, kind, param, seed=5, mat_id=1)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(d.cpu().numpy(), h)


@pytest.mark.parametrize("ozaki", [False, True])
def test_autotune_tile_policy(tmm, ozaki):
    """The autotuned tile policy picks memory-fitting tiles; results equal the reference policy's on
    integer inputs (exact for any tiling) and under a small memory cap (out of core)."""
    rng = np.random.default_rng(31)
    m, n, k = 1500, 1300, 2100
    a, lda, b, ldb, c, ldc = make_problem(rng, "T", "N", m, n, k, kind="int09")
    ref = tmm.make_context(np.float64, 2, 512, 512, 512)
    auto = tmm.make_context(np.float64, 2, 4096, 4096, 4096)
    auto.set_tile_policy(tmm.TILE_POLICY_AUTOTUNE)
    capped = tmm.make_context(np.float64, 2, 4096, 4096, 4096)
    capped.set_tile_policy(tmm.TILE_POLICY_AUTOTUNE)
    capped.set_memory_limit(48 * 1024 * 1024)  # below the ~156 MB the full-size tiles need
    if ozaki:
        for x in (ref, auto, capped):
            x.set_path(tmm.PATH_OZAKI, 2)
    outs = []
    for ctx in (ref, auto, capped):
        cc = c.copy()
        tmm.gemm(ctx, "T", "N", m, n, k, 1.0, a, lda, b, ldb, 1.0, cc, ldc)
        outs.append(cc)
    np.testing.assert_array_equal(outs[0], outs[1])
    np.testing.assert_array_equal(outs[0], outs[2])
    tm, tn, tk = auto.get_tile_sizes()
    assert (tm, tn) == (m, n) and tk <= k  # everything fits: one C tile
    ctm, ctn, ctk = capped.get_tile_sizes()
    assert ctm * ctn * ctk < tm * tn * tk  # the cap forces smaller tiles


def test_autotuner_times_candidates_then_keeps_the_fastest(tmm, tmp_path):
    """TMM_TILE_POLICY_AUTOTUNE: the first calls of a size class each run one untimed candidate
    (state 1), then every call uses the fastest measured one (state 2); every call computes the
    whole product (integer inputs: exact under any tiling); the report names the candidates and
    the choice, and a cache file carries the choice into a fresh process (state 3)."""
    import json
    import os
    import subprocess
    import sys

    rng = np.random.default_rng(33)
    m, n, k = 2500, 2300, 4100
    a, lda, b, ldb, c, ldc = make_problem(rng, "N", "N", m, n, k, kind="int09")
    ref = tmm.make_context(np.float64, 2, 512, 512, 512)
    exact = c.copy()
    tmm.gemm(ref, "N", "N", m, n, k, 1.0, a, lda, b, ldb, 1.0, exact, ldc)
    ctx = tmm.make_context(np.float64, 2, 4096, 4096, 4096)
    ctx.set_tile_policy(tmm.TILE_POLICY_AUTOTUNE)
    seen, states = [], []
    for _ in range(8):
        cc = c.copy()
        tmm.gemm(ctx, "N", "N", m, n, k, 1.0, a, lda, b, ldb, 1.0, cc, ldc)
        np.testing.assert_array_equal(cc, exact)
        st = ctx.stats()
        states.append(st["autotune_state"])
        seen.append((st["tile_m"], st["tile_n"], st["tile_k"]))
        if st["autotune_state"] == 2:
            break
    assert states[-1] == 2 and set(states[:-1]) == {1}, states
    explored = seen[:-1]
    assert len(set(explored)) == len(explored) >= 2, explored  # distinct candidates, each timed once
    assert seen[-1] in explored
    report = ctx.autotune_report()
    assert "(chosen)" in report and "TFLOP/s" in report, report
    ctx.close()
    ref.close()

    cache = tmp_path / "tune.txt"
    code = ("import sys, numpy as np; sys.path.insert(0, %r); import tiledmm as t;"
            "ctx = t.make_context(np.float64, 2, 4096, 4096, 4096); ctx.set_tile_policy(t.TILE_POLICY_AUTOTUNE);"
            "a = np.ones(%d); b = np.ones(%d); c = np.zeros(%d); states = []\n"
            "for _ in range(8):\n"
            "    t.gemm(ctx, 'N', 'N', %d, %d, %d, 1.0, a, %d, b, %d, 0.0, c, %d); s = ctx.stats(); states.append(s['autotune_state'])\n"
            "    if s['autotune_state'] >= 2: break\n"
            "assert c[0] == %d; print(states[-1], s['tile_m'], s['tile_n'], s['tile_k'])"
            ) % (str(tmm.LIB_PATH.parents[2]), m * k, k * n, m * n, m, n, k, m, k, m, k)
    env = dict(os.environ, TMM_AUTOTUNE_CACHE=str(cache))
    first = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=600)
    assert first.returncode == 0, first.stderr
    assert first.stdout.split()[0] == "2" and "tiles " in cache.read_text()
    second = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=600)
    assert second.returncode == 0, second.stderr
    assert second.stdout.split()[0] == "3"
    assert second.stdout.split()[1:] == first.stdout.split()[1:]  # the cached choice is the measured one


@pytest.mark.parametrize("trans", ["NN", "NT", "TN", "TT"])
@pytest.mark.parametrize("shape", [(300, 517, 1000), (129, 77, 4099), (1024, 768, 2048)])
def test_fp32_tensor_core_engine_accuracy(tmm, monkeypatch, trans, shape):
    """Float contexts multiply tiles on the tcgen05 tensor cores (three bf16 parts per FP32
    value, six exact part products, FP32 accumulation): componentwise error against the FP64
    product within 4 k 2^-24 (|alpha| |op(A)||op(B)| + |beta| |C|), and no worse than twice the
    FFMA tile kernel's (TMM_F32_KERNEL=simt) on the same inputs."""
    m, n, k = shape
    ta, tb = trans
    rng = np.random.default_rng(m + n + k)
    a, lda, b, ldb, c, ldc = make_problem(rng, ta, tb, m, n, k, dtype=np.float32, pad=3)
    A = op(a, lda, ta, m, k).astype(np.float64)
    B = op(b, ldb, tb, k, n).astype(np.float64)
    C0 = c.reshape(n, ldc).T[:m].astype(np.float64)
    alpha, beta = 1.5, -0.75
    exact = alpha * (A @ B) + beta * C0
    bound = 4 * k * 2.0 ** -24 * (abs(alpha) * (np.abs(A) @ np.abs(B)) + abs(beta) * np.abs(C0))
    errs = {}
    for kernel in ("tc", "simt"):
        if kernel == "simt":
            monkeypatch.setenv("TMM_F32_KERNEL", "simt")
        else:
            monkeypatch.delenv("TMM_F32_KERNEL", raising=False)
        ctx = tmm.make_context(np.float32, 2, 512, 512, 4096)
        out = c.copy()
        tmm.gemm(ctx, ta, tb, m, n, k, np.float32(alpha), a, lda, b, ldb, np.float32(beta), out, ldc)
        ctx.close()
        O = out.reshape(n, ldc).T[:m].astype(np.float64)
        assert (np.abs(O - exact) <= bound).all(), kernel
        errs[kernel] = float((np.abs(O - exact) / bound).max())
    assert errs["tc"] <= 2 * errs["simt"] + 1e-3, errs


def test_fp32_tensor_core_engine_nonfinite(tmm):
    """An Inf or a NaN in the FP32 engine's operands reaches the product: the rows of op(A) and
    columns of op(B) that hold one are not finite, every other entry is."""
    rng = np.random.default_rng(3)
    m, n, k = 200, 160, 300
    a, lda, b, ldb, c, ldc = make_problem(rng, "N", "N", m, n, k, dtype=np.float32)
    a[4 + 9 * lda] = np.inf
    b[20 + 7 * ldb] = np.nan  # column 7 of B
    ctx = tmm.make_context(np.float32, 2, 4096, 4096, 4096)
    out = c.copy()
    tmm.gemm(ctx, "N", "N", m, n, k, np.float32(1.0), a, lda, b, ldb, np.float32(0.0), out, ldc)
    O = out.reshape(n, ldc).T[:m]
    mask = np.zeros((m, n), bool)
    mask[4, :] = True
    mask[:, 7] = True
    assert not np.isfinite(O[mask]).any()
    assert np.isfinite(O[~mask]).all()
