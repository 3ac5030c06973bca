"""The benchmark configurations as parity cases at reduced sizes: each keeps its configuration's
structure (trans flags, leading-dimension padding, scalars, value distribution, stream count,
tile policy, host-buffer kind, copy mode) and checks the C ABI's result against the oracle.
The full sizes are measured by bench.py; these run in seconds."""
import numpy as np
import pytest

from oracle_lib import oracle_gemm, ozaki_oracle, reference_tiles

pytestmark = pytest.mark.gpu


def _stored(tmm, rows, cols, ld, kind, param, mat_id, pinned=None):
    x = np.zeros(ld * cols)
    tmm.fill_host(x, rows, cols, ld, kind, param, seed=3, mat_id=mat_id)
    if pinned is None:
        return x
    p = tmm.PinnedArray(x.shape)
    p.array[:] = x
    pinned.append(p)
    return p.array


def test_plain_square_pinned_copy_back(tmm, oracle):
    """m = n = k = 4096 NN, alpha = beta = 1, uniform[-1,1), tiles of half the size, 2 streams,
    page-locked buffers, C copied back; here m = n = k = 512 with tiles of 256."""
    m = n = k = 512
    keep = []
    a = _stored(tmm, m, k, m, tmm.GEN_UNIFORM, 0.0, 0, keep)
    b = _stored(tmm, k, n, k, tmm.GEN_UNIFORM, 0.0, 1, keep)
    c = _stored(tmm, m, n, m, tmm.GEN_UNIFORM, 0.0, 2, keep)
    c0 = c.copy()
    ctx = tmm.make_context(np.float64, 2, 256, 256, 256)
    tmm.gemm(ctx, "N", "N", m, n, k, 1.0, a, m, b, k, 1.0, c, m, True, True)
    want = c0.copy()
    oracle_gemm(oracle, "N", "N", m, n, k, 1.0, a, m, b, k, 1.0, want, m, (256, 256, 256))
    np.testing.assert_allclose(c, want, rtol=0, atol=4 * k * 2.0 ** -53 * np.abs(want).max())
    for p in keep:
        p.free()


def test_out_of_core_tn_padded_three_streams(tmm, oracle):
    """m = n = k = 100000 TN, leading dimensions padded by 64, alpha = 1, beta = 0.5, uniform,
    3 streams, reference tile policy from 8192 (which it turns into 6250); here m = n = k =
    1000 from 384, under a memory cap that forces tile eviction."""
    m = n = k = 1000
    pad = 64
    lda, ldb, ldc = k + pad, k + pad, m + pad
    a = _stored(tmm, k, m, lda, tmm.GEN_UNIFORM, 0.0, 0)
    b = _stored(tmm, k, n, ldb, tmm.GEN_UNIFORM, 0.0, 1)
    c = _stored(tmm, m, n, ldc, tmm.GEN_UNIFORM, 0.0, 2)
    c0 = c.copy()
    ctx = tmm.make_context(np.float64, 3, 384, 384, 384)
    ctx.set_memory_limit(14 * 384 * 384 * 8)  # 6 C slots + fewer A/B slots than the 18 tiles
    tmm.gemm(ctx, "T", "N", m, n, k, 1.0, a, lda, b, ldb, 0.5, c, ldc, True, True)
    tiles = reference_tiles(oracle, m, n, k, (384, 384, 384))
    assert ctx.get_tile_sizes() == tiles
    st = ctx.stats()
    assert st["n_streams"] == 3
    assert st["tiles_loaded"] > 18  # evicted tiles came back
    want = c0.copy()
    oracle_gemm(oracle, "T", "N", m, n, k, 1.0, a, lda, b, ldb, 0.5, want, ldc, tiles)
    np.testing.assert_allclose(c, want, rtol=0, atol=4 * k * 2.0 ** -53 * np.abs(want).max())
    pads = c.reshape(n, ldc)[:, m:]
    np.testing.assert_array_equal(pads, c0.reshape(n, ldc)[:, m:])  # padding rows untouched


@pytest.mark.parametrize("slices", [7, 13])
def test_ozaki_square_uexp(tmm, oracle, slices):
    """Ozaki FP64 m = n = k = 32768 NN, u * 2^e with e in [-20, 20]; here 640 x 576 x 1152 with
    k tiles from 512 (the reference policy makes them 384): bit for bit the oracle's Ozaki
    product; at 13 slices the componentwise
    error metric is within the native path's.  (The smallest count that meets it depends on
    k: 11 at the full size, 12 here by the oracle's own calibration.)"""
    m, n, k = 640, 576, 1152
    a = _stored(tmm, m, k, m, tmm.GEN_UEXP, 20.0, 0)
    b = _stored(tmm, k, n, k, tmm.GEN_UEXP, 20.0, 1)
    ctx = tmm.make_context(np.float64, 2, 4096, 4096, 512)
    ctx.set_path(tmm.PATH_OZAKI, slices)
    c = np.zeros(m * n)
    tmm.gemm(ctx, "N", "N", m, n, k, 1.0, a, m, b, k, 0.0, c, m, True, True)
    eng = ctx.ozaki_engine()
    tk = ctx.get_tile_sizes()[2]  # the reference policy's k tile (1152 from 512: 384)
    want = ozaki_oracle(oracle, "N", "N", m, n, k, 1.0, a, m, b, k, 0.0, np.zeros(m * n), m, slices, tk,
                        eng["k_block"], eng["pass_blocks"])
    np.testing.assert_array_equal(c, want)
    if slices == 13:
        nat = tmm.make_context(np.float64, 2, 4096, 4096, 512)
        cn = np.zeros(m * n)
        tmm.gemm(nat, "N", "N", m, n, k, 1.0, a, m, b, k, 0.0, cn, m, True, True)
        e_oz = tmm.error_metric("N", "N", m, n, k, 1.0, a, m, b, k, 0.0, None, m, c, m, n_samples=2048, seed=4)
        e_nat = tmm.error_metric("N", "N", m, n, k, 1.0, a, m, b, k, 0.0, None, m, cn, m, n_samples=2048, seed=4)
        assert e_oz <= e_nat


def test_out_of_core_ozaki_nt_pageable_no_copy_back(tmm, oracle):
    """Ozaki FP64 m = n = 65536, k = 131072 NT, alpha = -1, beta = 1, N(0,1) with row factors
    2^U[-10,10] on the stored rows of A and B, pageable buffers registered by the call, C left
    on the device (copy_c_back = false), autotuned tiles and streams; here m = n = 768,
    k = 1536, 11 slices: the device-resident C equals the oracle's Ozaki product with the
    chosen k tile bit for bit, and the caller's C is not written."""
    m, n, k = 768, 768, 1536
    a = _stored(tmm, m, k, m, tmm.GEN_NORMAL_ROWEXP, 10.0, 0)
    b = _stored(tmm, n, k, n, tmm.GEN_NORMAL_ROWEXP, 10.0, 1)
    c = _stored(tmm, m, n, m, tmm.GEN_UNIFORM, 0.0, 2)
    c0 = c.copy()
    ctx = tmm.make_context(np.float64, 2, 65536, 65536, 65536)
    ctx.set_tile_policy(tmm.TILE_POLICY_AUTOTUNE)
    ctx.set_path(tmm.PATH_OZAKI, 11)
    tmm.gemm(ctx, "N", "T", m, n, k, -1.0, a, m, b, n, 1.0, c, m, True, False)
    np.testing.assert_array_equal(c, c0)
    full = np.zeros(m * n)
    ctx.get_full_device_buffer_c().to_host(full)
    tm, tn, tk = ctx.get_tile_sizes()
    assert tk <= k and (tm, tn) == (m, n)
    eng = ctx.ozaki_engine()
    want = ozaki_oracle(oracle, "N", "T", m, n, k, -1.0, a, m, b, n, 1.0, c0.copy(), m, 11, tk, eng["k_block"],
                        eng["pass_blocks"])
    np.testing.assert_array_equal(full, want)
