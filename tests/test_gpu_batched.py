"""GPU parity of the batched persistent path (tmm_gemm_batched) through the C ABI: mixed FP64 /
FP32 problems of uneven shapes and trans flags against the oracle, CUDA-graph capture and replay
for page-locked host operands, device operands, and both autotuned FP32 tile shapes."""
import numpy as np
import pytest

from gpu_helpers import dense, make_problem, op, tol_for
from oracle_lib import oracle_gemm

pytestmark = pytest.mark.gpu


def make_batch(rng, count, pinned=None, sizes=(1, 300), kmax=300):
    probs = []
    for i in range(count):
        dt = np.float64 if i % 2 == 0 else np.float32
        m, n = (int(x) for x in rng.integers(sizes[0], sizes[1], 2))
        k = 0 if i == 5 else int(rng.integers(1, kmax))
        ta, tb = rng.choice(["N", "T", "C"]), rng.choice(["N", "T"])
        a, lda, b, ldb, c, ldc = make_problem(rng, ta, tb, m, n, k, dt, pad=int(rng.integers(0, 3)))
        if pinned is not None:
            a, b, c = (pinned(x) for x in (a, b, c))
        alpha = float(rng.uniform(-2, 2))
        beta = 0.0 if i % 3 == 0 else float(rng.uniform(-1, 1))
        probs.append(dict(trans_a=ta, trans_b=tb, m=m, n=n, k=k, alpha=alpha, a=a, ld_a=lda, b=b, ld_b=ldb,
                          beta=beta, c=c, ld_c=ldc))
    return probs


def expected(oracle, p, c0):
    dt = p["a"].dtype
    want = c0.copy()
    k = p["k"]
    tiles = (max(p["m"], 1), max(p["n"], 1), max(k, 1))
    if k == 0:
        want_v = dense(want, p["ld_c"], p["m"], p["n"])
        want_v[:] = p["beta"] * want_v if p["beta"] != 0 else 0
        return want
    oracle_gemm(oracle, p["trans_a"], p["trans_b"], p["m"], p["n"], k, dt.type(p["alpha"]), p["a"], p["ld_a"],
                p["b"], p["ld_b"], dt.type(p["beta"]), want, p["ld_c"], tiles)
    return want


def check(oracle, probs, c0s):
    for p, c0 in zip(probs, c0s):
        want = expected(oracle, p, c0)
        scale = max(1.0, float(np.abs(want).max()) if want.size else 1.0)
        np.testing.assert_allclose(p["c"], want, rtol=0, atol=tol_for(p["a"].dtype, max(p["k"], 1)) * scale * 4)


def test_mixed_batch_pageable(tmm, oracle):
    rng = np.random.default_rng(1)
    probs = make_batch(rng, 24)
    c0s = [p["c"].copy() for p in probs]
    ctx = tmm.make_context(np.float64, 2, 4096, 4096, 4096)
    tmm.gemm_batched(ctx, probs)
    assert ctx.stats()["batch_graph"] == 0  # pageable host memory: no graph
    check(oracle, probs, c0s)


def test_graph_capture_and_replay(tmm, oracle):
    rng = np.random.default_rng(2)
    keep = []

    def pinned(x):
        pa = tmm.PinnedArray(x.shape, x.dtype)
        pa.array[:] = x
        keep.append(pa)
        return pa.array

    probs = make_batch(rng, 20, pinned=pinned)
    c0s = [p["c"].copy() for p in probs]
    ctx = tmm.make_context(np.float64, 2, 4096, 4096, 4096)
    tmm.gemm_batched(ctx, probs)
    assert ctx.stats()["batch_graph"] == 1  # captured
    check(oracle, probs, c0s)
    # new data in the same buffers: the replayed graph copies it in again
    for p in probs:
        p["a"][:] = rng.uniform(-1, 1, p["a"].size)
        p["c"][:] = rng.uniform(-1, 1, p["c"].size)
    c0s = [p["c"].copy() for p in probs]
    tmm.gemm_batched(ctx, probs)
    st = ctx.stats()
    assert st["batch_graph"] == 2  # replayed
    assert st["kernels"] >= 1 and st["h2d_bytes"] > 0 and st["d2h_bytes"] > 0
    check(oracle, probs, c0s)
    for pa in keep:
        pa.free()


def test_device_operands(tmm, oracle):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(3)
    probs = make_batch(rng, 12)
    c0s = [p["c"].copy() for p in probs]
    dev = []
    for p in probs:
        d = dict(p)
        for key in ("a", "b", "c"):
            d[key] = torch.from_numpy(p[key].copy()).cuda()
        d["dtype"] = p["a"].dtype
        dev.append(d)
    ctx = tmm.make_context(np.float64, 2, 4096, 4096, 4096)
    tmm.gemm_batched(ctx, dev, device_operands=True)
    for p, d in zip(probs, dev):
        p["c"][:] = d["c"].cpu().numpy()
    check(oracle, probs, c0s)


@pytest.mark.parametrize("tile", ["64", "128"])
def test_fp32_tile_variants(tmm, oracle, monkeypatch, tile):
    """The grouped FFMA kernel's two tile shapes (TMM_F32_KERNEL=simt; by default a batch's
    FP32 problems run on the FP32 tensor-core engine)."""
    monkeypatch.setenv("TMM_F32_KERNEL", "simt")
    monkeypatch.setenv("TMM_BATCH_F32_TILE", tile)
    rng = np.random.default_rng(4)
    probs = [p for p in make_batch(rng, 16, sizes=(100, 700), kmax=500) if p["a"].dtype == np.float32]
    c0s = [p["c"].copy() for p in probs]
    ctx = tmm.make_context(np.float32, 1, 4096, 4096, 4096)
    tmm.gemm_batched(ctx, probs)
    check(oracle, probs, c0s)


def test_batch_matches_plain_path_fp64_bit_exact_on_integers(tmm):
    """Integer inputs make any correct FP64 GEMM exact: batched and plain paths agree bit for bit."""
    rng = np.random.default_rng(5)
    probs, plain = [], []
    ctx = tmm.make_context(np.float64, 2, 4096, 4096, 4096)
    for i in range(10):
        m, n, k = (int(x) for x in rng.integers(1, 400, 3))
        a, lda, b, ldb, c, ldc = make_problem(rng, "N", "T", m, n, k, np.float64, kind="int09")
        probs.append(dict(trans_a="N", trans_b="T", m=m, n=n, k=k, alpha=1.0, a=a, ld_a=lda, b=b, ld_b=ldb, beta=1.0,
                          c=c.copy(), ld_c=ldc))
        cc = c.copy()
        tmm.gemm(ctx, "N", "T", m, n, k, 1.0, a, lda, b, ldb, 1.0, cc, ldc)
        plain.append(cc)
    tmm.gemm_batched(ctx, probs)
    for p, cc in zip(probs, plain):
        np.testing.assert_array_equal(p["c"], cc)


def test_batch_rejects_complex(tmm):
    ctx = tmm.make_context(np.float64, 1, 64, 64, 64)
    a = np.zeros(4, dtype=np.complex128)
    with pytest.raises(RuntimeError, match="GPU ERROR"):
        tmm.gemm_batched(ctx, [dict(trans_a="N", trans_b="N", m=2, n=2, k=2, alpha=1.0, a=a, ld_a=2, b=a, ld_b=2,
                                    beta=0.0, c=a, ld_c=2)])


# ---------------------------------------------------------------- FP64 problems on the Ozaki path
def ozaki_expected(oracle, p, c0, slices, tk, eng):
    """The oracle's Ozaki product with k tiles of tk (what tmm_gemm_device computes).  FP32
    problems (alpha = 1): per k tile the product of the FP64 embedding, then T + beta C
    (first k tile) or T + C in double, rounded to float after every k tile."""
    from oracle_lib import ozaki_oracle

    ta = "T" if p["trans_a"] == "C" else p["trans_a"]
    tb = "T" if p["trans_b"] == "C" else p["trans_b"]
    if p["k"] == 0:
        return expected(oracle, p, c0)
    if p["a"].dtype == np.float64:
        return ozaki_oracle(oracle, ta, tb, p["m"], p["n"], p["k"], p["alpha"], p["a"], p["ld_a"], p["b"], p["ld_b"],
                            p["beta"], c0.copy(), p["ld_c"], slices, tk, eng["k_block"], eng["pass_blocks"])
    assert p["alpha"] == 1.0
    m, n, k = p["m"], p["n"], p["k"]
    A = op(p["a"].astype(np.float64), p["ld_a"], ta, m, k)
    B = op(p["b"].astype(np.float64), p["ld_b"], tb, k, n)
    beta = float(np.float32(p["beta"]))
    C = dense(c0, p["ld_c"], m, n).copy()
    for kt, k0 in enumerate(range(0, k, tk)):
        kk = min(tk, k - k0)
        t = np.zeros(m * n)
        ozaki_oracle(oracle, "N", "N", m, n, kk, 1.0, np.asfortranarray(A[:, k0:k0 + kk]).flatten(order="F"), m,
                     np.asfortranarray(B[k0:k0 + kk, :]).flatten(order="F"), kk, 0.0, t, m, slices, kk,
                     eng["k_block"], eng["pass_blocks"])
        T = t.reshape(n, m).T
        Cw = C.astype(np.float64)
        if kt == 0:
            Cw = T + beta * Cw if beta != 0.0 else T
        else:
            Cw = T + Cw
        C = Cw.astype(np.float32)
    out = c0.copy()
    dense(out, p["ld_c"], m, n)[:] = C
    return out


def ozaki_batch(rng, count, **kw):
    """make_batch with alpha = 1 on the FP32 problems (their expected values are emulated exactly)."""
    probs = make_batch(rng, count, **kw)
    for p in probs:
        if p["a"].dtype == np.float32:
            p["alpha"] = 1.0
    return probs


def check_ozaki(oracle, probs, c0s, slices, tk, eng, f32_on_engine=False, slices_f32=6):
    """FP64 problems bit for bit the oracle's Ozaki product with `slices`; FP32 problems the
    same for their FP64 embedding with `slices_f32` when they run on the engine, else as on
    the native path."""
    for p, c0 in zip(probs, c0s):
        if p["a"].dtype == np.float64 or f32_on_engine:
            s = slices if p["a"].dtype == np.float64 else slices_f32
            np.testing.assert_array_equal(p["c"], ozaki_expected(oracle, p, c0, s, tk, eng))
        else:
            check(oracle, [p], [c0])


@pytest.mark.parametrize("engine", ["tcgen05", "imma"])
def test_ozaki_batch_bit_exact(tmm, oracle, engine):
    """On an Ozaki context the batch's FP64 problems (uneven shapes, N/T/C, k == 0, several k
    tiles of max_tile_k) run on the engine -- the tcgen05 engine in one grouped launch per
    chunk and k-tile round -- and equal the oracle's Ozaki product bit for bit; FP32 problems
    stay on the grouped FP32 kernel."""
    f32_on_engine = False
    rng = np.random.default_rng(11)
    probs = ozaki_batch(rng, 24, sizes=(1, 400), kmax=400)
    c0s = [p["c"].copy() for p in probs]
    ctx = tmm.make_context(np.float64, 2, 4096, 4096, 160)
    ctx.set_path(tmm.PATH_OZAKI, 7)
    ctx.set_ozaki_engine(engine)
    tmm.gemm_batched(ctx, probs)
    st = ctx.stats()
    assert st["path"] == tmm.PATH_OZAKI and st["ozaki_slices"] == 7
    check_ozaki(oracle, probs, c0s, 7, 160, ctx.ozaki_engine(), f32_on_engine)


def test_ozaki_batch_graph_capture_replay_and_device_operands(tmm, oracle):
    """Page-locked operands: the Ozaki launches are captured with the copies and replayed on new
    data; the same batch from device operands gives the same bits."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(12)
    keep = []

    def pinned(x):
        pa = tmm.PinnedArray(x.shape, x.dtype)
        pa.array[:] = x
        keep.append(pa)
        return pa.array

    probs = ozaki_batch(rng, 20, pinned=pinned, sizes=(50, 500), kmax=600)
    ctx = tmm.make_context(np.float64, 2, 4096, 4096, 256)
    ctx.set_path(tmm.PATH_OZAKI, 8)
    eng = ctx.ozaki_engine()
    c0s = [p["c"].copy() for p in probs]
    tmm.gemm_batched(ctx, probs)
    assert ctx.stats()["batch_graph"] == 1
    check_ozaki(oracle, probs, c0s, 8, 256, eng)
    for p in probs:
        p["a"][:] = rng.uniform(-1, 1, p["a"].size)
        p["c"][:] = rng.uniform(-1, 1, p["c"].size)
    c0s = [p["c"].copy() for p in probs]
    tmm.gemm_batched(ctx, probs)
    assert ctx.stats()["batch_graph"] == 2
    check_ozaki(oracle, probs, c0s, 8, 256, eng)
    host_out = [p["c"].copy() for p in probs]
    dev = []
    for p, c0 in zip(probs, c0s):
        d = dict(p)
        d["a"], d["b"], d["c"] = (torch.from_numpy(x.copy()).cuda() for x in (p["a"], p["b"], c0))
        d["dtype"] = p["a"].dtype
        dev.append(d)
    tmm.gemm_batched(ctx, dev, device_operands=True)
    for d, h in zip(dev, host_out):
        np.testing.assert_array_equal(d["c"].cpu().numpy(), h)
    for pa in keep:
        pa.free()


def test_fp32_problems_on_the_tensor_core_engine(tmm, oracle):
    """A batch's FP32 problems (uneven shapes, N/T, k == 0 among them) run in one grouped launch
    of the FP32 tensor-core engine, FP32-accurate against the oracle, from host and from device
    operands, and the FP64 problems beside them on their own kernel."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(9)
    probs = make_batch(rng, 30, sizes=(1, 900), kmax=1500)
    c0s = [p["c"].copy() for p in probs]
    ctx = tmm.make_context(np.float64, 2, 4096, 4096, 4096)
    tmm.gemm_batched(ctx, probs)
    check(oracle, probs, c0s)
    dev = []
    for p, c0 in zip(probs, c0s):
        d = dict(p)
        d["a"], d["b"], d["c"] = (torch.from_numpy(x.copy()).cuda() for x in (p["a"], p["b"], c0))
        d["dtype"] = p["a"].dtype
        dev.append(d)
    tmm.gemm_batched(ctx, dev, device_operands=True)
    for p, d in zip(probs, dev):
        p["c"][:] = d["c"].cpu().numpy()
    check(oracle, probs, c0s)
