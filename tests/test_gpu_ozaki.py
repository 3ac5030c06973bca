"""GPU parity of the Ozaki (emulated-FP64) path through the C ABI: bit-exact against the oracle's
restatement of the same algorithm, exact on integer inputs, and within the native path's
componentwise error bound on real-valued inputs."""
from pathlib import Path

import numpy as np
import pytest

from gpu_helpers import dense, exact_product, make_problem
from oracle_lib import dd_entries, ozaki_oracle, reference_tiles

pytestmark = pytest.mark.gpu

GOLDEN = np.load(Path(__file__).parent / "golden" / "reference_host_golden.npz")


ENGINES = ["imma", "tcgen05"]


def ozaki_ctx(tmm, slices, tiles=(4096, 4096, 4096), streams=2, engine="tcgen05"):
    ctx = tmm.make_context(np.float64, streams, *tiles)
    ctx.set_path(tmm.PATH_OZAKI, slices)
    ctx.set_ozaki_engine(engine)
    return ctx


@pytest.mark.parametrize("engine", ENGINES)
def test_exact_accumulation_at_the_pass_limit(tmm, engine):
    """Integers in [-15, 15] are one exact digit each; at k = 65536 the per-pass sums reach
    15 * 15 * 65536 < 2^24, the limit of exact FP32 accumulation: the product must be exact."""
    rng = np.random.default_rng(21)
    m, n, k = 256, 256, 65536
    a = rng.integers(-15, 16, m * k).astype(np.float64)
    b = rng.integers(-15, 16, k * n).astype(np.float64)
    a[: m * 512] = 15.0  # long runs of maximal products
    b[: 512] = 15.0
    c = np.zeros(m * n)
    ctx = ozaki_ctx(tmm, 1, (65536, 65536, 65536), 1, engine)
    tmm.gemm(ctx, "N", "N", m, n, k, 1.0, a, m, b, k, 0.0, c, m)
    A = a.reshape(k, m).T.astype(np.int64)
    B = b.reshape(n, k).T.astype(np.int64)
    want = (A @ B).astype(np.float64)
    np.testing.assert_array_equal(c.reshape(n, m).T, want)


@pytest.mark.parametrize("engine", ENGINES)
@pytest.mark.parametrize("trans", ["NN", "NT", "TN", "TT"])
@pytest.mark.parametrize("shape,tiles", [((129, 77, 200), (4096, 4096, 4096)),
                                         ((300, 260, 517), (128, 256, 128)),
                                         ((64, 1, 33), (4096, 4096, 4096)),
                                         ((700, 530, 1100), (512, 512, 1024))])
def test_bit_exact_vs_oracle(tmm, oracle, engine, trans, shape, tiles):
    m, n, k = shape
    ta, tb = trans
    rng = np.random.default_rng(abs(hash((trans, shape))) % 2**32)
    a, lda, b, ldb, c, ldc = make_problem(rng, ta, tb, m, n, k, pad=3, kind="uexp")
    slices = 7
    ctx = ozaki_ctx(tmm, slices, tiles, engine=engine)
    eng = ctx.ozaki_engine()
    out = c.copy()
    tmm.gemm(ctx, ta, tb, m, n, k, 0.75, a, lda, b, ldb, -1.25, out, ldc)
    tm, tn, tk = reference_tiles(oracle, m, n, k, tiles)
    assert ctx.get_tile_sizes() == (tm, tn, tk)
    want = ozaki_oracle(oracle, ta, tb, m, n, k, 0.75, a, lda, b, ldb, -1.25, c.copy(), ldc, slices, tk,
                        eng["k_block"], eng["pass_blocks"])
    np.testing.assert_array_equal(out, want)


@pytest.mark.parametrize("cluster", ["1", "pair", "pair7"])
@pytest.mark.parametrize("shape", [(700, 530, 1100), (1100, 300, 700), (129, 600, 257)])
def test_tcgen05_engine_forms_bit_exact(tmm, oracle, monkeypatch, cluster, shape):
    """Both engine forms -- one CTA per SM on 128 x 256 tiles, and CTA pairs issuing
    cta_group::2 MMAs on 256 x 256 tiles (a peer CTA whose rows are all padding at
    m = 129), the latter with its 6- and 7-stage rings -- give the oracle's bits."""
    monkeypatch.setenv("TMM_TC_CLUSTER", cluster[:4])
    if cluster == "pair7":
        monkeypatch.setenv("TMM_TC_PAIR_STAGES", "7")
    m, n, k = shape
    rng = np.random.default_rng(m * 7 + n)
    a, lda, b, ldb, c, ldc = make_problem(rng, "N", "T", m, n, k, pad=1, kind="uexp")
    ctx = ozaki_ctx(tmm, 6, (4096, 4096, 512), engine="tcgen05")
    out = c.copy()
    tmm.gemm(ctx, "N", "T", m, n, k, 1.0, a, lda, b, ldb, 0.5, out, ldc)
    eng = ctx.ozaki_engine()
    tk = reference_tiles(oracle, m, n, k, (4096, 4096, 512))[2]
    want = ozaki_oracle(oracle, "N", "T", m, n, k, 1.0, a, lda, b, ldb, 0.5, c.copy(), ldc, 6, tk, eng["k_block"],
                        eng["pass_blocks"])
    np.testing.assert_array_equal(out, want)


@pytest.mark.parametrize("engine", ENGINES)
@pytest.mark.parametrize("name", ["ci_small_tiles", "ci_smaller_than_tile", "beta_one", "beta_alpha", "tn", "nt",
                                  "tt", "default_tiles", "tn_short_k_tile"])
def test_reference_known_answers_exact(tmm, engine, name):
    """Integer inputs are represented exactly by one slice: the emulated product is exact."""
    p = GOLDEN[f"{name}/params"]
    m, n, k, ta, tb = int(p[0]), int(p[1]), int(p[2]), chr(p[3]), chr(p[4])
    tm, tn, tk, streams = (int(x) for x in p[5:9])
    lda, ldb, ldc = (int(x) for x in p[9:12])
    alpha, beta = (float(x) for x in GOLDEN[f"{name}/scalars"])
    a = GOLDEN[f"{name}/a"].astype(np.float64)
    b = GOLDEN[f"{name}/b"].astype(np.float64)
    c = GOLDEN[f"{name}/c"].astype(np.float64)
    ctx = ozaki_ctx(tmm, 3, (tm, tn, tk), streams, engine)
    out = c.copy()
    tmm.gemm(ctx, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, out, ldc)
    np.testing.assert_array_equal(dense(out, ldc, m, n), exact_product(ta, tb, m, n, k, alpha, a, lda, b, ldb, beta,
                                                                         c, ldc))
    if name != "tn_short_k_tile":
        np.testing.assert_array_equal(out, GOLDEN[f"{name}/c_copy_back"])


@pytest.mark.parametrize("engine", ENGINES)
@pytest.mark.parametrize("kind", ["uniform", "uexp"])
def test_error_within_native_bound(tmm, oracle, engine, kind):
    rng = np.random.default_rng(11)
    m, n, k = 256, 192, 1024
    a, lda, b, ldb, c, ldc = make_problem(rng, "N", "N", m, n, k, kind=kind)
    native = tmm.make_context(np.float64, 2, 4096, 4096, 4096)
    cn = c.copy()
    tmm.gemm(native, "N", "N", m, n, k, 1.0, a, lda, b, ldb, 0.0, cn, ldc)
    ii, jj = np.repeat(np.arange(0, m, 7), len(range(0, n, 5))), np.tile(np.arange(0, n, 5), len(range(0, m, 7)))
    ref, mag = dd_entries(oracle, "N", "N", m, n, k, 1.0, a, lda, b, ldb, 0.0, None, ldc, ii, jj)

    def metric(x):
        v = dense(x, ldc, m, n)[ii, jj].copy()
        return oracle.tmmo_error_metric(len(ii), v.ctypes.data, ref.ctypes.data, mag.ctypes.data, k)

    e_native = metric(cn)
    errs = {}
    for s in (4, 8, 11, 13, 16):
        ctx = ozaki_ctx(tmm, s, engine=engine)
        co = c.copy()
        tmm.gemm(ctx, "N", "N", m, n, k, 1.0, a, lda, b, ldb, 0.0, co, ldc)
        errs[s] = metric(co)
    assert errs[4] > errs[16]  # more slices, less error
    assert errs[16] <= max(e_native, 1e-3)  # enough slices meet the native path's bound
    assert e_native < 1.0


@pytest.mark.parametrize("engine", ENGINES)
def test_device_entry_matches_host_entry(tmm, engine):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(12)
    m, n, k = 200, 300, 400
    a, lda, b, ldb, c, ldc = make_problem(rng, "T", "N", m, n, k, kind="uexp")
    ctx = ozaki_ctx(tmm, 9, (4096, 4096, 4096), engine=engine)
    host = c.copy()
    tmm.gemm(ctx, "T", "N", m, n, k, 1.0, a, lda, b, ldb, 0.5, host, ldc)
    da, db, dc = (torch.from_numpy(x.copy()).cuda() for x in (a, b, c))
    s = torch.cuda.current_stream()
    tmm.gemm_device(ctx, "T", "N", m, n, k, 1.0, da, lda, db, ldb, 0.5, dc, ldc, stream=s.cuda_stream)
    s.synchronize()
    np.testing.assert_array_equal(dc.cpu().numpy(), host)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_device_status_after_asynchronous_calls(tmm, dtype):
    """tmm_device_status waits for the stream and reports no gave-up wait after ordinary
    device-resident calls on the tensor-core engines (FP64 on the Ozaki engine, FP32 on the
    FP32 engine); the results are the host entry's."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(13)
    m, n, k = 384, 320, 512
    a, lda, b, ldb, c, ldc = make_problem(rng, "N", "T", m, n, k, dtype=dtype)
    ctx = tmm.make_context(dtype, 2, 4096, 4096, 4096)
    if dtype == np.float64:
        ctx.set_path(tmm.PATH_OZAKI, 11)
        ctx.set_ozaki_engine("tcgen05")
    host = c.copy()
    tmm.gemm(ctx, "N", "T", m, n, k, 1.0, a, lda, b, ldb, 0.0, host, ldc)
    da, db, dc = (torch.from_numpy(x.copy()).cuda() for x in (a, b, c))
    s = torch.cuda.current_stream()
    for _ in range(3):
        tmm.gemm_device(ctx, "N", "T", m, n, k, 1.0, da, lda, db, ldb, 0.0, dc, ldc, stream=s.cuda_stream)
    assert ctx.device_status(s.cuda_stream) == 0
    np.testing.assert_array_equal(dc.cpu().numpy(), host)


@pytest.mark.parametrize("engine", ENGINES)
def test_out_of_core_ozaki_matches_in_core(tmm, engine):
    rng = np.random.default_rng(13)
    m, n, k = 512, 384, 640
    a, lda, b, ldb, c, ldc = make_problem(rng, "N", "N", m, n, k, kind="uexp")
    big = ozaki_ctx(tmm, 8, (128, 128, 128), engine=engine)
    small = ozaki_ctx(tmm, 8, (128, 128, 128), engine=engine)
    small.set_memory_limit(100 * 1024 * 1024)  # forces A/B tile eviction (the tcgen05 workspace is 37 MB/stream)
    o1, o2 = c.copy(), c.copy()
    tmm.gemm(big, "N", "N", m, n, k, 1.0, a, lda, b, ldb, 1.0, o1, ldc)
    tmm.gemm(small, "N", "N", m, n, k, 1.0, a, lda, b, ldb, 1.0, o2, ldc)
    np.testing.assert_array_equal(o1, o2)


def test_device_operands_through_tmm_gemm_ozaki(tmm, oracle):
    """Ozaki path, device pointers through the host-pointer call: the device-resident path
    (k tiles of max_tile_k over all of C), bit for bit the oracle's."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(33)
    m, n, k = 400, 300, 700
    a, lda, b, ldb, c, ldc = make_problem(rng, "N", "N", m, n, k, pad=2, kind="uexp")
    ctx = ozaki_ctx(tmm, 8, (256, 256, 512), engine="tcgen05")
    da, db, dc = (torch.from_numpy(x.copy()).cuda() for x in (a, b, c))
    tmm.gemm(ctx, "N", "N", m, n, k, 0.5, da, lda, db, ldb, 2.0, dc, ldc)
    assert ctx.stats()["h2d_bytes"] == 0
    eng = ctx.ozaki_engine()
    want = ozaki_oracle(oracle, "N", "N", m, n, k, 0.5, a, lda, b, ldb, 2.0, c.copy(), ldc, 8, 512, eng["k_block"],
                        eng["pass_blocks"])
    np.testing.assert_array_equal(dc.cpu().numpy(), want)


# ------------------------------------------------ float and complex on the engine (real embedding)
def _cplx_op(x, ld, t, rows, cols):
    """op(X) (rows x cols) of a stored column-major array, widened to float64 / complex128."""
    wide = np.complex128 if np.iscomplexobj(x) else np.float64
    x = x.astype(wide)
    if t == "N":
        return x.reshape(-1, ld).T[:rows, :cols]
    m = x.reshape(-1, ld).T[:cols, :rows].T
    return m.conj() if t == "C" else m


def complex_ozaki_expected(oracle, ta, tb, m, n, k, a, lda, b, ldb, beta, c, ldc, slices, tk, eng):
    """alpha = 1, real beta: per k tile of tk, the real Ozaki oracle on the FP64 embedding
    (float: op(A) x op(B); complex: [[Re A, -Im A], [Im A, Re A]] x [Re B; Im B]), then
    C = T + beta C (first k tile) or T + C in double, rounded to C's type after every k
    tile, as on the GPU."""
    cplx = np.iscomplexobj(c)
    A, B = _cplx_op(a, lda, ta, m, k), _cplx_op(b, ldb, tb, k, n)
    C = c.reshape(-1, ldc).T[:m, :n].copy()
    for kt, k0 in enumerate(range(0, k, tk)):
        kk = min(tk, k - k0)
        Ak, Bk = A[:, k0:k0 + kk], B[k0:k0 + kk, :]
        if cplx:
            ahat = np.block([[Ak.real, -Ak.imag], [Ak.imag, Ak.real]])
            bhat = np.vstack([Bk.real, Bk.imag])
        else:
            ahat, bhat = Ak, Bk
        me, ke = ahat.shape
        t = np.zeros(me * n)
        ozaki_oracle(oracle, "N", "N", me, n, ke, 1.0, np.asfortranarray(ahat).flatten(order="F"), me,
                     np.asfortranarray(bhat).flatten(order="F"), ke, 0.0, t, me, slices, ke, eng["k_block"],
                     eng["pass_blocks"])
        T = t.reshape(n, me).T
        tc = T[:m] + 1j * T[m:] if cplx else T
        Cw = C.astype(np.complex128 if cplx else np.float64)
        if kt == 0:
            Cw = tc + beta * Cw if beta != 0.0 else tc
        else:
            Cw = tc + Cw
        C = Cw.astype(c.dtype)
    out = c.copy().reshape(-1, ldc).T
    out[:m, :n] = C
    return out.T.flatten()


@pytest.mark.parametrize("engine", ENGINES)
@pytest.mark.parametrize("trans", ["NN", "NT", "TN", "CN", "NC", "CC"])
def test_complex_ozaki_bit_exact_vs_oracle(tmm, oracle, engine, trans):
    """Complex double through tmm_gemm on the Ozaki path (tiles 128 x 96 x 80: several C tiles
    and k tiles, conjugate transposes) equals the oracle's real Ozaki product of the same
    embedding, combined with the same roundings."""
    ta, tb = trans
    rng = np.random.default_rng(ord(ta) * 7 + ord(tb))
    m, n, k = 230, 170, 200
    a, lda, b, ldb, c, ldc = make_problem(rng, ta, tb, m, n, k, dtype=np.complex128, pad=2)
    ctx = tmm.make_context(np.complex128, 2, 128, 96, 80)
    ctx.set_tile_policy(tmm.TILE_POLICY_FIXED)
    ctx.set_path(tmm.PATH_OZAKI, 7)
    ctx.set_ozaki_engine(engine)
    out = c.copy()
    tmm.gemm(ctx, ta, tb, m, n, k, 1.0, a, lda, b, ldb, 0.5, out, ldc)
    want = complex_ozaki_expected(oracle, ta, tb, m, n, k, a, lda, b, ldb, 0.5, c, ldc, 7, 80, ctx.ozaki_engine())
    np.testing.assert_array_equal(out, want)
    assert ctx.stats()["path"] == tmm.PATH_OZAKI


def test_complex_ozaki_gaussian_integers_exact(tmm):
    """Gaussian integers with small parts are one exact digit per part: the product is exact."""
    rng = np.random.default_rng(5)
    m, n, k = 150, 120, 333
    a = (rng.integers(-9, 10, m * k) + 1j * rng.integers(-9, 10, m * k)).astype(np.complex128)
    b = (rng.integers(-9, 10, k * n) + 1j * rng.integers(-9, 10, k * n)).astype(np.complex128)
    c = (rng.integers(-9, 10, m * n) + 1j * rng.integers(-9, 10, m * n)).astype(np.complex128)
    ctx = tmm.make_context(np.complex128, 2, 4096, 4096, 4096)
    ctx.set_path(tmm.PATH_OZAKI, 2)
    out = c.copy()
    tmm.gemm(ctx, "N", "N", m, n, k, 2 - 1j, a, m, b, k, 1j, out, m)
    want = (2 - 1j) * (a.reshape(k, m).T @ b.reshape(n, k).T) + 1j * c.reshape(n, m).T
    np.testing.assert_array_equal(out.reshape(n, m).T, want)


def test_complex_ozaki_device_entry_and_accuracy(tmm):
    """Device entry equals the host entry bit for bit (one k tile each), and with 13 slices the
    result agrees with the double-precision complex product to a few ulps of its magnitude,
    for complex alpha and beta."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(6)
    m, n, k = 300, 260, 400
    a, lda, b, ldb, c, ldc = make_problem(rng, "T", "C", m, n, k, dtype=np.complex128, pad=1)
    ctx = tmm.make_context(np.complex128, 2, 4096, 4096, 4096)
    ctx.set_path(tmm.PATH_OZAKI, 13)
    alpha, beta = 0.75 - 0.25j, -0.5 + 1j
    host = c.copy()
    tmm.gemm(ctx, "T", "C", m, n, k, alpha, a, lda, b, ldb, beta, host, ldc)
    da, db, dc = (torch.from_numpy(x.copy()).cuda() for x in (a, b, c))
    s = torch.cuda.current_stream()
    tmm.gemm_device(ctx, "T", "C", m, n, k, alpha, da, lda, db, ldb, beta, dc, ldc, stream=s.cuda_stream)
    s.synchronize()
    np.testing.assert_array_equal(dc.cpu().numpy(), host)
    A, B = _cplx_op(a, lda, "T", m, k), _cplx_op(b, ldb, "C", k, n)
    want = alpha * (A @ B) + beta * c.reshape(-1, ldc).T[:m, :n]
    got = host.reshape(-1, ldc).T[:m, :n]
    scale = np.abs(A).max() * np.abs(B).max() * k
    assert np.abs(got - want).max() <= 1e-14 * scale


@pytest.mark.parametrize("engine", ENGINES)
@pytest.mark.parametrize("dtype,trans", [(np.float32, "NN"), (np.float32, "NT"), (np.float32, "TN"),
                                         (np.float32, "TT"), (np.complex64, "NN"), (np.complex64, "CN"),
                                         (np.complex64, "NC"), (np.complex64, "TC")])
def test_float_ozaki_bit_exact_vs_oracle(tmm, oracle, engine, dtype, trans):
    """Float and complex float through tmm_gemm on the Ozaki path (several C tiles and k tiles)
    equal the oracle's real Ozaki product of the FP64 embedding, combined in double and rounded
    to the context's type after every k tile."""
    ta, tb = trans
    rng = np.random.default_rng(ord(ta) * 11 + ord(tb) + np.dtype(dtype).itemsize)
    m, n, k = 230, 170, 200
    a, lda, b, ldb, c, ldc = make_problem(rng, ta, tb, m, n, k, dtype=dtype, pad=2)
    ctx = tmm.make_context(dtype, 2, 128, 96, 80)
    ctx.set_tile_policy(tmm.TILE_POLICY_FIXED)
    ctx.set_path(tmm.PATH_OZAKI, 5)
    ctx.set_ozaki_engine(engine)
    out = c.copy()
    tmm.gemm(ctx, ta, tb, m, n, k, 1.0, a, lda, b, ldb, 0.5, out, ldc)
    want = complex_ozaki_expected(oracle, ta, tb, m, n, k, a, lda, b, ldb, 0.5, c, ldc, 5, 80, ctx.ozaki_engine())
    np.testing.assert_array_equal(out, want)
    st = ctx.stats()
    assert st["path"] == tmm.PATH_OZAKI and st["ozaki_slices"] == 5


@pytest.mark.parametrize("dtype", [np.float32, np.complex64])
def test_float_ozaki_default_slices_beat_native(tmm, dtype):
    """With the float default (6 slices) the Ozaki path's componentwise error is below the
    native FP32 path's on the same problem and within a few units of FP32 rounding;
    general alpha and beta; the device entry equals the host entry bit for bit."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(17)
    m, n, k = 384, 320, 3000
    ta, tb = ("T", "N") if dtype == np.float32 else ("C", "N")
    a, lda, b, ldb, c, ldc = make_problem(rng, ta, tb, m, n, k, dtype=dtype, pad=1)
    alpha, beta = (0.75, -1.25) if dtype == np.float32 else (0.75 - 0.5j, -1.25 + 0.25j)
    oz = tmm.make_context(dtype, 2, 4096, 4096, 4096)
    oz.set_path(tmm.PATH_OZAKI, 0)
    assert oz.get_path() == (tmm.PATH_OZAKI, 6)
    nat = tmm.make_context(dtype, 2, 4096, 4096, 4096)
    got_oz, got_nat = c.copy(), c.copy()
    tmm.gemm(oz, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, got_oz, ldc)
    tmm.gemm(nat, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, got_nat, ldc)
    A, B = _cplx_op(a, lda, ta, m, k), _cplx_op(b, ldb, tb, k, n)
    C0 = _cplx_op(c, ldc, "N", m, n)
    exact = alpha * (A @ B) + beta * C0
    den = abs(alpha) * (np.abs(A) @ np.abs(B)) + abs(beta) * np.abs(C0)
    if dtype == np.complex64:
        den = 2 * den  # |Re| and |Im| parts each bounded by the sum of the component magnitudes
    def err(x):
        return float(np.max(np.abs(_cplx_op(x, ldc, "N", m, n) - exact) / den))
    e_oz, e_nat = err(got_oz), err(got_nat)
    assert e_oz <= e_nat
    assert e_oz <= 4 * 2.0 ** -24
    da, db, dc = (torch.from_numpy(x.copy()).cuda() for x in (a, b, c))
    s = torch.cuda.current_stream()
    tmm.gemm_device(oz, ta, tb, m, n, k, alpha, da, lda, db, ldb, beta, dc, ldc, stream=s.cuda_stream)
    s.synchronize()
    np.testing.assert_array_equal(dc.cpu().numpy(), got_oz)


def test_ozaki_default_slices_per_type(tmm):
    for dtype, want in ((np.float32, 6), (np.complex64, 6), (np.float64, 13), (np.complex128, 13)):
        ctx = tmm.make_context(dtype, 2, 64, 64, 64)
        ctx.set_path(tmm.PATH_OZAKI, 0)
        assert ctx.get_path() == (tmm.PATH_OZAKI, want)
        ctx.set_path(tmm.PATH_OZAKI, 9)
        assert ctx.get_path() == (tmm.PATH_OZAKI, 9)
    with pytest.raises(RuntimeError):
        ctx.set_path(tmm.PATH_OZAKI, 99)




@pytest.mark.parametrize("engine", ENGINES)
@pytest.mark.parametrize("device", [False, True])
def test_nonfinite_lines_give_nan(tmm, oracle, engine, device):
    """An Inf or a NaN in a row of op(A) or a column of op(B) makes that row or column of the
    product NaN (the digit split cannot represent it); every other entry keeps the oracle's bits.
    Two k tiles: a non-finite value in the second k tile only still reaches its row."""
    rng = np.random.default_rng(77)
    m, n, k = 200, 150, 300
    a, lda, b, ldb, c, ldc = make_problem(rng, "N", "T", m, n, k, kind="uexp")
    a[3 + 10 * lda] = np.inf
    a[17 + 250 * lda] = np.nan  # second k tile (tile_k 256)
    b[5 + 7 * ldb] = -np.inf  # op(B) = B^T: column 5 of op(B) is row 5 of the stored B
    ctx = ozaki_ctx(tmm, 7, (4096, 4096, 256), engine=engine)
    eng = ctx.ozaki_engine()
    if device:
        torch = pytest.importorskip("torch")
        da, db = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
        dc = torch.from_numpy(c.copy()).cuda()
        tmm.gemm_device(ctx, "N", "T", m, n, k, 1.5, da, lda, db, ldb, 0.5, dc, ldc,
                        stream=torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        out = dc.cpu().numpy()
        tk = 256
    else:
        out = c.copy()
        tmm.gemm(ctx, "N", "T", m, n, k, 1.5, a, lda, b, ldb, 0.5, out, ldc)
        tk = reference_tiles(oracle, m, n, k, (4096, 4096, 256))[2]
    want = ozaki_oracle(oracle, "N", "T", m, n, k, 1.5, a, lda, b, ldb, 0.5, c.copy(), ldc, 7, tk, eng["k_block"],
                        eng["pass_blocks"])
    O = out.reshape(n, ldc).T[:m]
    W = want.reshape(n, ldc).T[:m]
    nan_mask = np.zeros((m, n), bool)
    nan_mask[[3, 17], :] = True
    nan_mask[:, 5] = True
    assert np.isnan(O[nan_mask]).all() and np.isnan(W[nan_mask]).all()
    assert np.isfinite(O[~nan_mask]).all()
    np.testing.assert_array_equal(O[~nan_mask], W[~nan_mask])
