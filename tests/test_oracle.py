"""The oracle pinned against the reference: tile policy, tile geometry and tiled GEMM results
must equal those of the reference's own host code (golden vectors under tests/golden/, and
the live reference host build where the reference sources are present)."""
from fractions import Fraction
from pathlib import Path

import numpy as np
import pytest

from oracle_lib import dd_entries, oracle_gemm, ozaki_oracle, ref_gemm

GOLDEN = np.load(Path(__file__).parent / "golden" / "reference_host_golden.npz")
CASES = sorted({k.split("/")[0] for k in GOLDEN.files if "/" in k})


def _case(name):
    p = GOLDEN[f"{name}/params"]
    m, n, k = int(p[0]), int(p[1]), int(p[2])
    ta, tb = chr(p[3]), chr(p[4])
    lda, ldb, ldc = int(p[9]), int(p[10]), int(p[11])
    tiles = tuple(int(x) for x in p[12:15])
    alpha, beta = (float(x) for x in GOLDEN[f"{name}/scalars"])
    a = GOLDEN[f"{name}/a"].astype(np.float64)
    b = GOLDEN[f"{name}/b"].astype(np.float64)
    c = GOLDEN[f"{name}/c"].astype(np.float64)
    return m, n, k, ta, tb, lda, ldb, ldc, tiles, alpha, beta, a, b, c


def _dense(x, ld, rows, cols):
    return x.reshape(cols, ld).T[:rows]


def test_tile_policy_matches_reference(oracle):
    for dim, cur, mx, want in GOLDEN["tile_policy"]:
        assert oracle.tmmo_optimal_tile_size(int(dim), int(cur), int(mx)) == want, (dim, cur, mx)


def test_tile_geometry_matches_reference(oracle):
    for rows, cols, ld, tr, tc, ci, cj, ntr, ntc, dr, dc, off in GOLDEN["tile_geometry"]:
        assert oracle.tmmo_num_tiles(int(rows), int(tr)) == ntr
        assert oracle.tmmo_num_tiles(int(cols), int(tc)) == ntc
        assert oracle.tmmo_tile_extent(int(rows), int(tr), int(ci)) == dr
        assert oracle.tmmo_tile_extent(int(cols), int(tc), int(cj)) == dc
        # 64-bit offset of the tile's first element (the reference's is int)
        assert ci * min(tr, rows) + cj * min(tc, cols) * ld == off


@pytest.mark.parametrize("name", [c for c in CASES if c != "tn_short_k_tile"])
@pytest.mark.parametrize("copy_c_back", [True, False])
def test_oracle_reproduces_reference_golden(oracle, name, copy_c_back):
    m, n, k, ta, tb, lda, ldb, ldc, tiles, alpha, beta, a, b, c = _case(name)
    cc = c.copy()
    _, full = oracle_gemm(oracle, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, cc, ldc, tiles, copy_c_back)
    if copy_c_back:
        np.testing.assert_array_equal(cc, GOLDEN[f"{name}/c_copy_back"])
        return
    np.testing.assert_array_equal(cc, c)  # host C untouched
    if ldc == m:
        np.testing.assert_array_equal(full, GOLDEN[f"{name}/full_c"])
    else:
        # The reference builds its device full-C view with ld_c but multiplies into it with
        # ld = m (tiled_mm.cpp:438-446, 585-587): consistent only when ld_c == m.  The oracle
        # (and the GPU path) keep the documented layout: compact m x n, ld = m.
        A = _dense(a, lda, m, k) if ta == "N" else _dense(a, lda, k, m).T
        B = _dense(b, ldb, k, n) if tb == "N" else _dense(b, ldb, n, k).T
        exact = alpha * (A @ B) + beta * _dense(c, ldc, m, n)
        np.testing.assert_array_equal(full.reshape(n, m).T, exact)
        assert not np.array_equal(GOLDEN[f"{name}/full_c"], full)


def test_reference_short_k_tile_deviation(oracle):
    """The reference's transposed-A tile k extent bug (tiled_mm.cpp:148-165) gives a wrong
    product when k has a short edge tile; the oracle (and the GPU path) compute the product."""
    m, n, k, ta, tb, lda, ldb, ldc, tiles, alpha, beta, a, b, c = _case("tn_short_k_tile")
    A = _dense(a, lda, k, m).T
    B = _dense(b, ldb, k, n)
    exact = alpha * A @ B
    ref = _dense(GOLDEN["tn_short_k_tile/c_copy_back"], ldc, m, n)
    assert np.abs(ref - exact).max() > 0  # the reference is wrong here
    cc = c.copy()
    oracle_gemm(oracle, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, cc, ldc, tiles)
    np.testing.assert_array_equal(_dense(cc, ldc, m, n), exact)


DTYPES = [np.float32, np.float64, np.complex64, np.complex128]


def _rand(rng, n, dt):
    if np.dtype(dt).kind == "c":
        return (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)).astype(dt)
    return rng.uniform(-1, 1, n).astype(dt)


@pytest.mark.parametrize("dt", DTYPES)
@pytest.mark.parametrize("trans", ["NN", "TN", "NT", "TT", "CN", "NC"])
def test_oracle_bit_exact_vs_live_reference(oracle, refhost, dt, trans):
    rng = np.random.default_rng(7)
    m, n, k = 23, 17, 24  # k tiles divide k: avoids the reference's transposed-A short-tile bug
    ta, tb = trans
    a_rows, a_cols = (m, k) if ta == "N" else (k, m)
    b_rows, b_cols = (k, n) if tb == "N" else (n, k)
    lda, ldb = a_rows + 2, b_rows + 1
    alpha = dt(0.75) if np.dtype(dt).kind != "c" else dt(0.75 - 0.25j)
    beta = dt(-0.5) if np.dtype(dt).kind != "c" else dt(-0.5 + 0.5j)
    a, b = _rand(rng, lda * a_cols, dt), _rand(rng, ldb * b_cols, dt)
    # full-C mode only where the reference is self-consistent (ld_c == m, see above)
    for copy_c_back, ldc in ((True, m + 3), (False, m)):
        c = _rand(rng, ldc * n, dt)
        c_ref, c_or = c.copy(), c.copy()
        _, f_ref, tiles = ref_gemm(refhost, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c_ref, ldc, 2, (8, 8, 8),
                                   copy_c_back)
        _, f_or = oracle_gemm(oracle, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c_or, ldc, tiles, copy_c_back)
        if copy_c_back:
            np.testing.assert_array_equal(c_or, c_ref)
        else:
            np.testing.assert_array_equal(f_or, f_ref)


def test_oracle_beta_zero_ignores_nan(oracle):
    rng = np.random.default_rng(3)
    m, n, k = 9, 7, 5
    a, b = rng.uniform(-1, 1, m * k), rng.uniform(-1, 1, k * n)
    c = np.full(m * n, np.nan)
    oracle_gemm(oracle, "N", "N", m, n, k, 1.0, a, m, b, k, 0.0, c, m, (4, 4, 4))
    np.testing.assert_allclose(c.reshape(n, m).T, a.reshape(k, m).T @ b.reshape(n, k).T, rtol=1e-14)


def test_oracle_thread_count_does_not_change_results(oracle):
    rng = np.random.default_rng(5)
    m, n, k = 40, 70, 33
    a, b, c = rng.uniform(-1, 1, m * k), rng.uniform(-1, 1, k * n), rng.uniform(-1, 1, m * n)
    c1, c8 = c.copy(), c.copy()
    oracle_gemm(oracle, "N", "N", m, n, k, 1.0, a, m, b, k, 1.0, c1, m, (16, 8, 8), nthreads=1)
    oracle_gemm(oracle, "N", "N", m, n, k, 1.0, a, m, b, k, 1.0, c8, m, (16, 8, 8), nthreads=8)
    np.testing.assert_array_equal(c1, c8)


def test_dd_entries_exact_on_small_case(oracle):
    rng = np.random.default_rng(11)
    m, n, k = 6, 5, 40
    a, b, c = rng.uniform(-1, 1, m * k), rng.uniform(-1, 1, k * n), rng.uniform(-1, 1, m * n)
    ii, jj = np.repeat(np.arange(m), n), np.tile(np.arange(n), m)
    got, mag = dd_entries(oracle, "N", "N", m, n, k, 0.5, a, m, b, k, -1.5, c, m, ii, jj)
    for t, (i, j) in enumerate(zip(ii, jj)):
        s = sum(Fraction(a[i + l * m]) * Fraction(b[l + j * k]) for l in range(k))
        exact = Fraction(0.5) * s + Fraction(-1.5) * Fraction(c[i + j * m])
        assert abs(Fraction(got[t]) - exact) <= abs(exact) * Fraction(2) ** -52 + Fraction(2) ** -1000


def test_error_metric_zero_for_exact(oracle):
    x = np.array([1.0, 2.0, 3.0])
    mag = np.array([1.0, 2.0, 0.0])
    ref = np.array([1.0, 2.0, 3.0])
    assert oracle.tmmo_error_metric(3, x.ctypes.data, ref.ctypes.data, mag.ctypes.data, 10) == 0.0


# ---------------------------------------------------------------- Ozaki restatement
def test_ozaki_split_reconstructs(oracle):
    rng = np.random.default_rng(1)
    rows, kk, s, w = 7, 50, 6, 5
    x = rng.uniform(-1, 1, rows * kk) * 2.0 ** rng.integers(-20, 21, rows * kk)
    kpad = 128
    digits = np.zeros(s * rows * kpad, dtype=np.int8)
    exps = np.zeros(rows, dtype=np.int32)
    oracle.tmmo_ozaki_split(x.ctypes.data, rows, b"N", rows, kk, kpad, s, w, digits.ctypes.data, exps.ctypes.data)
    d = digits.reshape(s, rows, kpad).astype(np.float64)
    assert np.abs(d).max() <= 16
    X = x.reshape(kk, rows).T
    for r in range(rows):
        rec = sum(d[p, r, :kk] * 2.0 ** (-4 - 5 * p) for p in range(s)) * 2.0 ** exps[r]
        rowmax = np.abs(X[r]).max()
        assert 2.0 ** (exps[r] - 1) <= rowmax < 2.0 ** exps[r]
        assert np.abs(rec - X[r]).max() <= 2.0 ** (exps[r] - 5 * s)


def test_ozaki_oracle_integer_kat_exact(oracle):
    rng = np.random.default_rng(2)
    m, n, k = 20, 13, 70
    a = rng.integers(0, 10, m * k).astype(np.float64)
    b = rng.integers(0, 10, k * n).astype(np.float64)
    c = rng.integers(0, 10, m * n).astype(np.float64)
    want = a.reshape(k, m).T @ b.reshape(n, k).T + c.reshape(n, m).T
    got = ozaki_oracle(oracle, "N", "N", m, n, k, 1.0, a, m, b, k, 1.0, c.copy(), m, slices=2, tk=32, kb=128,
                       pass_blocks=512)
    np.testing.assert_array_equal(got.reshape(n, m).T, want)


def test_ozaki_oracle_accuracy_with_enough_slices(oracle):
    rng = np.random.default_rng(4)
    m, n, k = 16, 12, 300
    a, b = rng.uniform(-1, 1, m * k), rng.uniform(-1, 1, k * n)
    c = np.zeros(m * n)
    got = ozaki_oracle(oracle, "N", "N", m, n, k, 1.0, a, m, b, k, 0.0, c, m, slices=13, tk=k, kb=128, pass_blocks=512)
    ii, jj = np.repeat(np.arange(m), n), np.tile(np.arange(n), m)
    ref, mag = dd_entries(oracle, "N", "N", m, n, k, 1.0, a, m, b, k, 0.0, None, m, ii, jj)
    vals = got.reshape(n, m).T[ii, jj].copy()
    metric = oracle.tmmo_error_metric(len(ii), vals.ctypes.data, ref.ctypes.data, mag.ctypes.data, k)
    assert metric < 0.05


def test_ozaki_complex_embedding_on_the_oracle(oracle):
    """The real embedding [[Re A, -Im A], [Im A, Re A]] x [Re B; Im B] multiplied by the real
    Ozaki restatement gives the complex product: exact on Gaussian integers of one digit."""
    rng = np.random.default_rng(8)
    m, n, k = 9, 7, 40
    A = rng.integers(-9, 10, (m, k)) + 1j * rng.integers(-9, 10, (m, k))
    B = rng.integers(-9, 10, (k, n)) + 1j * rng.integers(-9, 10, (k, n))
    ahat = np.block([[A.real, -A.imag], [A.imag, A.real]])
    bhat = np.vstack([B.real, B.imag])
    t = np.zeros(2 * m * n)
    ozaki_oracle(oracle, "N", "N", 2 * m, n, 2 * k, 1.0, ahat.flatten(order="F"), 2 * m, bhat.flatten(order="F"),
                 2 * k, 0.0, t, 2 * m, slices=2, tk=2 * k, kb=128, pass_blocks=512)
    T = t.reshape(n, 2 * m).T
    np.testing.assert_array_equal(T[:m] + 1j * T[m:], A @ B)


@pytest.mark.parametrize("dist", ["uniform", "row_exponents"])
def test_float_default_slices_beat_fp32_accumulation(oracle, dist):
    """The float contexts' default of 6 slices on the FP64 embedding of FP32 operands, rounded
    once to float, has a smaller componentwise error than an FP32-accumulating product, within
    about one FP32 rounding of the result."""
    rng = np.random.default_rng(12)
    m, n, k = 48, 40, 1024
    if dist == "uniform":
        A = rng.uniform(-1, 1, (m, k)).astype(np.float32)
        B = rng.uniform(-1, 1, (k, n)).astype(np.float32)
    else:
        A = (rng.uniform(-1, 1, (m, k)) * 2.0 ** rng.integers(-8, 9, (m, 1))).astype(np.float32)
        B = (rng.uniform(-1, 1, (k, n)) * 2.0 ** rng.integers(-8, 9, (1, n))).astype(np.float32)
    A64, B64 = A.astype(np.float64), B.astype(np.float64)
    exact = A64 @ B64
    den = np.abs(A64) @ np.abs(B64)
    acc = np.zeros((m, n), np.float32)  # FP32 accumulation in k order
    for l in range(k):
        acc += np.outer(A[:, l], B[l, :])

    def oz(slices):
        c = np.zeros(m * n)
        ozaki_oracle(oracle, "N", "N", m, n, k, 1.0, A64.flatten(order="F"), m, B64.flatten(order="F"), k, 0.0, c, m,
                     slices=slices, tk=k, kb=128, pass_blocks=512)
        return c.reshape(n, m).T.astype(np.float32).astype(np.float64)

    err = lambda X: float(np.max(np.abs(X - exact) / den))  # noqa: E731
    e_fp32, e6 = err(acc.astype(np.float64)), err(oz(6))
    assert e6 < e_fp32 / 4
    assert e6 <= 2 * 2.0 ** -24  # within about one FP32 rounding of the result


def test_ozaki_oracle_nonfinite_lines(oracle):
    """The Ozaki restatement: a row of op(A) or a column of op(B) holding an Inf or a NaN gives a
    NaN row or column of the product, and leaves every other entry as it is without them."""
    from oracle_lib import ozaki_oracle

    rng = np.random.default_rng(5)
    m, n, k = 40, 30, 50
    a = rng.uniform(-1, 1, m * k)
    b = rng.uniform(-1, 1, k * n)
    c = rng.uniform(-1, 1, m * n)
    clean = ozaki_oracle(oracle, "N", "N", m, n, k, 1.0, a, m, b, k, 1.0, c.copy(), m, 6, k, 128, 512)
    a2, b2 = a.copy(), b.copy()
    a2[7 + 3 * m] = np.inf
    b2[11 + 4 * k] = np.nan  # column 4 of B
    out = ozaki_oracle(oracle, "N", "N", m, n, k, 1.0, a2, m, b2, k, 1.0, c.copy(), m, 6, k, 128, 512)
    O, W = out.reshape(n, m).T, clean.reshape(n, m).T
    assert np.isnan(O[7, :]).all() and np.isnan(O[:, 4]).all()
    mask = np.ones((m, n), bool)
    mask[7, :] = False
    mask[:, 4] = False
    np.testing.assert_array_equal(O[mask], W[mask])
