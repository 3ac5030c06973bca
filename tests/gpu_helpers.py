"""Shared helpers of the GPU parity tests: stored-matrix shapes, seeded inputs, dense views."""
from __future__ import annotations

import numpy as np


def stored_shapes(ta, tb, m, n, k):
    a_rows, a_cols = (m, k) if ta == "N" else (k, m)
    b_rows, b_cols = (k, n) if tb == "N" else (n, k)
    return (a_rows, a_cols), (b_rows, b_cols)


def rand(rng, size, dtype, kind="uniform"):
    dt = np.dtype(dtype)
    if kind == "int09":
        v = rng.integers(0, 10, size).astype(np.float64)
    elif kind == "uexp":
        v = rng.uniform(-1, 1, size) * 2.0 ** rng.integers(-20, 21, size)
    else:
        v = rng.uniform(-1, 1, size)
    if dt.kind == "c":
        w = rng.uniform(-1, 1, size) if kind != "int09" else rng.integers(0, 10, size).astype(np.float64)
        return (v + 1j * w).astype(dt)
    return v.astype(dt)


def make_problem(rng, ta, tb, m, n, k, dtype=np.float64, pad=0, kind="uniform"):
    (ar, ac), (br, bc) = stored_shapes(ta, tb, m, n, k)
    lda, ldb, ldc = max(1, ar + pad), max(1, br + pad), max(1, m + pad)
    a = rand(rng, lda * ac, dtype, kind)
    b = rand(rng, ldb * bc, dtype, kind)
    c = rand(rng, ldc * n, dtype, kind)
    return a, lda, b, ldb, c, ldc


def dense(x, ld, rows, cols):
    return x.reshape(cols, ld).T[:rows]


def op(x, ld, t, rows_op, cols_op):
    """op(X) as a dense rows_op x cols_op array from the stored column-major buffer."""
    if t == "N":
        return dense(x, ld, rows_op, cols_op)
    s = dense(x, ld, cols_op, rows_op).T
    return np.conj(s) if t == "C" else s


def exact_product(ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc):
    A = op(a, lda, ta, m, k)
    B = op(b, ldb, tb, k, n)
    C0 = dense(c, ldc, m, n)
    out = alpha * (A @ B)
    if beta != 0:
        out = out + beta * C0
    return out


def tol_for(dtype, k):
    eps = np.finfo(np.dtype(dtype).type(0).real.dtype).eps
    return 4.0 * max(k, 1) * eps
