"""Multi-GPU partition of one GEMM: C is cut into a pr x pc grid of blocks, one per rank.

C tiles are independent and the k reduction is local to a C tile, so the product
shards without any collective: rank (r, c) reads the rows of op(A) and the
columns of op(B) its block needs straight from host memory over its own host
link and writes its block of C.  Assembling C on one rank, if an application
wants that, is the application's exchange (in the reference's main user, COSMA,
the distribution lives above Tiled-MM: src/Tiled-MM/tiled_mm.cpp:492-624 is a
single-GPU call).

`block_of(rank, world, m, n)` gives a rank's block, `sub_problem(...)` the
pointer offsets and sizes of its sub-GEMM on the caller's column-major host
buffers, and `gemm_sharded(...)` runs it through tiledmm.gemm on the rank's GPU.
"""
from __future__ import annotations

import math


def process_grid(world: int, m: int = 1, n: int = 1) -> tuple[int, int]:
    """pr x pc = world, pr / pc close to m / n (square-ish blocks of C)."""
    best = (world, 1)
    best_cost = math.inf
    for pr in range(1, world + 1):
        if world % pr:
            continue
        pc = world // pr
        cost = abs(math.log(max(m, 1) / pr) - math.log(max(n, 1) / pc))
        if cost < best_cost:
            best, best_cost = (pr, pc), cost
    return best


def split(length: int, parts: int, idx: int) -> tuple[int, int]:
    """[begin, end) of part idx of length cut into `parts` nearly equal pieces."""
    return length * idx // parts, length * (idx + 1) // parts


def block_of(rank: int, world: int, m: int, n: int) -> tuple[int, int, int, int]:
    """(row0, row1, col0, col1) of the C block owned by `rank`."""
    pr, pc = process_grid(world, m, n)
    r, c = divmod(rank, pc)
    r0, r1 = split(m, pr, r)
    c0, c1 = split(n, pc, c)
    return r0, r1, c0, c1


def sub_problem(rank: int, world: int, trans_a: str, trans_b: str, m: int, n: int, k: int, lda: int, ldb: int,
                ldc: int) -> dict:
    """Element offsets into A, B, C and the sizes of the rank's sub-GEMM
    C[r0:r1, c0:c1] = alpha op(A)[r0:r1, :] op(B)[:, c0:c1] + beta C[r0:r1, c0:c1]."""
    r0, r1, c0, c1 = block_of(rank, world, m, n)
    ta, tb = trans_a.upper(), trans_b.upper()
    # rows r0.. of op(A): rows of A (N) or columns of A (T, C)
    off_a = r0 if ta == "N" else r0 * lda
    # columns c0.. of op(B): columns of B (N) or rows of B (T, C)
    off_b = c0 * ldb if tb == "N" else c0
    off_c = r0 + c0 * ldc
    return {"m": r1 - r0, "n": c1 - c0, "k": k, "off_a": off_a, "off_b": off_b, "off_c": off_c,
            "rows": (r0, r1), "cols": (c0, c1)}


def gemm_sharded(ctx, rank: int, world: int, trans_a: str, trans_b: str, m: int, n: int, k: int, alpha, a, lda: int,
                 b, ldb: int, beta, c, ldc: int, pin_host_buffers: bool = True) -> dict:
    """This rank's share of C = alpha op(A) op(B) + beta C through tiledmm.gemm (no collective).
    a, b, c are the full column-major host arrays (flat NumPy views); only the rank's block of
    c is written."""
    from . import gemm

    sp = sub_problem(rank, world, trans_a, trans_b, m, n, k, lda, ldb, ldc)
    if sp["m"] and sp["n"]:
        gemm(ctx, trans_a, trans_b, sp["m"], sp["n"], k, alpha, a[sp["off_a"]:], lda, b[sp["off_b"]:], ldb, beta,
             c[sp["off_c"]:], ldc, pin_host_buffers=pin_host_buffers, copy_c_back=True)
    return sp
