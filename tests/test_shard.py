"""Multi-GPU C-block partition (tiledmm/shard.py), tested on the CPU: the blocks cover C exactly
once for every world size, and world-size-2 gloo ranks that each compute their block (with the
oracle standing in for a rank's GPU) and gather them reproduce the whole product."""
import os
import sys

import numpy as np
import pytest

from conftest import PKG, ROOT

sys.path.insert(0, str(PKG / "tiledmm"))
import shard  # noqa: E402  (pure host logic; the package __init__ needs the CUDA library)


@pytest.mark.parametrize("world", [1, 2, 3, 4, 6, 8])
@pytest.mark.parametrize("shape", [(100, 37), (5, 400), (1, 1), (64, 64)])
def test_blocks_cover_c_exactly_once(world, shape):
    m, n = shape
    cover = np.zeros((m, n), dtype=int)
    for r in range(world):
        r0, r1, c0, c1 = shard.block_of(r, world, m, n)
        cover[r0:r1, c0:c1] += 1
    assert (cover == 1).all()


def test_process_grid_follows_aspect_ratio():
    assert shard.process_grid(8, 1000, 1000) in ((2, 4), (4, 2))
    assert shard.process_grid(8, 100000, 10) == (8, 1)
    assert shard.process_grid(6, 10, 100000) == (1, 6)


def _worker(rank, world, port, q):
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT / "tests"))
    sys.path.insert(0, str(PKG / "tiledmm"))
    import shard as sh
    from oracle_lib import load_oracle, oracle_gemm

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import torch

    rng = np.random.default_rng(0)  # same inputs on every rank
    m, n, k = 45, 38, 29
    for ta, tb in (("N", "N"), ("T", "N"), ("N", "T"), ("T", "T")):
        ar, ac = (m, k) if ta == "N" else (k, m)
        br, bc = (k, n) if tb == "N" else (n, k)
        lda, ldb, ldc = ar + 2, br + 1, m + 3
        a, b, c = rng.uniform(-1, 1, lda * ac), rng.uniform(-1, 1, ldb * bc), rng.uniform(-1, 1, ldc * n)
        oracle = load_oracle()
        sp = sh.sub_problem(rank, world, ta, tb, m, n, k, lda, ldb, ldc)
        mine = c.copy()
        if sp["m"] and sp["n"]:
            oracle_gemm(oracle, ta, tb, sp["m"], sp["n"], k, 0.5, a[sp["off_a"]:].copy(), lda,
                        b[sp["off_b"]:].copy(), ldb, -1.0, view := mine[sp["off_c"]:].copy(), ldc,
                        (sp["m"], sp["n"], k))
            mine[sp["off_c"]:] = view
        # gather every rank's C (the application's exchange, not the library's)
        parts = [torch.zeros(len(mine), dtype=torch.float64) for _ in range(world)]
        dist.all_gather(parts, torch.from_numpy(mine))
        if rank == 0:
            full = c.copy()
            oracle_gemm(oracle, ta, tb, m, n, k, 0.5, a, lda, b, ldb, -1.0, full, ldc, (m, n, k))
            got = c.copy().reshape(n, ldc)
            for r in range(world):
                r0, r1, c0, c1 = sh.block_of(r, world, m, n)
                got[c0:c1, r0:r1] = parts[r].numpy().reshape(n, ldc)[c0:c1, r0:r1]
            q.put(bool(np.array_equal(got.reshape(-1), full)))
    dist.destroy_process_group()


@pytest.mark.gpu
@pytest.mark.parametrize("world", [2, 3, 4])
def test_sharded_shares_reassemble_on_one_gpu(tmm, world):
    """Every rank's share computed in turn on this GPU (the ranks never wait on one another)
    writes exactly its block; together they equal one whole call, bit for bit."""
    from tiledmm import shard as tshard

    rng = np.random.default_rng(world)
    m, n, k = 700, 530, 300
    a = rng.uniform(-1, 1, k * m)  # stored k x m: op(A) = A^T
    b = rng.uniform(-1, 1, k * n)
    c = rng.uniform(-1, 1, m * n)
    whole = c.copy()
    ctx = tmm.make_context(np.float64, 2, 256, 256, 256)
    ctx.set_tile_policy(tmm.TILE_POLICY_FIXED)
    tmm.gemm(ctx, "T", "N", m, n, k, 2.0, a, k, b, k, 0.5, whole, m)
    parts = c.copy()
    for r in range(world):
        tshard.gemm_sharded(ctx, r, world, "T", "N", m, n, k, 2.0, a, k, b, k, 0.5, parts, m)
    np.testing.assert_allclose(parts, whole, rtol=1e-13, atol=1e-13)


def test_two_gloo_ranks_assemble_the_product():
    import multiprocessing as mp
    import socket

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    results = [q.get(timeout=5) for _ in range(4)]
    assert all(results)
