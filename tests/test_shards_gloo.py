"""Multi-rank path on CPU: two gloo ranks evolve disjoint shards of the triplets
(song2_shard_items) with the oracle and all-reduce the flat source buffer; the
result equals the single-rank run.  On GPUs each rank runs
song2_ctx_create_shard on its own device with no data-path collective."""
import ctypes as C
import os

import numpy as np
import pytest


def shard(lib, p, r, w):
    n = lib.song2_shard_items(C.byref(p.spec), r, w, None)
    out = np.zeros(n, dtype=np.int64)
    lib.song2_shard_items(C.byref(p.spec), r, w, out.ctypes.data_as(C.POINTER(C.c_int64)))
    return out


def test_shards_partition_the_work(lib):
    from helpers import problem
    p = problem(k_size=4, k3_size=3)
    for w in (1, 2, 3, 5):
        parts = [shard(lib, p, r, w) for r in range(w)]
        allv = np.sort(np.concatenate(parts))
        assert np.array_equal(allv, np.arange(p.n_triplets))
        sizes = [len(x) for x in parts]
        assert max(sizes) - min(sizes) <= 1


def _rank_main(rank, world, port, q):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path[:0] = [root, os.path.join(root, "oracle"), os.path.join(root, "tests")]
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch
    import torch.distributed as dist
    from song_gb300 import capi
    import oracle
    from helpers import problem
    dist.init_process_group("gloo", rank=rank, world_size=world)
    lib = capi.load()
    p = problem()
    p.set_first_order(oracle.first_order(p, nthreads=2))
    items = shard(lib, p, rank, world)
    src, _ = oracle.evolve(p, nthreads=2, items=items)
    t = torch.from_numpy(src)
    dist.all_reduce(t)
    if rank == 0:
        full, _ = oracle.evolve(p, nthreads=2)
        q.put(float(np.max(np.abs(t.numpy() - full))))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_reproduce_single_rank(lib, olib):
    torch = pytest.importorskip("torch")
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() % 1000)
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    for pr in procs:
        pr.join(timeout=300)
    assert all(pr.exitcode == 0 for pr in procs)
    assert q.get(timeout=10) == 0.0
