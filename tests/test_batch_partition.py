"""The synthetic batch on the host: the library's size generator against an independent
numpy restatement, the size-balanced rank partition, and the N > 1 path as two gloo ranks on
CPU (each rank computes the same partition without a collective; the test gathers the shares
to check that they are disjoint, cover the batch and balance the flops)."""
import os
import socket

import numpy as np
import pytest

from palial_gb300 import batched as B


def sizes_numpy(count, seed):
    m1, m2, m3, k1 = (np.uint64(0x9E3779B97F4A7C15), np.uint64(0xBF58476D1CE4E5B9),
                      np.uint64(0x94D049BB133111EB), np.uint64(0xD1B54A32D192ED03))

    def mix(z):
        with np.errstate(over="ignore"):
            z = z + m1
            z = (z ^ (z >> np.uint64(30))) * m2
            z = (z ^ (z >> np.uint64(27))) * m3
            return z ^ (z >> np.uint64(31))

    with np.errstate(over="ignore"):
        key = mix(np.array([np.uint64(seed) * k1 + np.uint64(6)], dtype=np.uint64))[0]
        r = mix(key + np.arange(count, dtype=np.uint64))
    u = (r >> np.uint64(11)).astype(np.float64) * 2.0 ** -53
    return np.minimum(np.floor(32.0 * 64.0 ** u).astype(np.int64), 2047), np.arange(count) % 2


@pytest.mark.parametrize("seed", [0, 2, 7])
def test_library_sizes_equal_numpy_restatement(seed):
    ns, algs = B.batch_sizes(2000, seed)
    ns2, algs2 = sizes_numpy(2000, seed)
    assert np.array_equal(ns, ns2) and np.array_equal(algs, algs2)


def flops(ns, algs):
    ns = np.asarray(ns, dtype=np.float64)
    return np.where(np.asarray(algs) == 0, ns ** 3 / 3.0, 2.0 * ns ** 3 / 3.0)


@pytest.mark.parametrize("world", [1, 2, 3, 4, 8])
def test_partition_balanced_and_complete(world):
    ns, algs = B.batch_sizes(2000, 2)
    owner = B.partition(ns, algs, world)
    assert owner.min() >= 0 and owner.max() < world and len(owner) == 2000
    load = np.bincount(owner, weights=flops(ns, algs), minlength=world)
    # LPT: the heaviest rank carries at most the mean plus one (largest) matrix
    assert load.max() <= load.mean() + flops(ns, algs).max() + 1.0
    assert load.max() / load.mean() < 1.01
    assert np.array_equal(owner, B.partition(ns, algs, world))


def test_partition_edge_cases():
    assert len(B.partition([], [], 4)) == 0
    owner = B.partition([100, 200, 300], [0, 1, 0], 8)  # more ranks than matrices
    assert len(set(owner.tolist())) == 3


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ns, algs = B.batch_sizes(2000, 2)
        owner = B.partition(ns, algs, world)
        mine = np.nonzero(owner == rank)[0]
        load = torch.tensor([flops(ns[mine], algs[mine]).sum()], dtype=torch.float64)
        loads = [torch.zeros(1, dtype=torch.float64) for _ in range(world)]
        dist.all_gather(loads, load)
        sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
        dist.all_gather(sizes, torch.tensor([len(mine)]))
        mx = int(max(int(s) for s in sizes))
        pad = torch.full((mx,), -1, dtype=torch.int64)
        pad[:len(mine)] = torch.from_numpy(mine)
        shares = [torch.zeros(mx, dtype=torch.int64) for _ in range(world)]
        dist.all_gather(shares, pad)
        if rank == 0:
            idx = np.concatenate([s.numpy()[s.numpy() >= 0] for s in shares])
            q.put((sorted(idx.tolist()) == list(range(2000)), [float(x) for x in loads]))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_shard_without_overlap():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    cover, loads = q.get(timeout=240)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert cover
    assert max(loads) / (sum(loads) / 2) < 1.01
