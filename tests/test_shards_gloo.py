"""Row-range shards on the host, and the N>1 host paths over gloo on CPU.

A graph split by source-row range needs one exchange step per update (each
rank's batch partitioned by shard, the parts swapped) and an OR of the next
frontier per BFS level. Both are exercised here with world_size 2 on CPU:
each rank keeps its shard in the oracle (test-only), and the sharded results
must equal the unsharded graph's. The bench's replica aggregation (the
slowest rank's time, all ranks' units) is checked the same way."""
import os
import socket

import numpy as np
import pytest

import torch.multiprocessing as mp

from oracle.oracle import OracleGPMA

GUARD_COL = 0xFFFFFFFF
KEY_MAX = 0xFFFFFFFFFFFFFFFE


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _edges(keys):
    keys = np.asarray(keys, np.uint64)
    keys = keys[(keys != np.uint64(KEY_MAX)) & ((keys & np.uint64(GUARD_COL)) != np.uint64(GUARD_COL))]
    return (keys >> np.uint64(32)).astype(np.int64), (keys & np.uint64(GUARD_COL)).astype(np.int64)


def test_partition_rows_is_a_stable_shard_sort(built_lib):
    import gpma_bfs_gb300 as G

    rng = np.random.default_rng(3)
    for row_num, shards in ((1000, 1), (1000, 2), (1000, 3), (997, 7), (5, 9)):
        rows = rng.integers(0, row_num, 4000, dtype=np.uint64)
        keys = (rows << np.uint64(32)) | rng.integers(0, 1 << 20, 4000, dtype=np.uint64)
        vals = rng.integers(0, 2, 4000).astype(np.uint8)
        first = np.array([G.shard_first_row(row_num, shards, s) for s in range(shards + 1)], np.int64)
        assert first[0] == 0 and first[-1] == row_num and np.all(np.diff(first) >= 0)
        shard = np.searchsorted(first, rows.astype(np.int64), side="right") - 1
        order = np.argsort(shard, kind="stable")
        for rebase in (False, True):
            ok, ov, off = G.partition_rows(keys, vals, row_num, shards, rebase)
            assert np.array_equal(off, np.concatenate([[0], np.cumsum(np.bincount(shard, minlength=shards))]))
            want = keys[order]
            if rebase:
                base = first[shard[order]].astype(np.uint64) << np.uint64(32)
                want = want - base
            assert np.array_equal(ok, want) and np.array_equal(ov, vals[order])
    ok, ov, off = G.partition_rows(np.zeros(0, np.uint64), np.zeros(0, np.uint8), 10, 3)
    assert len(ok) == 0 and np.array_equal(off, np.zeros(4, np.uint64))
    with pytest.raises(G.GPMAError):
        G.partition_rows(np.array([10 << 32], np.uint64), np.ones(1, np.uint8), 10, 2)


def _shard_worker(rank, world, port):
    import torch
    import torch.distributed as dist

    import gpma_bfs_gb300 as G

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    n = 1 << 10
    src, dst = G.gen_rmat(10, 8, seed=11)
    keys = G.edges_to_keys(src, dst)
    lo, hi = G.shard_first_row(n, world, rank), G.shard_first_row(n, world, rank + 1)
    shard = OracleGPMA(hi - lo, threads=1)
    full = OracleGPMA(n, threads=1)
    batches = [(keys, np.ones(len(keys), np.uint8)), (keys[::5], np.zeros(len(keys[::5]), np.uint8))]
    for bk, bv in batches:
        full.update(bk, bv)
        # this rank's share of the batch, by position; one exchange step
        mk, mv = bk[rank::world], bv[rank::world]
        pk, pv, off = G.partition_rows(mk, mv, n, world, rebase=True)
        parts = [(pk[off[s]:off[s + 1]], pv[off[s]:off[s + 1]]) for s in range(world)]
        got = [None] * world
        dist.all_gather_object(got, parts)
        shard.update(np.concatenate([p[rank][0] for p in got]), np.concatenate([p[rank][1] for p in got]))
    # the shard's live edges are the full graph's edges of its rows
    ss, sd = _edges(shard.compact_keys())
    fs, fd = _edges(full.compact_keys())
    mine = (fs >= lo) & (fs < hi)
    assert np.array_equal(ss + lo, fs[mine]) and np.array_equal(sd, fd[mine])
    # level-synchronous BFS over the shards: expand own rows, OR the next frontier
    levels = np.zeros(n, np.uint32)
    levels[0] = 1
    frontier = np.zeros(n, bool)
    frontier[0] = True
    level = 1
    while True:
        nxt = np.zeros(n, np.uint8)
        hit = frontier[ss + lo]
        nxt[sd[hit]] = 1
        t = torch.from_numpy(nxt)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        new = t.numpy().astype(bool) & (levels == 0)
        if not new.any():
            break
        level += 1
        levels[new] = level
        frontier = new
    want, reached = full.bfs(0)
    assert np.array_equal(levels, want) and int((levels > 0).sum()) == reached
    dist.barrier()
    dist.destroy_process_group()


def test_two_row_shards_over_gloo_equal_one_graph(built_lib):
    mp.spawn(_shard_worker, args=(2, _free_port()), nprocs=2, join=True)


def _replica_worker(rank, world, port):
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    t = bench.max_over_ranks(1.5 + rank, world, device="cpu")
    assert t == 2.5
    # each rank did 1000 units; the job's rate is all units over the slowest time
    assert bench.replica_value(1000, t, world) == 2000 / 2.5
    dist.destroy_process_group()


def test_bench_replica_aggregation_over_gloo():
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    mp.spawn(_replica_worker, args=(2, _free_port()), nprocs=2, join=True)
