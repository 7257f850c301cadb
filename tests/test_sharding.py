"""Multi-rank host logic on CPU: row shards and the merge of partial groups,
with two gloo ranks each evaluating its shard through the oracle's NumPy
evaluator; the merged result equals the whole-table result."""
import os
import socket

import numpy as np
import pytest

from shadowvm_gb300.sharding import merge_partial_groups, shard_range


def test_shard_ranges_cover_rows_once():
    for total in (0, 1, 7, 1000, 600_000_001):
        for world in (1, 2, 3, 8):
            spans = [shard_range(total, world, r) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == total
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            sizes = [e - b for b, e in spans]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_range(10, 2, 2)


def test_merge_sums_by_key():
    a = (np.array([[1, 2], [3, 4]], np.int32), np.array([[10], [20]], np.int64))
    b = (np.array([[0, 9], [3, 4]], np.int32), np.array([[5], [7]], np.int64))
    k, s = merge_partial_groups([a, b, (np.zeros((0, 2), np.int32), np.zeros((0, 1), np.int64))])
    np.testing.assert_array_equal(k, [[0, 9], [1, 2], [3, 4]])
    np.testing.assert_array_equal(s, [[5], [10], [27]])
    k, s = merge_partial_groups([(np.zeros((1, 0), np.int32), np.array([[3, 4]])),
                                 (np.zeros((1, 0), np.int32), np.array([[5, -6]]))])
    assert k.shape == (1, 0) and s.tolist() == [[8, -2]]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, config, rows, q):
    import torch.distributed as dist

    from oracle import sql_exact
    from shadowvm_gb300 import workloads as W
    from shadowvm_gb300.sharding import gather_and_merge, shard_range
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w = W.make(config, fact_rows=rows, tuple_per_bulk=100_000)
        b, e = shard_range(rows, world, rank)
        objs = {name: list(cols) for name, cols in w.dims.items()}
        for p in w.dim_pipelines:
            objs[p.id] = sql_exact.run_select(p, objs[p.pre_pipeline_id[0]])
        local = sql_exact.run_reduce(w.query, w.fact_host(b, e - b),
                                     [objs[i] for i in w.query.pre_pipeline_id[1:]])
        merged = gather_and_merge(local)
        q.put((rank, merged[0].tolist(), merged[1].tolist()))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("config", [0, 2])
def test_two_gloo_ranks_merge_to_the_whole_table_result(config):
    import multiprocessing as mp

    import oracle
    from shadowvm_gb300 import workloads as W
    rows = 200_003
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, config, rows, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=240) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    w = W.make(config, fact_rows=rows, tuple_per_bulk=100_000)
    ek, es = oracle.exact_workload(w)
    for _, k, s in got:
        np.testing.assert_array_equal(np.array(k, np.int32).reshape(ek.shape), ek)
        np.testing.assert_array_equal(np.array(s, np.int64).reshape(es.shape), es)
