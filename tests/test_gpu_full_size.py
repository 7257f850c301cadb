"""The four-dimension star query at its full size (600 M fact rows, 3 M
customers), checked through properties that hold at any size since the
oracle cannot run it in seconds:

  * the grouped sums add up to the same query's scalar sum (no GROUP BY);
  * every key lies in the filtered regions' nations and the year window;
  * the batched path (one launch for both queries) equals single launches;
  * the String-dimension variant (config 5: region / nation names, Hash
    keys) is the integer query with each nation relabelled to the Hash of
    its name -- the same seeds, rows and filters.
"""
import copy

import numpy as np
import pytest

from oracle import sql_exact
from shadowvm_gb300 import workloads as W
from shadowvm_gb300.pipeline import fact_pipeline

pytestmark = pytest.mark.gpu


def scalar_variant(w, pid):
    q = w.query
    return fact_pipeline(pid, "lineorder", w.fact_schema(), list(q.pre_pipeline_id[1:]),
                         [("$(0.0)", "$(1.0)"), ("$(0.5)", "$(2.0)"), ("$(0.6)", "$(3.0)")], "", "$(0.7)-$(0.8)")


def test_full_size_star_query_properties(engine_factory):
    w = W.make(2)
    assert w.fact_rows == 600_000_000
    eng = engine_factory(tuple_per_bulk=w.tuple_per_bulk)
    W.load_engine(eng, w)
    keys, sums = W.run_engine(eng, w)
    scalar = scalar_variant(w, "q2_total")
    eng.run(scalar)
    _, total = eng.result("q2_total", 0)
    assert int(sums.sum()) == int(total[0, 0])
    r, r2, y = w.params["c_region"], w.params["s_region"], w.params["year_lo"]
    assert 0 < len(keys) <= 75
    assert ((keys[:, 0] >= 5 * r) & (keys[:, 0] < 5 * r + 5)).all()
    assert ((keys[:, 1] >= 5 * r2) & (keys[:, 1] < 5 * r2 + 5)).all()
    assert ((keys[:, 2] >= y) & (keys[:, 2] <= y + 2)).all()
    # batched: both queries in one launch
    grouped_b, scalar_b = copy.deepcopy(w.query), scalar_variant(w, "q2_total_b")
    grouped_b.id = "q2_b"
    eng.run_batch([grouped_b, scalar_b])
    kb, sb = eng.result("q2_b", 3)
    np.testing.assert_array_equal(kb, keys)
    np.testing.assert_array_equal(sb, sums)
    assert eng.result("q2_total_b", 0)[1][0, 0] == total[0, 0]
    eng.close()  # free the 21.6 GB table before the String variant loads its own

    # the String-dimension variant: the same groups under Hash(nation name)
    w5 = W.make(5)
    assert w5.params["year_lo"] == y
    eng5 = engine_factory(tuple_per_bulk=w5.tuple_per_bulk)
    W.load_engine(eng5, w5)
    k5, s5 = W.run_engine(eng5, w5)
    relabel = {n: sql_exact.hash_value(W.nation_name(n).encode(), W.NATION_W) for n in range(25)}
    expect = np.array([[relabel[int(a)], relabel[int(b)], int(c)] for a, b, c in keys], np.int64)
    order = np.lexsort(expect.T[::-1])
    np.testing.assert_array_equal(k5, expect[order].astype(np.int32))
    np.testing.assert_array_equal(s5, sums[order])


def test_full_size_batch_mix_equals_single_launches(engine_factory):
    """The 256-query mix over the 600 M-row table: one svm_run_batch equals
    one svm_run_pipeline per query, bit for bit."""
    bw = W.make_batch(256)
    eng = engine_factory(tuple_per_bulk=bw.fact.tuple_per_bulk, batch_policy="always")
    W.load_batch(eng, bw)
    eng.run_batch([q.pipe for q in bw.queries])
    batched = {q.pipe.id: eng.result(q.pipe.id, q.key_num) for q in bw.queries}
    for q in bw.queries:
        eng.run(q.pipe)
        k, s = eng.result(q.pipe.id, q.key_num)
        np.testing.assert_array_equal(k, batched[q.pipe.id][0], err_msg=q.pipe.id)
        np.testing.assert_array_equal(s, batched[q.pipe.id][1], err_msg=q.pipe.id)


def test_full_size_text_loader_round_trip(engine_factory):
    """1 GB of SSB-like text (10 M lines of 9 fields) loads into exactly the
    values it was printed from."""
    text, cols = W.ssb_like_text(10_000_000, 9, 21)
    assert len(text) == 1_000_000_000
    eng = engine_factory()
    assert eng.load_text("big", text, [2] * 9) == 10_000_000
    for k in range(9):
        np.testing.assert_array_equal(eng.read("big", k), cols[k].astype(np.int32), err_msg=f"column {k}")
