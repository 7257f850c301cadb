"""GPU parity of the batched path (svm_run_batch): many fact pipelines over
views of one resident fact table in one persistent launch must give, query
by query, exactly the results of running each pipeline alone (which the
parity tests pin to the reference), and in EXACT mode the NumPy evaluation."""
import numpy as np
import pytest

from oracle_helpers import exact_batch_query
from shadowvm_gb300 import workloads as W
from shadowvm_gb300.pipeline import dim_pipeline, fact_pipeline
from shadowvm_gb300.proto import ValType

pytestmark = pytest.mark.gpu

SMALL = dict(fact_rows=3_000_000, min_rows=5_000, tuple_per_bulk=1_000_000, n_part=140_000,
             n_cust=300_000, n_supp=20_000)


def singles(eng, bw, idx=None):
    out = {}
    for i in (range(len(bw.queries)) if idx is None else idx):
        q = bw.queries[i]
        eng.run(q.pipe)
        out[i] = eng.result(q.pipe.id, q.key_num)
    return out


def batched(eng, bw, idx=None):
    idx = list(range(len(bw.queries))) if idx is None else idx
    eng.run_batch([bw.queries[i].pipe for i in idx])
    return {i: eng.result(bw.queries[i].pipe.id, bw.queries[i].key_num) for i in idx}


@pytest.mark.parametrize("mode", ["ref_compat", "exact"])
def test_batch_equals_one_launch_per_query(engine_factory, mode):
    bw = W.make_batch(64, qseed=11, **SMALL)
    eng = engine_factory(tuple_per_bulk=bw.fact.tuple_per_bulk, join_mode=mode, batch_policy="always")
    W.load_batch(eng, bw)
    one = singles(eng, bw)
    first = batched(eng, bw)  # builds and caches the merged probe tables
    n0 = eng.kernel_launches()
    many = batched(eng, bw)
    launches = eng.kernel_launches() - n0
    assert launches < 10, launches  # one scan kernel plus the finalize kernels
    for i in one:
        np.testing.assert_array_equal(first[i][1], many[i][1])
    nonempty = 0
    for i in one:
        np.testing.assert_array_equal(many[i][0], one[i][0], err_msg=f"keys of query {i}")
        np.testing.assert_array_equal(many[i][1], one[i][1], err_msg=f"sums of query {i}")
        nonempty += len(one[i][1]) > 0 and np.any(one[i][1] != 0)
    assert nonempty > 32


def test_batch_exact_equals_numpy(engine_factory):
    bw = W.make_batch(24, qseed=5, **SMALL)
    eng = engine_factory(tuple_per_bulk=bw.fact.tuple_per_bulk, join_mode="exact", batch_policy="always")
    W.load_batch(eng, bw)
    got = batched(eng, bw)
    fact = bw.fact.fact_host(0, bw.fact.fact_rows)
    for i in range(len(bw.queries)):
        ek, es = exact_batch_query(bw, i, fact)
        np.testing.assert_array_equal(got[i][0], ek, err_msg=f"keys of query {i}")
        np.testing.assert_array_equal(got[i][1], es, err_msg=f"sums of query {i}")


def test_batch_mixed_with_selects_and_unbatchable(engine_factory):
    """Dimension pipelines in the same batch run first; a pipeline the batch
    kernel does not take (int32 sums, a division) runs alone; empty filters
    and empty views keep their single-query results."""
    bw = W.make_batch(12, qseed=3, **SMALL)
    eng = engine_factory(tuple_per_bulk=bw.fact.tuple_per_bulk, batch_policy="always")
    W.load_batch(eng, bw, build_dims=False)
    schema = bw.fact.fact_schema()
    extra = [
        fact_pipeline("x_int32", "lo_q0", schema, ["b_date"], [("$(0.0)", "$(1.0)")], "$(1.1)", "$(0.1)",
                      metric_type=ValType.Int32),
        fact_pipeline("x_div", "lo_q1", schema, ["b_date"], [("$(0.0)", "$(1.0)")], "$(1.1)", "$(0.7)/7"),
        fact_pipeline("x_empty", "lo_q2", schema, ["b_date"], [("$(0.0)", "$(1.0)")], "$(1.1)", "$(0.7)",
                      predication="$(0.1)>60"),
        fact_pipeline("x_scalar", "lo_q3", schema, [], [], "", "$(0.7)+$(0.8)",
                      predication="$(0.2)==4"),
    ]
    # Sparse keys give a hash-layout table: that query takes the per-query
    # batch kernel beside the merged one.
    sk = np.arange(0, bw.fact.n_part, 97, dtype=np.int32)
    eng.put("sparse", [sk, (sk % 13).astype(np.int32)])
    bw.dim_pipelines.append(dim_pipeline("b_sparse", "sparse", W.int_schema(2), "$(0.0),$(0.1)", None))
    extra.append(fact_pipeline("x_hash", "lo_q4", schema, ["b_sparse"], [("$(0.4)", "$(1.0)")], "$(1.1)",
                               "$(0.7)-$(0.8)"))
    eng.view("lo_none", "lineorder", 10, 0)
    extra.append(fact_pipeline("x_none", "lo_none", schema, ["b_date"], [("$(0.0)", "$(1.0)")], "$(1.1)",
                               "$(0.7)"))
    if not any(p.id == "b_date" for p in bw.dim_pipelines):
        bw.dim_pipelines.append(dim_pipeline("b_date", "date", W.int_schema(3), "$(0.0),$(0.1)", None))
    pipes = list(bw.dim_pipelines) + [q.pipe for q in bw.queries] + extra
    eng.run_batch(pipes)
    facts = pipes[len(bw.dim_pipelines):]
    nkeys = {p.id: len([k for k in p.workflow[-2].args["dim"].split(",") if k]) for p in facts}
    got = {p.id: eng.result(p.id, nkeys[p.id]) for p in facts}
    for p in facts:
        eng.run(p)
        k, s = eng.result(p.id, nkeys[p.id])
        np.testing.assert_array_equal(got[p.id][0], k, err_msg=p.id)
        np.testing.assert_array_equal(got[p.id][1], s, err_msg=p.id)
    assert got["x_empty"][1].shape[0] == 0
    assert got["x_none"][1].shape[0] == 0
    assert got["x_scalar"][1].shape == (1, 1)


def test_batch_full_range_and_overlaps(engine_factory):
    """Queries whose ranges start and end mid-tile, coincide, nest and cover
    the whole table, including one-row views."""
    bw = W.make_batch(8, qseed=9, **SMALL)
    n = bw.fact.fact_rows
    spans = [(0, n), (0, n), (1, n - 1), (1023, 1), (1024, 1025), (n - 1, 1), (777, 3_333), (5, 2_000_000)]
    for q, (r0, ln) in zip(bw.queries, spans):
        q.row0, q.nrows = r0, ln
    eng = engine_factory(tuple_per_bulk=bw.fact.tuple_per_bulk, batch_policy="always")
    W.load_batch(eng, bw)
    one = singles(eng, bw)
    many = batched(eng, bw)
    for i in one:
        np.testing.assert_array_equal(many[i][0], one[i][0])
        np.testing.assert_array_equal(many[i][1], one[i][1])


def test_batch_larger_than_one_launch(engine_factory):
    """More queries than one merged launch keeps in shared memory: the batch
    is split over several launches with the same results."""
    bw = W.make_batch(700, qseed=21, **SMALL)
    eng = engine_factory(tuple_per_bulk=bw.fact.tuple_per_bulk, batch_policy="always")
    W.load_batch(eng, bw)
    idx = list(range(0, 700, 7))
    one = singles(eng, bw, idx)
    many = batched(eng, bw)
    for i in idx:
        np.testing.assert_array_equal(many[i][0], one[i][0], err_msg=f"keys of query {i}")
        np.testing.assert_array_equal(many[i][1], one[i][1], err_msg=f"sums of query {i}")


def test_batch_tuned_on_first_use_over_several_launches(engine_factory):
    """A batch split over several merged launches whose later launch meets a
    new batch shape (another query-count class, so the launch tuner times
    its candidates on it) keeps what the earlier launches wrote: every
    query equals its run alone."""
    bw = W.make_batch(520, qseed=31, **SMALL)
    eng = engine_factory(tuple_per_bulk=bw.fact.tuple_per_bulk, batch_policy="always", autotune=True)
    W.load_batch(eng, bw)
    one = singles(eng, bw)
    many = batched(eng, bw)
    launch = eng.last_launch()
    assert launch["kernel"] == "batch" and launch["merged_launches"] >= 2 and launch["tuned"], launch
    for i in range(len(bw.queries)):
        np.testing.assert_array_equal(many[i][0], one[i][0], err_msg=f"keys of query {i}")
        np.testing.assert_array_equal(many[i][1], one[i][1], err_msg=f"sums of query {i}")


def test_served_loop_results_equal_alone(engine_factory):
    """Requests arriving from several threads are folded into batched
    launches by the served loop; each result equals the query run alone."""
    import threading

    from shadowvm_gb300 import serving
    bw = W.make_batch(96, qseed=17, **SMALL)
    eng = engine_factory(tuple_per_bulk=bw.fact.tuple_per_bulk, batch_policy="always")
    W.load_batch(eng, bw)
    alone = singles(eng, bw)
    futs = {}
    with serving.BatchLoop(eng, fetch=True, drop_results=True) as loop:
        def client(k):
            for i in range(k, len(bw.queries), 4):
                q = bw.queries[i]
                p = fact_pipeline(f"srv{i}", f"lo_q{i}", bw.fact.fact_schema(), q.pipe.pre_pipeline_id[1:],
                                  [(o.args["lkey"], o.args["rkey"]) for o in q.pipe.workflow if "lkey" in o.args],
                                  next(o.args["dim"] for o in q.pipe.workflow if "dim" in o.args),
                                  next(o.args["metric"] for o in q.pipe.workflow if "metric" in o.args),
                                  predication=next((o.args["predication"] for o in q.pipe.workflow
                                                    if "predication" in o.args), None))
                futs[i] = loop.submit(p, q.key_num)
        ts = [threading.Thread(target=client, args=(k,)) for k in range(4)]
        for t in ts:
            t.start()
        for t in ts:
            t.join()
        got = {i: f.result(timeout=120) for i, f in futs.items()}
    assert max(loop.folds) > 1
    for i in alone:
        np.testing.assert_array_equal(got[i][0], alone[i][0], err_msg=f"keys of query {i}")
        np.testing.assert_array_equal(got[i][1], alone[i][1], err_msg=f"sums of query {i}")


def test_objects_read_matches_single_reads(engine_factory):
    from shadowvm_gb300.serving import sink_types, split_result
    bw = W.make_batch(20, qseed=23, **SMALL)
    eng = engine_factory(tuple_per_bulk=bw.fact.tuple_per_bulk, batch_policy="always")
    W.load_batch(eng, bw)
    many = batched(eng, bw)
    cols = eng.read_objects([q.pipe.id for q in bw.queries], [sink_types(q.pipe) for q in bw.queries])
    for i, q in enumerate(bw.queries):
        k, s = split_result(cols[i], q.key_num)
        np.testing.assert_array_equal(k, many[i][0])
        np.testing.assert_array_equal(s, many[i][1])


@pytest.mark.parametrize("policy", ["never", "auto"])
def test_batch_policy(engine_factory, policy):
    """NEVER runs one launch per query, AUTO picks by the cost model; the
    results are the same either way."""
    from shadowvm_gb300 import capi
    bw = W.make_batch(6, qseed=29, **SMALL)
    eng = engine_factory(tuple_per_bulk=bw.fact.tuple_per_bulk, batch_policy=policy)
    W.load_batch(eng, bw)
    one = singles(eng, bw)
    eng.profile(True)
    eng.profile_reset()
    many = batched(eng, bw)
    n_batch, _ = eng.profile_read(capi.K_BATCH)
    n_star, _ = eng.profile_read(capi.K_STAR)
    eng.profile(False)
    if policy == "never":
        assert n_batch == 0 and n_star == 6
    else:
        assert (n_batch, n_star) in ((1, 0), (0, 6))
    for i in one:
        np.testing.assert_array_equal(many[i][0], one[i][0])
        np.testing.assert_array_equal(many[i][1], one[i][1])


def test_batch_launch_variants_equal_single_launches(engine_factory):
    """The merged kernel's launch variants the tuner chooses from -- 28 or 24
    consumer warps of 32, and the ring depth -- give each query the rows it
    has alone; the tuned launch too, and it is reported."""
    bw = W.make_batch(48, qseed=43, **SMALL)
    eng = engine_factory(tuple_per_bulk=bw.fact.tuple_per_bulk, batch_policy="always", autotune=False)
    W.load_batch(eng, bw)
    one = singles(eng, bw)
    seen = set()
    for cw in (28, 24):
        for st in (2, 3):
            eng.pin_batch_launch(cw, st)
            got = batched(eng, bw)
            launch = eng.last_launch()
            assert launch["kernel"] == "batch" and launch["consumer_warps"] == cw, launch
            seen.add((cw, launch["ring_stages"]))
            for i in one:
                np.testing.assert_array_equal(got[i][0], one[i][0], err_msg=f"{cw} warps, {st} stages, query {i}")
                np.testing.assert_array_equal(got[i][1], one[i][1], err_msg=f"{cw} warps, {st} stages, query {i}")
    eng.pin_batch_launch()
    assert len(seen) >= 3
    tuned = engine_factory(tuple_per_bulk=bw.fact.tuple_per_bulk, batch_policy="always", autotune=True)
    W.load_batch(tuned, bw)
    for _ in range(2):  # tuned on the first batch, cached for the second
        got = batched(tuned, bw)
        for i in one:
            np.testing.assert_array_equal(got[i][0], one[i][0])
            np.testing.assert_array_equal(got[i][1], one[i][1])
    assert tuned.last_launch()["tuned"] is True
