"""Folds in flight (svm_batch_begin / svm_batch_wait / svm_batch_release).

A fold's batched launch is enqueued without waiting; a second fold may be
begun while the first runs.  Each fold's results -- stored as objects and
copied to the host from its staging -- must equal the queries run one launch
each, which the parity tests pin to the reference; and the served loop, with
two folds in flight, must give every request the result it has alone."""
import numpy as np
import pytest

from shadowvm_gb300 import workloads as W
from shadowvm_gb300.pipeline import dim_pipeline, fact_pipeline
from shadowvm_gb300.serving import sink_types, split_result

pytestmark = pytest.mark.gpu

SMALL = dict(fact_rows=3_000_000, min_rows=5_000, tuple_per_bulk=1_000_000, n_part=140_000,
             n_cust=300_000, n_supp=20_000)


def singles(eng, bw, idx):
    out = {}
    for i in idx:
        q = bw.queries[i]
        eng.run(q.pipe)
        out[i] = eng.result(q.pipe.id, q.key_num)
    return out


def renamed(q, pid):
    return fact_pipeline(pid, q.pipe.pre_pipeline_id[0], W.int_schema(9), q.pipe.pre_pipeline_id[1:],
                         [(o.args["lkey"], o.args["rkey"]) for o in q.pipe.workflow if "lkey" in o.args],
                         next(o.args["dim"] for o in q.pipe.workflow if "dim" in o.args),
                         next(o.args["metric"] for o in q.pipe.workflow if "metric" in o.args),
                         predication=next((o.args["predication"] for o in q.pipe.workflow
                                           if "predication" in o.args), None))


def test_two_folds_in_flight_equal_single_launches(engine_factory):
    bw = W.make_batch(80, qseed=31, **SMALL)
    eng = engine_factory(tuple_per_bulk=bw.fact.tuple_per_bulk, batch_policy="always")
    W.load_batch(eng, bw)
    alone = singles(eng, bw, range(80))
    a = [renamed(q, f"fa{i}") for i, q in enumerate(bw.queries[:40])]
    b = [renamed(q, f"fb{i}") for i, q in enumerate(bw.queries[40:])]
    fa = eng.batch_begin(a, host_results=True)
    fb = eng.batch_begin(b, host_results=True)  # begun while the first runs
    rows_a = fa.wait()
    ra = fa.release([sink_types(p) for p in a])
    rows_b = fb.wait()
    rb = fb.release([sink_types(p) for p in b])
    for j, (rows, res, pipes, off) in enumerate([(rows_a, ra, a, 0), (rows_b, rb, b, 40)]):
        for k, p in enumerate(pipes):
            i = off + k
            key_num = bw.queries[i].key_num
            hk, hs = split_result(res[k], key_num)
            np.testing.assert_array_equal(hk, alone[i][0], err_msg=f"host keys of query {i}")
            np.testing.assert_array_equal(hs, alone[i][1], err_msg=f"host sums of query {i}")
            assert rows[k] == len(alone[i][1])
            ok, os_ = eng.result(p.id, key_num)  # the stored object
            np.testing.assert_array_equal(ok, alone[i][0])
            np.testing.assert_array_equal(os_, alone[i][1])


def test_fold_takes_the_cached_or_rule_launch(engine_factory):
    """A fold never times launch configurations: on a fresh context it runs
    the rule's (reported untuned), after svm_run_batch has tuned the same
    batch shape it takes that choice; both give the queries' own results."""
    bw = W.make_batch(40, qseed=37, **SMALL)
    eng = engine_factory(tuple_per_bulk=bw.fact.tuple_per_bulk, batch_policy="always", autotune=True)
    W.load_batch(eng, bw)
    alone = singles(eng, bw, range(40))
    for round_, tuned in ((0, False), (1, True)):
        if tuned:
            eng.run_batch([renamed(q, f"warm{i}") for i, q in enumerate(bw.queries)])
        pipes = [renamed(q, f"f{round_}_{i}") for i, q in enumerate(bw.queries)]
        f = eng.batch_begin(pipes, host_results=False)
        f.wait()
        f.release()
        launch = eng.last_launch()
        assert launch["kernel"] == "batch" and launch["tuned"] == tuned, launch
        for i, p in enumerate(pipes):
            k, v = eng.result(p.id, bw.queries[i].key_num)
            np.testing.assert_array_equal(k, alone[i][0], err_msg=f"keys of query {i}")
            np.testing.assert_array_equal(v, alone[i][1], err_msg=f"sums of query {i}")


def test_fold_with_maps_unbatchable_and_empty(engine_factory):
    """Map pipelines and reduce pipelines the batch kernel does not take
    complete inside begin; their results come back with the fold's."""
    from shadowvm_gb300.proto import ValType
    bw = W.make_batch(10, qseed=3, **SMALL)
    eng = engine_factory(tuple_per_bulk=bw.fact.tuple_per_bulk, batch_policy="always")
    W.load_batch(eng, bw, build_dims=False)
    schema = bw.fact.fact_schema()
    pipes = list(bw.dim_pipelines) + [q.pipe for q in bw.queries] + [
        fact_pipeline("x_int32", "lo_q0", schema, ["b_date"], [("$(0.0)", "$(1.0)")], "$(1.1)", "$(0.1)",
                      metric_type=ValType.Int32),
        fact_pipeline("x_empty", "lo_q2", schema, ["b_date"], [("$(0.0)", "$(1.0)")], "$(1.1)", "$(0.7)",
                      predication="$(0.1)>60"),
    ]
    # dimension pipelines' outputs end in a String (hash table) column: their host copy is not taken
    f = eng.batch_begin(pipes, host_results=False)
    rows = f.wait()
    f.release()
    ref = engine_factory(tuple_per_bulk=bw.fact.tuple_per_bulk, batch_policy="never")
    W.load_batch(ref, bw, build_dims=False)
    for p in pipes:
        ref.run(p)
    for k, p in enumerate(pipes):
        if p.id.startswith("b_"):
            continue
        key_num = 1 if p.id.startswith("x_") else next(q.key_num for q in bw.queries if q.pipe.id == p.id)
        got, want = eng.result(p.id, key_num), ref.result(p.id, key_num)
        np.testing.assert_array_equal(got[0], want[0], err_msg=p.id)
        np.testing.assert_array_equal(got[1], want[1], err_msg=p.id)
        assert rows[k] == len(want[1])
    assert rows[pipes.index(next(p for p in pipes if p.id == "x_empty"))] == 0


def test_served_loop_with_folds_in_flight_equals_alone(engine_factory):
    import threading

    from shadowvm_gb300 import serving
    bw = W.make_batch(120, qseed=37, **SMALL)
    eng = engine_factory(tuple_per_bulk=bw.fact.tuple_per_bulk, batch_policy="always")
    W.load_batch(eng, bw)
    alone = singles(eng, bw, range(len(bw.queries)))
    futs = {}
    with serving.BatchLoop(eng, fetch=True, drop_results=True, inflight=2) as loop:
        def client(k):
            for i in range(k, len(bw.queries), 4):
                futs[i] = loop.submit(renamed(bw.queries[i], f"srv{i}"), bw.queries[i].key_num)
        ts = [threading.Thread(target=client, args=(k,)) for k in range(4)]
        for t in ts:
            t.start()
        for t in ts:
            t.join()
        got = {i: f.result(timeout=120) for i, f in futs.items()}
    assert len(loop.folds) > 1
    for i in alone:
        np.testing.assert_array_equal(got[i][0], alone[i][0], err_msg=f"keys of query {i}")
        np.testing.assert_array_equal(got[i][1], alone[i][1], err_msg=f"sums of query {i}")
