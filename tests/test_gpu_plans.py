"""The fused scan's launch variants all compute the reference's result.

Each golden case (the reference's own results for configs 0, 1, 2, 5 and 6
at test scale, including an empty fact table and a dimension the capped
insert drops keys from) runs under every pinned choice the tuner varies:
the kernel compiled for the plan's shape with 4 rows per consumer lane
(built for 3 or 4 blocks per SM) or 8 (for 2, predicated or in each
row-list form), or the interpreted kernel; 2 or 3 ring stages; small tables
staged in shared memory or probed in L2.  Every variant must equal the
golden rows bit for bit, and the shapes of configs 0, 1 and 2 must have a
compiled kernel (the launch reports it)."""
import json
import os

import numpy as np
import pytest

from shadowvm_gb300 import SvmError
from shadowvm_gb300 import workloads as W
from shadowvm_gb300.pipeline import dim_pipeline

pytestmark = pytest.mark.gpu

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_results.json")))
CASES = ["c0_small", "c0_q2", "c0_empty", "c1_small", "c1_q3", "c2_small", "c2_q11", "c2_drops", "c2_bulk0",
         "c5_small", "c5_q9", "c6_edges"]


def golden_rows(case, key_num):
    rows = len(case["sums"])
    keys = np.array(case["keys"], np.int32).reshape(rows, key_num)
    sums = np.array(case["sums"], np.int64).reshape(rows, -1) if rows else np.zeros((0, 1), np.int64)
    return keys, sums


@pytest.mark.parametrize("name", CASES)
def test_every_launch_variant_equals_the_reference(engine_factory, name):
    case = GOLDEN[name]
    w = W.make(case["config"], **case["kwargs"])
    if case["unfiltered_customer"]:
        w.dim_pipelines[1] = dim_pipeline("q2_cust", "customer", W.int_schema(4), "$(0.0),$(0.2)", None)
    gk, gs = golden_rows(case, w.key_num)
    eng = engine_factory(tuple_per_bulk=w.tuple_per_bulk, autotune=False)
    W.load_engine(eng, w, generate_on_device=w.fact_rows > 0)
    for p in w.dim_pipelines:
        eng.run(p)
    kernels = set()
    for rows, minb in ((4, 3), (4, 4), (8, 2), (0, 0)):
        for stages in (2, 3):
            for staged in (1, 0):
                for list_after in ((3, 0, 1, 4) if rows == 8 else (-1,)):
                    eng.pin_launch(rows, stages, staged, blocks_per_sm=minb)
                    eng.pin_list_after(list_after)
                    try:
                        eng.run(w.query)
                    except SvmError as e:
                        assert rows != 0, e  # the interpreted kernel takes every plan
                        continue
                    got = eng.result(w.query.id, w.key_num)
                    what = f"{rows} rows, {stages} stages, staged {staged}, list after {list_after}"
                    np.testing.assert_array_equal(got[0], gk, err_msg=what)
                    np.testing.assert_array_equal(got[1], gs, err_msg=what)
                    if w.fact_rows == 0:
                        continue  # no rows: nothing is launched
                    launch = eng.last_launch()
                    assert launch["ring_stages"] == stages
                    if list_after >= 0:
                        assert launch["list_after_step"] == list_after
                    kernels.add((launch["kernel"], launch["rows_per_lane"], launch["list_after_step"]))
    eng.pin_launch()
    eng.pin_list_after()
    kernels_rows = {(k, r) for k, r, _ in kernels}
    if w.fact_rows == 0:
        return
    if case["config"] in (0, 1, 2) and not case["unfiltered_customer"]:
        assert ("compiled plan", 4) in kernels_rows and ("compiled plan", 8) in kernels_rows, kernels
    if name in ("c0_small", "c2_small"):
        assert ("compiled plan", 8, 0) in kernels, kernels  # the row-list form ran
    assert ("interpreted", 4) in kernels_rows


def test_tuned_launch_equals_the_fixed_rule(engine_factory):
    """The tuner's pick (timed on first use of the shape, cached after) and the
    rule's pick give the same rows; the tuned pick is reported."""
    case = GOLDEN["c2_small"]
    w = W.make(case["config"], **case["kwargs"])
    gk, gs = golden_rows(case, w.key_num)
    for tune in (True, False):
        eng = engine_factory(tuple_per_bulk=w.tuple_per_bulk, autotune=tune)
        W.load_engine(eng, w)
        for _ in range(2):
            k, s = W.run_engine(eng, w)
            np.testing.assert_array_equal(k, gk)
            np.testing.assert_array_equal(s, gs)
        launch = eng.last_launch()
        assert launch["tuned"] == tune
        if not tune:
            assert launch["kernel"] == "compiled plan" and launch["rows_per_lane"] == 4
        eng.close()


def test_star_join_list_form_keeps_three_blocks_per_sm(engine_factory):
    """The star join's compiled row-list form (8 rows per lane, 8-bit kept
    entries, tables probed in L2) stays small enough in registers and
    shared memory for three resident blocks per SM, and equals the golden
    rows.  A change that grows the kernel past that loses a third of its
    warps and shows here before it shows in a bench."""
    case = GOLDEN["c2_small"]
    w = W.make(case["config"], **case["kwargs"])
    gk, gs = golden_rows(case, w.key_num)
    eng = engine_factory(tuple_per_bulk=w.tuple_per_bulk, autotune=False)
    W.load_engine(eng, w)
    eng.pin_launch(8, 2, 0, blocks_per_sm=2)
    eng.pin_list_after(0)
    k, s = W.run_engine(eng, w)
    np.testing.assert_array_equal(k, gk)
    np.testing.assert_array_equal(s, gs)
    launch = eng.last_launch()
    assert launch["kernel"] == "compiled plan" and launch["list_after_step"] == 0, launch
    assert launch["blocks_per_sm"] >= 3, launch
    for bad in (-2, 5):  # list_after is -1 (any), 0..2, 3 (none) or 4
        with pytest.raises(SvmError):
            eng.pin_list_after(bad)
    eng.close()


def test_query_mix_compiled_equals_interpreted(engine_factory):
    """Every query of the batched mix run alone: the compiled kernel (its
    shapes include a price range in each place the planner puts it) and the
    interpreted kernel give the same rows, and the mix's shapes all have a
    compiled kernel."""
    bw = W.make_batch(60, fact_rows=3_000_000, min_rows=5_000, tuple_per_bulk=1_000_000, n_part=140_000,
                      n_cust=300_000, n_supp=20_000, qseed=41)
    eng = engine_factory(tuple_per_bulk=bw.fact.tuple_per_bulk, autotune=False)
    W.load_batch(eng, bw)
    compiled = 0
    for q in bw.queries:
        eng.pin_launch(0)
        eng.run(q.pipe)
        want = eng.result(q.pipe.id, q.key_num)
        eng.pin_launch(-1)
        eng.run(q.pipe)
        got = eng.result(q.pipe.id, q.key_num)
        compiled += eng.last_launch()["kernel"] == "compiled plan"
        np.testing.assert_array_equal(got[0], want[0], err_msg=q.pipe.id)
        np.testing.assert_array_equal(got[1], want[1], err_msg=q.pipe.id)
    eng.pin_launch()
    assert compiled == len(bw.queries), compiled


def test_plan_cache_follows_replaced_objects(engine_factory):
    """Plans are cached by pipeline content and the versions and row ranges
    of the objects they read: replacing a dimension, rerunning its pipeline
    and viewing another row range each give the result a fresh plan gives."""
    import oracle
    case = GOLDEN["c2_small"]
    w = W.make(case["config"], **case["kwargs"])
    eng = engine_factory(tuple_per_bulk=w.tuple_per_bulk, join_mode="exact")
    W.load_engine(eng, w)
    k1, s1 = W.run_engine(eng, w)
    ek, es = oracle.exact_workload(w)
    np.testing.assert_array_equal(k1, ek)
    np.testing.assert_array_equal(s1, es)
    # the same pipeline text again: the cached plan, the same rows
    eng.run(w.query)
    k2, s2 = eng.result(w.query.id, w.key_num)
    np.testing.assert_array_equal(s2, s1)
    # a different customer table under the same id: every customer's nation shifts by one within its region
    cust = [c.copy() for c in w.dims["customer"]]
    cust[2] = (cust[3] * 5 + (cust[2] - cust[3] * 5 + 1) % 5).astype(np.int32)
    w.dims["customer"] = cust
    eng.put("customer", cust)
    k3, s3 = W.run_engine(eng, w)
    ek3, es3 = oracle.exact_workload(w)
    np.testing.assert_array_equal(k3, ek3)
    np.testing.assert_array_equal(s3, es3)
    assert not np.array_equal(k3, k1) or not np.array_equal(s3, s1)
    # a view of a row range: its own plan
    eng.view("lo_part", "lineorder", 1000, 50_000)
    q = W.fact_pipeline("q2_part", "lo_part", w.fact_schema(), list(w.query.pre_pipeline_id[1:]),
                        [("$(0.0)", "$(1.0)"), ("$(0.5)", "$(2.0)"), ("$(0.6)", "$(3.0)")],
                        "$(2.1),$(3.1),$(1.1)", "$(0.7)-$(0.8)")
    eng.run(q)
    kp, sp = eng.result("q2_part", 3)
    fact = [c[1000:51_000] for c in w.fact_host(0, w.fact_rows)]
    ekp, esp = oracle.exact_workload(w, fact)
    np.testing.assert_array_equal(kp, ekp)
    np.testing.assert_array_equal(sp, esp)
