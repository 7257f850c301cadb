"""Joined projections on the GPU (JoinWith -> Map, no ReduceBy).

The reference generates its join block and then its select block for such a
pipeline (codegen/codegen.cpp:121-180): each fact row passing the filter
probes every joined table, a missing key drops the row, and the projected
expressions may read the matched rows of the joined objects; rows come out in
order (j += cond).  The GPU path must reproduce, bit for bit and in order,
the rows the reference's own code produced (tests/golden/
reference_joinmap.json) in REF_COMPAT mode -- including keys its capped
table dropped and joined objects larger than one bulk -- and the NumPy
evaluation in EXACT mode."""
import json
import os

import numpy as np
import pytest

import oracle
from shadowvm_gb300 import workloads as W
from shadowvm_gb300.pipeline import dim_pipeline

pytestmark = pytest.mark.gpu

JOINMAP = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_joinmap.json")))


def build_case(case):
    w = W.make(case["config"], **case["kwargs"])
    if case["unfiltered_customer"]:
        w.dim_pipelines[1] = dim_pipeline("q2_cust", "customer", W.int_schema(4), "$(0.0),$(0.2)", None)
    return w


def run_gpu(engine_factory, w, mode):
    eng = engine_factory(tuple_per_bulk=w.tuple_per_bulk, join_mode=mode)
    W.load_engine(eng, w)
    for p in w.dim_pipelines:
        eng.run(p)
    eng.run(w.query)
    return eng, eng.read_all(w.query.id)


@pytest.mark.parametrize("name", sorted(JOINMAP))
def test_joined_projection_equals_reference_rows(engine_factory, name):
    case = JOINMAP[name]
    w = build_case(case)
    _, cols = run_gpu(engine_factory, w, "ref_compat")
    assert len(cols) == len(case["columns"])
    for c, (got, want) in enumerate(zip(cols, case["columns"])):
        np.testing.assert_array_equal(got, np.array(want, np.int32), err_msg=f"column {c}")
    assert len(cols[0]) > 100


@pytest.mark.parametrize("name", sorted(JOINMAP))
def test_joined_projection_exact_mode_equals_numpy(engine_factory, name):
    w = build_case(JOINMAP[name])
    _, cols = run_gpu(engine_factory, w, "exact")
    for c, (got, want) in enumerate(zip(cols, oracle.exact_workload_rows(w))):
        np.testing.assert_array_equal(got, want, err_msg=f"column {c}")


def test_joined_projection_output_joins_again(engine_factory):
    """The joined projection's output is an object like any other: a reduce
    pipeline over it (GROUP BY its c_nation column, SUM of its profit column)
    equals the same reduce over the NumPy rows."""
    from shadowvm_gb300.pipeline import fact_pipeline
    case = JOINMAP["c7_small"]
    w = build_case(case)
    eng, cols = run_gpu(engine_factory, w, "ref_compat")
    q = fact_pipeline("q7_sum", "q7", W.int_schema(6), [], [], "$(0.2)", "$(0.4)")
    eng.run(q)
    keys, sums = eng.result("q7_sum", 1)
    nat = np.array(case["columns"][2], np.int64)
    profit = np.array(case["columns"][4], np.int64)
    uniq = np.unique(nat)
    np.testing.assert_array_equal(keys[:, 0], uniq.astype(np.int32))
    np.testing.assert_array_equal(sums[:, 0], np.array([profit[nat == u].sum() for u in uniq], np.int64))
