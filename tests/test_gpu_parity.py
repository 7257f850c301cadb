"""GPU parity: the CUDA path through the C ABI against the oracle.

REF_COMPAT results must equal, bit for bit, the reference's own results
committed in tests/golden/reference_results.json (int64 sums, rows sorted by
key); EXACT results must equal the NumPy sql_exact evaluation."""
import json
import os

import numpy as np
import pytest

import oracle
from shadowvm_gb300 import SvmError, capi
from shadowvm_gb300 import datagen as dg
from shadowvm_gb300 import workloads as W
from shadowvm_gb300.pipeline import dim_pipeline, fact_pipeline

pytestmark = pytest.mark.gpu

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_results.json")))


def build_case(case):
    w = W.make(case["config"], **case["kwargs"])
    if case["unfiltered_customer"]:
        w.dim_pipelines[1] = dim_pipeline("q2_cust", "customer", W.int_schema(4), "$(0.0),$(0.2)", None)
    return w


def golden_arrays(case, key_num):
    rows = len(case["sums"])
    keys = np.array(case["keys"], np.int32).reshape(rows, key_num)
    sums = np.array(case["sums"], np.int64).reshape(rows, -1) if rows else np.zeros((0, 1), np.int64)
    return keys, sums


def run_gpu(engine_factory, w, mode="ref_compat", on_device=True):
    eng = engine_factory(tuple_per_bulk=w.tuple_per_bulk, join_mode=mode)
    W.load_engine(eng, w, generate_on_device=on_device and w.fact_rows > 0)
    return W.run_engine(eng, w)


@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_ref_compat_equals_reference(engine_factory, name):
    case = GOLDEN[name]
    w = build_case(case)
    keys, sums = run_gpu(engine_factory, w)
    gk, gs = golden_arrays(case, w.key_num)
    np.testing.assert_array_equal(keys, gk)
    np.testing.assert_array_equal(sums, gs)


@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_exact_equals_sql_exact(engine_factory, name):
    w = build_case(GOLDEN[name])
    keys, sums = run_gpu(engine_factory, w, mode="exact")
    ek, es = oracle.exact_workload(w)
    np.testing.assert_array_equal(keys, ek)
    np.testing.assert_array_equal(sums, es)


def test_device_generator_matches_numpy(engine_factory):
    eng = engine_factory()
    n = 100_003
    eng.create("g", 2, n)
    eng.gen_uniform("g", 0, 123, 4, 90_000, 10_500_000)
    lut = np.arange(10, 20, dtype=np.int32) * 7
    eng.gen_uniform("g", 1, 5, 1, 0, 9, lookup=lut)
    np.testing.assert_array_equal(eng.read("g", 0), dg.uniform(123, 4, 90_000, 10_500_000, 0, n))
    np.testing.assert_array_equal(eng.read("g", 1), lut[dg.uniform(5, 1, 0, 9, 0, n)])


def test_select_pipeline_matches_numpy(engine_factory):
    from oracle import sql_exact
    eng = engine_factory(tuple_per_bulk=1000)
    rng = np.random.default_rng(1)
    cols = [rng.integers(-50, 50, 5000).astype(np.int32) for _ in range(3)]
    eng.put("t", cols)
    p = dim_pipeline("s", "t", W.int_schema(3), "$(0.0),$(0.1)*3-$(0.2),$(0.2)/7",
                     "$(0.0)>-10 && ($(0.1)%3==1 || $(0.2)<0)")
    eng.run(p)
    got = eng.read_all("s")
    want = sql_exact.run_select(p, cols)
    for g, e in zip(got, want):
        np.testing.assert_array_equal(g, e)


def test_general_expressions_and_int32_sums(engine_factory):
    """Residual (non-range) predicates, bytecode metrics, Int32-declared sums
    that wrap like the reference's int32 accumulation."""
    from oracle import sql_exact
    eng = engine_factory(tuple_per_bulk=4096, join_mode="exact")
    rng = np.random.default_rng(7)
    n = 50_000
    fact = [rng.integers(0, 300, n).astype(np.int32), rng.integers(-1000, 1000, n).astype(np.int32),
            rng.integers(1, 2_000_000_000, n).astype(np.int32), rng.integers(0, 9, n).astype(np.int32)]
    dim = [np.arange(300, dtype=np.int32), rng.integers(0, 5, 300).astype(np.int32),
           rng.integers(-3, 4, 300).astype(np.int32)]
    eng.put("f", fact)
    eng.put("d", dim)
    dp = dim_pipeline("dd", "d", W.int_schema(3), "$(0.0),$(0.1),$(0.2)", "$(0.1)!=2")
    eng.run(dp)
    q = fact_pipeline("qq", "f", W.int_schema(4), ["dd"], [("$(0.0)", "$(1.0)")], "$(1.1),$(0.3)",
                      "$(0.2)+$(0.2),($(0.1)*$(1.2))/3,$(0.3)?$(0.1):-1",
                      predication="$(0.1)%5!=0 && $(0.3)>=2", metric_type=capi_i32())
    eng.run(q)
    keys, sums = eng.result("qq", 2)
    dims = [sql_exact.run_select(dp, dim)]
    ek, es = sql_exact.run_reduce(q, fact, dims, metric_wide=[False] * 3)
    np.testing.assert_array_equal(keys, ek)
    np.testing.assert_array_equal(sums, es)


def capi_i32():
    from shadowvm_gb300.proto import ValType
    return ValType.Int32


def test_errors_are_reported(engine_factory):
    eng = engine_factory(tuple_per_bulk=1000)
    eng.put("f", [np.arange(10, dtype=np.int32), np.arange(10, dtype=np.int32)])
    eng.put("d", [np.arange(10, dtype=np.int32), np.arange(10, dtype=np.int32)])
    eng.run(dim_pipeline("dd", "d", W.int_schema(2), "$(0.0),$(0.1)", None))
    with pytest.raises(SvmError) as e:
        eng.run(fact_pipeline("q", "missing", W.int_schema(2), ["dd"], [("$(0.0)", "$(1.0)")], "", "$(0.1)"))
    assert e.value.status == capi.E_NOT_FOUND
    with pytest.raises(SvmError) as e:  # the metric list splits on commas, as the reference's StrSplit
        eng.run(fact_pipeline("q", "f", W.int_schema(2), ["dd"], [("$(0.0)", "$(1.0)")], "",
                              "StrCmp($(0.1),\"x\",1)"))
    assert e.value.status == capi.E_INVALID_ARG
    with pytest.raises(SvmError) as e:  # StrCmp of an int column
        eng.run(fact_pipeline("q", "f", W.int_schema(2), ["dd"], [("$(0.0)", "$(1.0)")], "", "$(0.1)",
                              predication='StrCmp($(0.1),"x",1)==0'))
    assert e.value.status == capi.E_UNSUPPORTED
    with pytest.raises(SvmError) as e:  # a UDF call
        eng.run(fact_pipeline("q", "f", W.int_schema(2), ["dd"], [("$(0.0)", "$(1.0)")], "", "$(0.1)",
                              predication="udf($(0.1))==0"))
    assert e.value.status == capi.E_UNSUPPORTED
    with pytest.raises(SvmError) as e:
        eng.run(fact_pipeline("q", "f", W.int_schema(2), ["dd"], [("$(0.0)", "$(1.0)")], "", "100/$(0.1)"))
    assert e.value.status == capi.E_DEVICE
    # the context stays usable after an error
    eng.run(fact_pipeline("q", "f", W.int_schema(2), ["dd"], [("$(0.0)", "$(1.0)")], "", "$(0.1)"))
    assert eng.result("q", 0)[1].tolist() == [[45]]


def test_empty_dimension_and_no_passing_rows(engine_factory):
    w = W.make(2, fact_rows=50_000, tuple_per_bulk=20_000, n_part=1000, n_cust=5000, n_supp=500)
    w.dim_pipelines[1] = dim_pipeline("q2_cust", "customer", W.int_schema(4), "$(0.0),$(0.2)", "$(0.3)==99")
    keys, sums = run_gpu(engine_factory, w)
    assert keys.shape == (0, 3) and sums.shape[0] == 0
    w0 = W.make(0, fact_rows=50_000, tuple_per_bulk=20_000)
    w0.query.workflow[1].args["predication"] = "$(0.1)<0"
    keys, sums = run_gpu(engine_factory, w0)
    assert sums.tolist() == [[0]]


@pytest.mark.parametrize("config", [0, 1, 2, 5])
def test_autotuned_launch_equals_fixed_rule(engine_factory, config):
    """The launch tuner times several configurations on the query itself;
    whichever it keeps, the result equals the fixed rule's, first run and
    cached run alike."""
    w = W.make(config, fact_rows=400_000, tuple_per_bulk=200_000, n_part=20_000, n_cust=50_000, n_supp=6_000)
    res = []
    for tune in (True, False):
        eng = engine_factory(tuple_per_bulk=w.tuple_per_bulk, autotune=tune)
        W.load_engine(eng, w)
        first = W.run_engine(eng, w)
        eng.run(w.query)
        again = eng.result(w.query.id, w.key_num)
        np.testing.assert_array_equal(first[0], again[0])
        np.testing.assert_array_equal(first[1], again[1])
        res.append(first)
    np.testing.assert_array_equal(res[0][0], res[1][0])
    np.testing.assert_array_equal(res[0][1], res[1][1])
