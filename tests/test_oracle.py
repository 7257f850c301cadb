"""The oracle pinned against the reference: its results against the committed
fixtures produced by the reference's own CodeGen + runtime headers
(tests/golden/make_golden.py), its generated text against the reference
CodeGen's text, and the independent NumPy evaluator against both."""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle
from oracle import codegen
from shadowvm_gb300 import workloads as W
from shadowvm_gb300.pipeline import dim_pipeline

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


@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_port_reproduces_reference_results(name):
    case = GOLDEN[name]
    w = build_case(case)
    assert w.params == case["params"]
    (keys, sums), _ = oracle.run_workload(w, "port", threads=4)
    gk, gs = golden_arrays(case, w.key_num)
    np.testing.assert_array_equal(keys, gk)
    np.testing.assert_array_equal(sums, gs)


@pytest.mark.skipif(not oracle.ref_available(), reason="reference-compiled checker not built (oracle/_ref)")
@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_fixtures_equal_the_live_reference(name):
    """Where the reference tree is present, its own CodeGen and runtime headers
    (oracle mode "ref") reproduce every committed fixture now, not only when
    the fixtures were written."""
    case = GOLDEN[name]
    w = build_case(case)
    (keys, sums), _ = oracle.run_workload(w, "ref", threads=4)
    gk, gs = golden_arrays(case, w.key_num)
    np.testing.assert_array_equal(keys, gk)
    np.testing.assert_array_equal(sums, gs)


@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_exact_evaluator_agrees_where_reference_drops_nothing(name):
    case = GOLDEN[name]
    w = build_case(case)
    keys, sums = oracle.exact_workload(w)
    gk, gs = golden_arrays(case, w.key_num)
    same = keys.shape == gk.shape and (keys == gk).all() and (sums == gs).all()
    assert same == case["equals_exact"]


@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_codegen_text_matches_reference_codegen(name):
    case = GOLDEN[name]
    w = build_case(case)
    schemas = {p.id: [op.output for op in p.workflow if op.type == 7][0] for p in w.dim_pipelines}
    for p in w.dim_pipelines + [w.query]:
        refs = [schemas[i] for i in p.pre_pipeline_id[1:]] if p is w.query else []
        text = oracle.port_codegen(p, refs)
        assert hashlib.sha256(text.encode()).hexdigest() == case["codegen_sha256"][p.id], p.id


@pytest.mark.skipif(not oracle.ref_available(), reason="reference-compiled checker not built (oracle/_ref)")
def test_codegen_text_matches_live_reference_on_varied_pipelines():
    from shadowvm_gb300.pipeline import fact_pipeline
    from shadowvm_gb300.proto import ValType, create_schema
    src = W.int_schema(6)
    dim = create_schema([ValType.Int32, ValType.Int32, ValType.Int32, ValType.String], [4, 4, 4, 40])
    cases = [
        fact_pipeline("a", "f", src, ["d"], [("$(0.1)", "$(1.0)")], "$(1.2)", "$(0.3)/7,$(0.4)-$(1.1)",
                      predication="($(0.2)>3 || $(0.5)!=0) && !($(0.0)%2)"),
        fact_pipeline("b", "f", src, ["d", "e"], [("$(0.1)", "$(1.0)"), ("$(0.2)", "$(2.0)")],
                      "$(2.1), $(1.2)", "1", predication="$(0.3)<=-5", metric_type=ValType.Int32),
        dim_pipeline("c", "f", src, "$(0.0),$(0.1)*3,$(0.2)+$(0.3)", "$(0.4)>=1 && $(0.4)<=9"),
    ]
    for p in cases:
        refs = [dim] * (len(p.pre_pipeline_id) - 1)
        assert oracle.port_codegen(p, refs) == oracle.ref_codegen(p, refs), p.id


def test_str_split_matches_reference_rules():
    assert codegen.str_split("a,b,", ",") == ["a", "b"]
    assert codegen.str_split("a,,b", ",") == ["a", "", "b"]
    assert codegen.str_split("", ",") == []
    assert codegen.gen_key_index(" $(2.13))") == codegen.KeyIndex(2, 13)


def test_exact_evaluator_c_semantics():
    from oracle import sql_exact as S
    env = {(0, 0): np.array([-7, 7, 2**31 - 1], np.int32), (0, 1): np.array([2, -2, 2], np.int32)}
    np.testing.assert_array_equal(S.evaluate(S.parse("$(0.0)/$(0.1)"), env, 3), [-3, -3, 1073741823])
    np.testing.assert_array_equal(S.evaluate(S.parse("$(0.0)%$(0.1)"), env, 3), [-1, 1, 1])
    np.testing.assert_array_equal(S.evaluate(S.parse("$(0.0)*$(0.1)"), env, 3), [-14, -14, -2])
    np.testing.assert_array_equal(S.evaluate(S.parse("$(0.0)>0 && $(0.1)>0 || !$(0.0)"), env, 3), [0, 0, 1])
    np.testing.assert_array_equal(S.evaluate(S.parse("010 + 0x10"), env, 3), [24, 24, 24])


JOINMAP = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_joinmap.json")))


@pytest.mark.parametrize("name", sorted(JOINMAP))
def test_port_reproduces_reference_joined_projections(name):
    case = JOINMAP[name]
    w = build_case(case)
    assert w.params == case["params"]
    cols = oracle.run_workload_rows(w, "port", threads=4)
    assert len(cols) == len(case["columns"])
    for got, want in zip(cols, case["columns"]):
        np.testing.assert_array_equal(got, np.array(want, np.int32))
    exact = oracle.exact_workload_rows(w)
    same = all(len(a) == len(b) and (a == b).all() for a, b in zip(exact, cols))
    assert same == case["equals_exact"]


@pytest.mark.skipif(not oracle.ref_available(), reason="reference-compiled checker not built (oracle/_ref)")
@pytest.mark.parametrize("name", sorted(JOINMAP))
def test_joined_projection_fixtures_equal_the_live_reference(name):
    case = JOINMAP[name]
    w = build_case(case)
    cols = oracle.run_workload_rows(w, "ref", threads=4)
    for got, want in zip(cols, case["columns"]):
        np.testing.assert_array_equal(got, np.array(want, np.int32))


@pytest.mark.parametrize("name", sorted(JOINMAP))
def test_joined_projection_codegen_text_matches_reference_codegen(name):
    case = JOINMAP[name]
    w = build_case(case)
    schemas = {p.id: [op.output for op in p.workflow if op.type == 7][0] for p in w.dim_pipelines}
    for p in w.dim_pipelines + [w.query]:
        refs = [schemas[i] for i in p.pre_pipeline_id[1:]] if p is w.query else []
        assert hashlib.sha256(oracle.port_codegen(p, refs).encode()).hexdigest() == case["codegen_sha256"][p.id]
