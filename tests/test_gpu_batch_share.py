"""Merged probe groups share one payload field among tables that carry the
same value at every key they both hold (the same dimension column under
different filters).  A table whose value differs at such a key must end up
with a field of its own, and every query's result must stay exactly the
NumPy evaluation and the single-launch result, in the first batch (which
builds and checks the merged tables) and in later ones (which reuse them)."""
import numpy as np
import pytest

from oracle import sql_exact
from shadowvm_gb300 import workloads as W
from shadowvm_gb300.pipeline import dim_pipeline, fact_pipeline

pytestmark = pytest.mark.gpu

NKEY = 50_000


def _tables(rng, n):
    fact = [rng.integers(0, NKEY, n, dtype=np.int32), rng.integers(-1000, 1000, n, dtype=np.int32),
            rng.integers(0, 100, n, dtype=np.int32)]
    key = np.arange(NKEY, dtype=np.int32)
    # a and c hold the same values; b differs from a at most keys
    dim = [key, key % 13, (key * 7) % 11, key % 13]
    return fact, dim


def _check(eng, fact, dim, dims, queries):
    """queries: (pipeline, number of group keys) pairs."""
    pipes = [q for q, _ in queries]
    eng.run_batch(pipes)
    first = {q.id: eng.result(q.id, nk) for q, nk in queries}
    eng.run_batch(pipes)  # the merged tables now come from the cache
    dsel = {p.id: sql_exact.run_select(p, dim) for p in dims}
    for q, nk in queries:
        k, s = eng.result(q.id, nk)
        ek, es = sql_exact.run_reduce(q, fact, [dsel[i] for i in q.pre_pipeline_id[1:]])
        np.testing.assert_array_equal(k, ek, err_msg=q.id)
        np.testing.assert_array_equal(s, es, err_msg=q.id)
        np.testing.assert_array_equal(first[q.id][0], k, err_msg=q.id)
        np.testing.assert_array_equal(first[q.id][1], s, err_msg=q.id)
        eng.run(q)  # alone
        k1, s1 = eng.result(q.id, nk)
        np.testing.assert_array_equal(k1, k, err_msg=q.id)
        np.testing.assert_array_equal(s1, s, err_msg=q.id)


def _setup(engine_factory, seed):
    rng = np.random.default_rng(seed)
    fact, dim = _tables(rng, 2_000_000)
    eng = engine_factory(tuple_per_bulk=2_000_000, batch_policy="always")
    eng.put("f", fact)
    eng.put("d", dim)
    return eng, fact, dim


def test_shared_payload_field_with_a_disagreeing_table(engine_factory):
    eng, fact, dim = _setup(engine_factory, 21)
    ds = W.int_schema(4)
    dims = [dim_pipeline("pa1", "d", ds, "$(0.0),$(0.1)", "$(0.0) < 30000"),
            dim_pipeline("pa2", "d", ds, "$(0.0),$(0.1)", "$(0.0) >= 20000"),
            dim_pipeline("pb", "d", ds, "$(0.0),$(0.2)", "$(0.0) % 3 == 0"),
            dim_pipeline("pc", "d", ds, "$(0.0),$(0.3)", "$(0.0) % 2 == 0")]
    for p in dims:
        eng.run(p)
    fs = W.int_schema(3)
    j1 = [("$(0.0)", "$(1.0)")]
    queries = [(fact_pipeline(f"q_{d}", "f", fs, [d], j1, "$(1.1)", "$(0.1)", predication="$(0.2) < 60"), 1)
               for d in ("pa1", "pa2", "pb", "pc")]
    queries.append((fact_pipeline("q_ab", "f", fs, ["pa1", "pb"], [("$(0.0)", "$(1.0)"), ("$(0.0)", "$(2.0)")],
                                  "$(1.1),$(2.1)", "$(0.1)"), 2))
    _check(eng, fact, dim, dims, queries)


def test_shared_payload_field_over_disjoint_keys(engine_factory):
    """Tables with different payload columns but no key in common may share
    a field: each key's value is the one table's that holds it."""
    eng, fact, dim = _setup(engine_factory, 22)
    ds = W.int_schema(4)
    dims = [dim_pipeline("lo_a", "d", ds, "$(0.0),$(0.1)", "$(0.0) < 1000"),
            dim_pipeline("hi_b", "d", ds, "$(0.0),$(0.2)", "$(0.0) >= 49000"),
            dim_pipeline("mid_c", "d", ds, "$(0.0),$(0.3)", "$(0.0) >= 20000 && $(0.0) < 21000")]
    for p in dims:
        eng.run(p)
    fs = W.int_schema(3)
    queries = [(fact_pipeline(f"q_{d}", "f", fs, [d], [("$(0.0)", "$(1.0)")], "$(1.1)", "$(0.1)+$(0.2)"), 1)
               for d in ("lo_a", "hi_b", "mid_c")]
    _check(eng, fact, dim, dims, queries)
