"""String columns through dictionary encoding on the GPU: fixed-width values
round-trip, Map copies cut or NUL-pad into the output width, StrCmp filters
and Hash group keys equal the oracle (the reference's own results for the
golden cases are checked by test_gpu_parity.py), the batched path agrees, and
uses outside the reference's string grammar are refused."""
import numpy as np
import pytest

import oracle
from oracle import sql_exact
from shadowvm_gb300 import SvmError, capi
from shadowvm_gb300 import workloads as W
from shadowvm_gb300.pipeline import dim_pipeline, fact_pipeline
from shadowvm_gb300.proto import ValType, create_schema

pytestmark = pytest.mark.gpu

S = ValType.String
I32 = ValType.Int32


def test_string_columns_round_trip(engine_factory):
    eng = engine_factory()
    rng = np.random.default_rng(4)
    words = [b"", b"a", b"ab\x00c", b"ZZZZZZ", b"\xff\x80x", b"same", b"same"]
    a = np.array([words[i] for i in rng.integers(0, len(words), 10_000)], dtype="S6")
    b = np.array([bytes([65 + (i % 26)]) * (1 + i % 3) for i in range(10_000)], dtype="S3")
    ints = np.arange(10_000, dtype=np.int32)
    eng.put("s", [ints, a, b])
    assert eng.columns("s") == [(int(I32), 4), (int(S), 6), (int(S), 3)]
    np.testing.assert_array_equal(eng.read("s", 0), ints)
    assert eng.read("s", 1).tobytes() == a.tobytes()
    assert eng.read("s", 2, row0=17, n=100).tobytes() == b[17:117].tobytes()
    with pytest.raises(SvmError):
        eng.read_objects(["s"], [[int(I32), int(S), int(S)]])  # bulk reads are int-only


def test_map_copies_cut_and_pad(engine_factory):
    eng = engine_factory(tuple_per_bulk=4096)
    names = np.array([f"name-{i % 37:03d}-{'x' * (i % 5)}".encode() for i in range(5000)], dtype="S12")
    keys = np.arange(5000, dtype=np.int32)
    eng.put("t", [keys, names])
    src = create_schema([I32, S], [4, 12])
    for width in (4, 9, 12, 20):
        p = dim_pipeline(f"cut{width}", "t", src, "$(0.0),$(0.1)", 'StrCmp($(0.1),"name-01",12)!=0',
                         out_cols=[(I32, 4), (S, width)])
        eng.run(p)
        ek, en = sql_exact.run_select(p, [keys, names])
        np.testing.assert_array_equal(eng.read(p.id, 0), ek)
        got = eng.read(p.id, 1)
        assert got.dtype == np.dtype(f"S{width}")
        assert got.tobytes() == en.tobytes(), width


@pytest.mark.parametrize("mode", ["ref_compat", "exact"])
def test_string_star_equals_oracle(engine_factory, mode):
    """Config 5 (string regions and nations) at a size the oracle finishes in seconds."""
    w = W.make(5, fact_rows=400_000, tuple_per_bulk=200_000, n_part=20_000, n_cust=80_000, n_supp=9_000, qseed=3)
    eng = engine_factory(tuple_per_bulk=w.tuple_per_bulk, join_mode=mode)
    W.load_engine(eng, w)
    keys, sums = W.run_engine(eng, w)
    ek, es = oracle.exact_workload(w)
    np.testing.assert_array_equal(keys, ek)
    np.testing.assert_array_equal(sums, es)
    assert len(keys) == 75


def test_string_keys_through_the_batched_path(engine_factory):
    """Two string-keyed queries (different regions) and an int one in one svm_run_batch."""
    w = W.make(5, fact_rows=300_000, tuple_per_bulk=300_000, n_part=20_000, n_cust=60_000, n_supp=8_000)
    eng = engine_factory(tuple_per_bulk=w.tuple_per_bulk, batch_policy="always")
    W.load_engine(eng, w)
    for p in w.dim_pipelines:
        eng.run(p)
    nat = [(I32, 4), (S, W.NATION_W)]
    other = next(W.region_name(k) for k in range(5) if W.region_name(k) != w.params["c_region"])
    extra = dim_pipeline("q5_cust_b", "customer", w.dim_schema("customer"), "$(0.0),$(0.2)",
                         f'StrCmp($(0.3),"{other}",{W.REGION_W})==0', out_cols=nat)
    eng.run(extra)
    q2 = fact_pipeline("q5b", "lineorder", w.fact_schema(), ["q5_date", "q5_cust_b", "q5_supp"],
                       [("$(0.0)", "$(1.0)"), ("$(0.5)", "$(2.0)"), ("$(0.6)", "$(3.0)")],
                       "$(2.1),$(1.1)", "$(0.7)")
    q3 = fact_pipeline("q5c", "lineorder", w.fact_schema(), ["q5_date"], [("$(0.0)", "$(1.0)")], "$(1.1)",
                       "$(0.3)")
    eng.run_batch([w.query, q2, q3])
    batched = [eng.result(p.id, k) for p, k in ((w.query, 3), (q2, 2), (q3, 1))]
    objs = {n: list(c) for n, c in w.dims.items()}
    for p in w.dim_pipelines + [extra]:
        objs[p.id] = sql_exact.run_select(p, objs[p.pre_pipeline_id[0]])
    fact = w.fact_host(0, w.fact_rows)
    for (k, s), p in zip(batched, (w.query, q2, q3)):
        ek, es = sql_exact.run_reduce(p, fact, [objs[i] for i in p.pre_pipeline_id[1:]])
        np.testing.assert_array_equal(k, ek)
        np.testing.assert_array_equal(s, es)
    eng.run(w.query)  # alone, the same
    k, s = eng.result(w.query.id, 3)
    np.testing.assert_array_equal(k, batched[0][0])
    np.testing.assert_array_equal(s, batched[0][1])


def test_string_uses_outside_the_grammar_are_refused(engine_factory):
    eng = engine_factory(tuple_per_bulk=1000)
    eng.put("u", [np.arange(100, dtype=np.int32), np.array([b"abc", b"abd"] * 50, dtype="S3"),
                  np.arange(100, dtype=np.int32)])
    src = create_schema([I32, S, I32], [4, 3, 4])

    def refused(pred, select="$(0.0)", out=None):
        p = dim_pipeline("bad", "u", src, select, pred, out_cols=out)
        with pytest.raises(SvmError) as e:
            eng.run(p)
        assert e.value.status == capi.E_UNSUPPORTED, pred

    refused("$(0.1) == 3")                                  # a String as a number
    refused('StrCmp($(0.1),"abcd",4)==0')                   # reads past the 3-byte value
    refused('StrCmp($(0.2),"ab",2)==0')                     # StrCmp of an int column
    refused('StrCmp($(0.1),"ab",2) + 1 == 1')               # StrCmp in arithmetic
    refused(None, select="$(0.1)", out=[(I32, 4)])          # a String into an Int32 column
    eng.put("f", [np.arange(100, dtype=np.int32), np.array([b"abc"] * 100, dtype="S3")])
    eng.run(dim_pipeline("ok", "u", src, "$(0.0),$(0.1)", None, out_cols=[(I32, 4), (S, 3)]))
    q = fact_pipeline("badjoin", "f", create_schema([I32, S], [4, 3]), ["ok"], [("$(0.1)", "$(1.1)")],
                      "$(1.0)", "$(0.0)")
    with pytest.raises(SvmError) as e:
        eng.run(q)
    assert e.value.status == capi.E_UNSUPPORTED
    # accepted: the escaped-quote form of the Java DSL
    eng.run(dim_pipeline("esc", "u", src, "$(0.0)", 'StrCmp($(0.1),\\"abd\\",3)==0'))
    np.testing.assert_array_equal(eng.read("esc", 0), np.arange(1, 100, 2, dtype=np.int32))


def test_string_fact_keys_over_views_in_one_batch(engine_factory):
    """GROUP BY a String column of the fact table over two views with
    different row ranges, in one batched launch: the union scan covers both
    ranges, and the views share one hash-rank column spanning the table."""
    rng = np.random.default_rng(8)
    n = 1_000_000
    modes = np.array([b"RAIL", b"AIR", b"SHIP", b"", b"TRUCK", b"Aa", b"BB"], dtype="S5")
    fact = [rng.integers(0, 50, n, dtype=np.int32), modes[rng.integers(0, len(modes), n)],
            rng.integers(-1000, 1000, n, dtype=np.int32)]
    dim = [np.arange(50, dtype=np.int32), np.arange(50, dtype=np.int32) % 7]
    eng = engine_factory(tuple_per_bulk=2_000_000, batch_policy="always")
    eng.put("f", fact)
    eng.put("d", dim)
    eng.run(dim_pipeline("dd", "d", W.int_schema(2), "$(0.0),$(0.1)", "$(0.1) < 5"))
    eng.view("v1", "f", 0, 300_000)
    eng.view("v2", "f", 500_000, 500_000)
    src = create_schema([I32, S, I32], [4, 5, 4])
    qs = [fact_pipeline(f"m{v}", f"v{v}", src, ["dd"], [("$(0.0)", "$(1.0)")], "$(0.1),$(1.1)", "$(0.2)")
          for v in (1, 2)]
    eng.run_batch(qs)
    dsel = sql_exact.run_select(dim_pipeline("dd", "d", W.int_schema(2), "$(0.0),$(0.1)", "$(0.1) < 5"), dim)
    for q, (a, b) in zip(qs, [(0, 300_000), (500_000, 1_000_000)]):
        k, s = eng.result(q.id, 2)
        ek, es = sql_exact.run_reduce(q, [c[a:b] for c in fact], [dsel])
        np.testing.assert_array_equal(k, ek)
        np.testing.assert_array_equal(s, es)
