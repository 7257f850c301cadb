"""A fact table left in page-locked host memory (svm_object_put_host).

The reference keeps its fact bulks in mapped pinned host memory
(object/object.cpp:194-294); here a reduce pipeline's scan copies only the
columns its filter steps read and gathers the others from host memory at
the surviving rows.  The results must equal the reference's golden rows and
the same query over the table on the device; every other use of such an
object is refused."""
import copy
import json
import os

import numpy as np
import pytest

from shadowvm_gb300 import SvmError
from shadowvm_gb300 import workloads as W
from shadowvm_gb300.pipeline import dim_pipeline

pytestmark = pytest.mark.gpu

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_results.json")))


def golden_rows(case, key_num):
    rows = len(case["sums"])
    keys = np.array(case["keys"], np.int32).reshape(rows, key_num)
    sums = np.array(case["sums"], np.int64).reshape(rows, -1) if rows else np.zeros((0, 1), np.int64)
    return keys, sums


def pinned_copy(eng, oid, ncols):
    """Each column of device object `oid` copied into page-locked host memory."""
    import torch
    out, keep = [], []
    for c in range(ncols):
        a = eng.read(oid, c)
        t = torch.empty(len(a), dtype=torch.int32, pin_memory=True)
        t.numpy()[:] = a
        keep.append(t)
        out.append(t.numpy())
    return out, keep


def on(query, source):
    q = copy.deepcopy(query)
    q.id = query.id + "_" + source
    q.pre_pipeline_id[0] = source
    return q


@pytest.mark.parametrize("name", ["c0_small", "c1_small", "c2_small", "c2_drops"])
def test_host_resident_fact_table_equals_the_reference(engine_factory, name):
    case = GOLDEN[name]
    w = W.make(case["config"], **case["kwargs"])
    if case["unfiltered_customer"]:
        w.dim_pipelines[1] = dim_pipeline("q2_cust", "customer", W.int_schema(4), "$(0.0),$(0.2)", None)
    gk, gs = golden_rows(case, w.key_num)
    eng = engine_factory(tuple_per_bulk=w.tuple_per_bulk)
    W.load_engine(eng, w)
    dk, ds = W.run_engine(eng, w)  # the table on the device
    cols, keep = pinned_copy(eng, "lineorder", len(w.fact_cols))
    eng.put_host("lineorder_h", cols)
    q = on(w.query, "lineorder_h")
    eng.run(q)
    hk, hs = eng.result(q.id, w.key_num)
    np.testing.assert_array_equal(hk, gk)
    np.testing.assert_array_equal(hs, gs)
    np.testing.assert_array_equal(hk, dk)
    np.testing.assert_array_equal(hs, ds)
    launch = eng.last_launch()
    if name == "c2_drops":  # a hash-layout customer table: the interpreted kernel, every column copied
        assert launch["kernel"] == "interpreted" and launch["late_columns"] == 0, launch
    else:  # the compiled kernel, the metric columns gathered from host memory
        assert launch["kernel"] == "compiled plan" and launch["late_columns"] >= 1, launch
    # a view of it: rows [1000, n - 777)
    n = w.fact_rows
    eng.view("lineorder_hv", "lineorder_h", 1000, n - 1777)
    eng.view("lineorder_dv", "lineorder", 1000, n - 1777)
    qv, qd = on(w.query, "lineorder_hv"), on(w.query, "lineorder_dv")
    eng.run(qv)
    eng.run(qd)
    vk, vs = eng.result(qv.id, w.key_num)
    ek, es = eng.result(qd.id, w.key_num)
    np.testing.assert_array_equal(vk, ek)
    np.testing.assert_array_equal(vs, es)
    eng.drop("lineorder_hv")
    eng.drop("lineorder_h")
    del keep


def test_host_resident_object_refusals(engine_factory):
    case = GOLDEN["c2_small"]
    w = W.make(case["config"], **case["kwargs"])
    eng = engine_factory(tuple_per_bulk=w.tuple_per_bulk, batch_policy="always")
    W.load_engine(eng, w)
    for p in w.dim_pipelines:
        eng.run(p)
    cols, keep = pinned_copy(eng, "lineorder", len(w.fact_cols))
    eng.put_host("lineorder_h", cols)
    for call in (lambda: eng.read("lineorder_h", 0),
                 lambda: eng.gen_uniform("lineorder_h", 0, 1, 1, 0, 9),
                 lambda: eng.run(dim_pipeline("map_h", "lineorder_h", W.int_schema(len(w.fact_cols)),
                                              "$(0.0),$(0.1)", "$(0.1)<10"))):
        with pytest.raises(SvmError) as ei:
            call()
        assert "UNSUPPORTED" in str(ei.value), ei.value
    # batched with a query over the device table: it runs alone, same rows
    q_h, q_d = on(w.query, "lineorder_h"), on(w.query, "lineorder")
    eng.run_batch([q_h, q_d])
    hk, hs = eng.result(q_h.id, w.key_num)
    dk, ds = eng.result(q_d.id, w.key_num)
    np.testing.assert_array_equal(hk, dk)
    np.testing.assert_array_equal(hs, ds)
    # pageable memory is refused
    plain = [np.array(c) for c in cols]
    with pytest.raises(SvmError) as ei:
        eng.put_host("lineorder_p", plain)
    assert "INVALID_ARG" in str(ei.value), ei.value
    eng.drop("lineorder_h")
    del keep


@pytest.mark.parametrize("config", [0, 2])
def test_host_resident_ragged_row_count(engine_factory, config):
    """A row count that is no multiple of 4 (the scan's last 16-byte reads run
    past the host column's end, whose rows the copy must not read) and a view
    that ends on the table's last row: the same rows as on the device."""
    kw = dict(fact_rows=123_457, tuple_per_bulk=100_000)
    if config == 2:
        kw.update(n_part=20_000, n_cust=30_000, n_supp=5_000)
    w = W.make(config, **kw)
    eng = engine_factory(tuple_per_bulk=w.tuple_per_bulk)
    W.load_engine(eng, w)
    dk, ds = W.run_engine(eng, w)
    cols, keep = pinned_copy(eng, "lineorder", len(w.fact_cols))
    eng.put_host("lineorder_h", cols)
    q = on(w.query, "lineorder_h")
    eng.run(q)
    hk, hs = eng.result(q.id, w.key_num)
    np.testing.assert_array_equal(hk, dk)
    np.testing.assert_array_equal(hs, ds)
    eng.view("lineorder_hv", "lineorder_h", 5, w.fact_rows - 5)
    eng.view("lineorder_dv", "lineorder", 5, w.fact_rows - 5)
    qv, qd = on(w.query, "lineorder_hv"), on(w.query, "lineorder_dv")
    eng.run(qv)
    eng.run(qd)
    np.testing.assert_array_equal(eng.result(qv.id, w.key_num)[1], eng.result(qd.id, w.key_num)[1])
    eng.drop("lineorder_hv")
    eng.drop("lineorder_h")
    del keep


def test_host_resident_query_in_a_fold(engine_factory):
    """A fold in flight (svm_batch_begin) with a query over a host-resident
    table runs that query alone inside the call; its result and the batched
    one over the device table both equal the queries run alone."""
    from shadowvm_gb300.serving import sink_types
    case = GOLDEN["c2_small"]
    w = W.make(case["config"], **case["kwargs"])
    eng = engine_factory(tuple_per_bulk=w.tuple_per_bulk, batch_policy="always")
    W.load_engine(eng, w)
    dk, ds = W.run_engine(eng, w)
    cols, keep = pinned_copy(eng, "lineorder", len(w.fact_cols))
    eng.put_host("lineorder_h", cols)
    q_h, q_d = on(w.query, "lineorder_h"), on(w.query, "lineorder")
    f = eng.batch_begin([q_h, q_d], host_results=True)
    rows = f.wait()
    f.release([sink_types(p) for p in (q_h, q_d)])
    for q in (q_h, q_d):
        k, v = eng.result(q.id, w.key_num)
        np.testing.assert_array_equal(k, dk)
        np.testing.assert_array_equal(v, ds)
    assert rows == [len(ds), len(ds)]
    eng.drop("lineorder_h")
    del keep

