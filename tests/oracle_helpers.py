"""Test-side helpers that evaluate workloads through the oracle (never part
of the product package)."""
from __future__ import annotations

import os

import numpy as np

import oracle
from oracle import sql_exact
from shadowvm_gb300 import datagen as dg


def exact_batch_query(bw, i: int, fact: list | None = None):
    """One query of a batch workload through the NumPy evaluator."""
    q = bw.queries[i]
    objs = {name: list(cols) for name, cols in bw.fact.dims.items()}
    for p in bw.dim_pipelines:
        if p.id in q.pipe.pre_pipeline_id:
            objs[p.id] = sql_exact.run_select(p, objs[p.pre_pipeline_id[0]])
    f = bw.fact.fact_host(q.row0, q.nrows) if fact is None else [c[q.row0:q.row0 + q.nrows] for c in fact]
    return sql_exact.run_reduce(q.pipe, f, [objs[x] for x in q.pipe.pre_pipeline_id[1:]])


# Fact columns each workload's query reads (the others stay zero for the oracle).
USED_COLS = {0: [0, 1, 2, 3], 1: [0, 4, 5], 2: [0, 5, 6, 7, 8], 5: [0, 5, 6, 7, 8]}


def fact_columns_read(w, row0: int = 0, n: int | None = None) -> list[np.ndarray]:
    """The workload's fact rows [row0, row0 + n) generated on the host, only the
    columns its query reads; the other columns are zeros (never read)."""
    n = w.fact_rows if n is None else n
    dk = w.dims["date"][0]
    out = []
    for c, name in enumerate(w.fact_cols):
        if c in USED_COLS[w.config]:
            out.append(dg.fact_column(name, row0, n, seed=w.seed, n_part=w.n_part, n_cust=w.n_cust,
                                      n_supp=w.n_supp, datekeys=dk))
        else:
            out.append(np.zeros(n, np.int32))
    return out


def port_threads() -> int:
    return max(1, min(32, os.cpu_count() or 1))


def port_workload(w, fact=None):
    """The reference's generated CPU path (oracle port) on the workload."""
    (keys, sums), _ = oracle.run_workload(w, "port", threads=port_threads(), fact=fact)
    return keys, sums


def port_dimension_objects(w, names=None):
    """The workload's dimension tables as oracle objects (tuple_per_bulk rows a
    bulk), keyed by name."""
    from shadowvm_gb300.workloads import schema_of
    tpb = w.tuple_per_bulk
    return {name: oracle.Obj.from_columns(cols, schema_of(cols), tpb, "port")
            for name, cols in w.dims.items() if names is None or name in names}


def port_query(w, dim_pipelines, query, fact_cols, fact_schema, key_num: int, metric_num: int = 1, objs=None):
    """One fact pipeline over host fact columns through the oracle port, after
    the dimension pipelines it needs; returns (keys, sums) merged and sorted."""
    tpb = w.tuple_per_bulk
    objs = port_dimension_objects(w) if objs is None else objs
    for p in dim_pipelines:
        if p.id not in objs:
            objs[p.id], _ = oracle.run_pipeline(p, objs[p.pre_pipeline_id[0]], [], tpb, port_threads(), "port")
    src = oracle.Obj.from_columns(fact_cols, fact_schema, tpb, "port")
    sink, _ = oracle.run_pipeline(query, src, [objs[i] for i in query.pre_pipeline_id[1:]], tpb,
                                  port_threads(), "port")
    return oracle.merge_groups(sink, key_num, metric_num)
