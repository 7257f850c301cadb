"""Generates tests/golden/*.json from the reference's own code path.

Run here, where the reference tree is present (x86):
    python oracle/build_ref.sh && python tests/golden/make_golden.py

For every case below it runs the workload through the reference's OWN
CodeGen and runtime headers (oracle mode "ref", built by oracle/build_ref.sh
from the reference sources) and records the merged, key-sorted result.  For
the code generator it records the SHA-256 of the host code the reference's
CodeGen emits for each pipeline (the text itself is not stored).  Joined
projections (JoinWith -> Map, no ReduceBy) go to reference_joinmap.json with
their output rows in order.  A GPU host
without the reference tree runs the tests against these files instead.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from shadowvm_gb300 import workloads as W  # noqa: E402
from shadowvm_gb300.pipeline import dim_pipeline  # noqa: E402

# (name, config, make() kwargs, unfiltered-customer variant)
CASES = [
    ("c0_small", 0, dict(fact_rows=250_000, tuple_per_bulk=100_000), False),
    ("c0_q2", 0, dict(fact_rows=120_000, tuple_per_bulk=50_000, qseed=2), False),
    ("c1_small", 1, dict(fact_rows=250_000, tuple_per_bulk=100_000, n_part=20_000), False),
    ("c1_q3", 1, dict(fact_rows=200_000, tuple_per_bulk=100_000, n_part=30_000, qseed=3), False),
    ("c2_small", 2, dict(fact_rows=300_000, tuple_per_bulk=100_000, n_part=20_000, n_cust=60_000,
                         n_supp=8_000), False),
    ("c2_q11", 2, dict(fact_rows=200_000, tuple_per_bulk=100_000, n_part=20_000, n_cust=50_000,
                       n_supp=6_000, qseed=11), False),
    # joined object larger than one bulk: only its bulk 0 is joinable
    ("c2_bulk0", 2, dict(fact_rows=200_000, tuple_per_bulk=40_000, n_part=20_000, n_cust=100_000,
                         n_supp=8_000, qseed=7), False),
    # unfiltered 300 K customers in a 1.5 M-slot table: the 10-step cap drops keys
    ("c2_drops", 2, dict(fact_rows=400_000, tuple_per_bulk=300_000, n_part=20_000, n_cust=300_000,
                         n_supp=8_000, qseed=7), True),
    # an empty fact table: no bulk, no result row
    ("c0_empty", 0, dict(fact_rows=0, tuple_per_bulk=100_000), False),
    # String dimension columns: StrCmp region filters, GROUP BY nation strings (Hash keys)
    ("c5_small", 5, dict(fact_rows=300_000, tuple_per_bulk=100_000, n_part=20_000, n_cust=60_000,
                         n_supp=8_000), False),
    ("c5_q9", 5, dict(fact_rows=200_000, tuple_per_bulk=100_000, n_part=20_000, n_cust=40_000,
                      n_supp=6_000, qseed=9), False),
    # StrCmp's NUL rules, a Hash collision, signed chars, a cut Map copy, a String fact column
    ("c6_edges", 6, dict(fact_rows=50_000, tuple_per_bulk=20_000), False),
]


# Joined projections (JoinWith -> Map, no ReduceBy): the rows themselves.
JOIN_MAP_CASES = [
    ("c7_small", 7, dict(fact_rows=200_000, tuple_per_bulk=100_000, n_part=20_000, n_cust=60_000,
                         n_supp=8_000), False),
    # unfiltered 300 K customers in a 1.5 M-slot table: rows whose customer key was dropped vanish
    ("c7_drops", 7, dict(fact_rows=60_000, tuple_per_bulk=300_000, n_part=20_000, n_cust=300_000,
                         n_supp=8_000, qseed=7), True),
    # joined objects larger than one bulk: only their bulk 0 is joinable; several fact bulks
    ("c7_bulk0", 7, dict(fact_rows=150_000, tuple_per_bulk=40_000, n_part=20_000, n_cust=100_000,
                         n_supp=8_000, qseed=7), False),
]


def build_case(cfg, kw, unfiltered_cust):
    w = W.make(cfg, **kw)
    if unfiltered_cust:
        w.dim_pipelines[1] = dim_pipeline("q2_cust", "customer", W.int_schema(4), "$(0.0),$(0.2)", None)
    return w


def main():
    if not oracle.ref_available():
        oracle.build_ref()
    out = {}
    for name, cfg, kw, unf in CASES:
        w = build_case(cfg, kw, unf)
        (keys, sums), _ = oracle.run_workload(w, "ref", threads=8)
        k2, s2 = oracle.exact_workload(w)
        same = keys.shape == k2.shape and (keys == k2).all() and (sums == s2).all()
        texts = {}
        for p in w.dim_pipelines + [w.query]:
            refs = []
            if p is w.query:
                refs = [dim_schema(w, i) for i in p.pre_pipeline_id[1:]]
            texts[p.id] = hashlib.sha256(oracle.ref_codegen(p, refs).encode()).hexdigest()
        out[name] = {"config": cfg, "kwargs": kw, "unfiltered_customer": unf, "params": w.params,
                     "keys": keys.tolist(), "sums": sums.tolist(), "equals_exact": bool(same),
                     "codegen_sha256": texts}
        print(name, len(keys), "equals_exact" if same else "differs from exact")
    with open(os.path.join(HERE, "reference_results.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    rows = {}
    for name, cfg, kw, unf in JOIN_MAP_CASES:
        w = build_case(cfg, kw, unf)
        cols = oracle.run_workload_rows(w, "ref", threads=8)
        exact = oracle.exact_workload_rows(w)
        same = all(len(a) == len(b) and (a == b).all() for a, b in zip(cols, exact))
        texts = {}
        for p in w.dim_pipelines + [w.query]:
            refs = [dim_schema(w, i) for i in p.pre_pipeline_id[1:]] if p is w.query else []
            texts[p.id] = hashlib.sha256(oracle.ref_codegen(p, refs).encode()).hexdigest()
        rows[name] = {"config": cfg, "kwargs": kw, "unfiltered_customer": unf, "params": w.params,
                      "columns": [c.tolist() for c in cols], "equals_exact": bool(same),
                      "codegen_sha256": texts}
        print(name, len(cols[0]), "equals_exact" if same else "differs from exact")
    with open(os.path.join(HERE, "reference_joinmap.json"), "w") as f:
        json.dump(rows, f, sort_keys=True)


def dim_schema(w, pid):
    for p in w.dim_pipelines:
        if p.id == pid:
            return [op.output for op in p.workflow if op.type == 7][0]
    raise KeyError(pid)


if __name__ == "__main__":
    main()
