"""The star-schema workloads, written as the reference's own drivers write them:
dimension-side Filter/Map pipelines, then one fact pipeline joining their
outputs and reducing (example/run_SSB_Q11.cu, run_SSB_Q31.cu).

  config 0  6 M-row fact, date join, SUM(extprice*discount), one row
  config 1  60 M-row fact, date + part join, GROUP BY (year, brand) SUM(revenue)
  config 2  600 M-row fact, date + customer + supplier join,
            GROUP BY (c_nation, s_nation, year) SUM(revenue - supplycost)

Every size can be scaled down for tests.  All columns are seeded and
counter-based (datagen.py), so the fact table is generated on the device by
the library and, for any row range, on the host for the oracle.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import datagen as dg
from .pipeline import dim_pipeline, fact_pipeline
from .proto import ObjectInfo, PipelineInfo, ValType, create_schema

FACT_COLS = {
    0: ["orderdate", "quantity", "discount", "extprice"],
    1: ["orderdate", "quantity", "discount", "extprice", "partkey", "revenue"],
    2: ["orderdate", "quantity", "discount", "extprice", "partkey", "custkey", "suppkey", "revenue",
        "supplycost"],
}


def int_schema(n: int) -> ObjectInfo:
    return create_schema([ValType.Int32] * n, [4] * n)


@dataclass
class Workload:
    config: int
    fact_rows: int
    tuple_per_bulk: int
    seed: int
    n_part: int = 400_000
    n_cust: int = 3_000_000
    n_supp: int = 200_000
    params: dict = field(default_factory=dict)
    dims: dict = field(default_factory=dict)        # name -> list of int32 columns (host)
    dim_pipelines: list = field(default_factory=list)
    query: PipelineInfo | None = None
    key_num: int = 0
    metric_num: int = 1

    @property
    def fact_cols(self) -> list[str]:
        return FACT_COLS[self.config]

    def fact_schema(self) -> ObjectInfo:
        return int_schema(len(self.fact_cols))

    def fact_host(self, row0: int, n: int) -> list[np.ndarray]:
        dk = self.dims["date"][0]
        return [dg.fact_column(c, row0, n, seed=self.seed, n_part=self.n_part, n_cust=self.n_cust,
                               n_supp=self.n_supp, datekeys=dk) for c in self.fact_cols]

    def fact_bytes_per_row(self) -> int:
        """Algorithmic bytes: 4 per distinct fact column the query reads."""
        return 4 * {0: 4, 1: 3, 2: 5}[self.config]


def make(config: int, *, fact_rows: int | None = None, seed: int = dg.DEFAULT_SEED,
         tuple_per_bulk: int | None = None, n_part: int | None = None, n_cust: int | None = None,
         n_supp: int | None = None, qseed: int | None = None) -> Workload:
    qs = seed if qseed is None else qseed

    def dflt(v, d):
        return d if v is None else v

    if config == 0:
        w = Workload(0, dflt(fact_rows, 6_000_000), dflt(tuple_per_bulk, 2_000_000), seed)
        y, d, q = dg.draw(qs, 1, 1992, 1998), dg.draw(qs, 2, 0, 8), dg.draw(qs, 3, 20, 35)
        w.params = {"year": y, "discount_lo": d, "quantity_lt": q}
        dt = dg.date_table()
        w.dims = {"date": [dt["datekey"], dt["year"], dt["month"]]}
        w.dim_pipelines = [dim_pipeline("q0_date", "date", int_schema(3), "$(0.0),$(0.1)", f"$(0.1)=={y}")]
        w.query = fact_pipeline("q0", "lineorder", w.fact_schema(), ["q0_date"], [("$(0.0)", "$(1.0)")],
                                "", "$(0.3)*$(0.2)",
                                predication=f"$(0.2)>={d} && $(0.2)<={d + 2} && $(0.1)<{q}")
        w.key_num = 0
    elif config == 1:
        w = Workload(1, dflt(fact_rows, 60_000_000), dflt(tuple_per_bulk, 2_000_000), seed,
                     n_part=dflt(n_part, 400_000))
        c = dg.draw(qs, 4, 0, 24)
        w.params = {"category": c}
        dt = dg.date_table()
        pt = dg.part_table(w.n_part, seed)
        w.dims = {"date": [dt["datekey"], dt["year"], dt["month"]],
                  "part": [pt["partkey"], pt["category"], pt["brand"]]}
        w.dim_pipelines = [dim_pipeline("q1_date", "date", int_schema(3), "$(0.0),$(0.1)", None),
                           dim_pipeline("q1_part", "part", int_schema(3), "$(0.0),$(0.2)", f"$(0.1)=={c}")]
        w.query = fact_pipeline("q1", "lineorder", w.fact_schema(), ["q1_date", "q1_part"],
                                [("$(0.0)", "$(1.0)"), ("$(0.4)", "$(2.0)")], "$(1.1),$(2.1)", "$(0.5)")
        w.key_num = 2
    elif config == 2:
        w = Workload(2, dflt(fact_rows, 600_000_000), dflt(tuple_per_bulk, 3_000_000), seed,
                     n_part=dflt(n_part, 1_400_000), n_cust=dflt(n_cust, 3_000_000),
                     n_supp=dflt(n_supp, 200_000))
        r, r2, y = dg.draw(qs, 5, 0, 4), dg.draw(qs, 6, 0, 4), dg.draw(qs, 7, 1992, 1996)
        w.params = {"c_region": r, "s_region": r2, "year_lo": y}
        dt = dg.date_table()
        ct = dg.customer_table(w.n_cust, seed)
        st = dg.supplier_table(w.n_supp, seed)
        w.dims = {"date": [dt["datekey"], dt["year"], dt["month"]],
                  "customer": [ct["key"], ct["city"], ct["nation"], ct["region"]],
                  "supplier": [st["key"], st["city"], st["nation"], st["region"]]}
        w.dim_pipelines = [
            dim_pipeline("q2_date", "date", int_schema(3), "$(0.0),$(0.1)", f"$(0.1)>={y} && $(0.1)<={y + 2}"),
            dim_pipeline("q2_cust", "customer", int_schema(4), "$(0.0),$(0.2)", f"$(0.3)=={r}"),
            dim_pipeline("q2_supp", "supplier", int_schema(4), "$(0.0),$(0.2)", f"$(0.3)=={r2}"),
        ]
        w.query = fact_pipeline("q2", "lineorder", w.fact_schema(), ["q2_date", "q2_cust", "q2_supp"],
                                [("$(0.0)", "$(1.0)"), ("$(0.5)", "$(2.0)"), ("$(0.6)", "$(3.0)")],
                                "$(2.1),$(3.1),$(1.1)", "$(0.7)-$(0.8)")
        w.key_num = 3
    else:
        raise ValueError(f"no config {config}")
    return w


# ------------------------------------------------------------------ GPU side
def gen_fact_on_device(engine, w: Workload, fact_id: str = "lineorder", row0: int = 0):
    """Rows row0 .. row0 + w.fact_rows - 1 of the workload's fact table,
    generated by the library on the device (same values as fact_host)."""
    engine.create(fact_id, len(w.fact_cols), w.fact_rows)
    dk = w.dims["date"][0]
    for c, name in enumerate(w.fact_cols):
        cid = dg.COL[name]
        if name == "orderdate":
            engine.gen_uniform(fact_id, c, w.seed, cid, 0, dg.N_DATE - 1, lookup=dk, row0=row0)
        elif name == "partkey":
            engine.gen_uniform(fact_id, c, w.seed, cid, 0, w.n_part - 1, row0=row0)
        elif name == "custkey":
            engine.gen_uniform(fact_id, c, w.seed, cid, 0, w.n_cust - 1, row0=row0)
        elif name == "suppkey":
            engine.gen_uniform(fact_id, c, w.seed, cid, 0, w.n_supp - 1, row0=row0)
        else:
            lo, hi = dg.RANGES[name]
            engine.gen_uniform(fact_id, c, w.seed, cid, lo, hi, row0=row0)


def load_engine(engine, w: Workload, fact_id: str = "lineorder", generate_on_device: bool = True,
                row0: int = 0):
    """Dimensions from host arrays; the fact table generated on the device."""
    for name, cols in w.dims.items():
        engine.put(name, cols)
    if generate_on_device:
        gen_fact_on_device(engine, w, fact_id, row0)
    else:
        engine.put(fact_id, w.fact_host(row0, w.fact_rows))


def run_engine(engine, w: Workload):
    for p in w.dim_pipelines:
        engine.run(p)
    engine.run(w.query)
    return engine.result(w.query.id, w.key_num)
