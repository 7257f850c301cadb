"""The star-schema workloads, written as the reference's own drivers write them:
dimension-side Filter/Map pipelines, then one fact pipeline joining their
outputs and reducing (example/run_SSB_Q11.cu, run_SSB_Q31.cu).

  config 0  6 M-row fact, date join, SUM(extprice*discount), one row
  config 1  60 M-row fact, date + part join, GROUP BY (year, brand) SUM(revenue)
  config 2  600 M-row fact, date + customer + supplier join,
            GROUP BY (c_nation, s_nation, year) SUM(revenue - supplycost)
  config 3  a batch of 256 queries shaped like configs 0-2 over views of the
            resident 600 M-row config-2 fact table (make_batch)
  config 5  config 2's query over dimension tables whose city / nation /
            region are fixed-width String columns: StrCmp region filters,
            GROUP BY the nation strings (Hash keys), as the reference's string
            SSB queries are written (java_vRDD/.../SSBHelper.java:176-206)

Every size can be scaled down for tests.  All columns are seeded and
counter-based (datagen.py), so the fact table is generated on the device by
the library and, for any row range, on the host for the oracle.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import datagen as dg
from .pipeline import dim_pipeline, fact_pipeline, join_map_pipeline
from .proto import ObjectInfo, PipelineInfo, ValType, create_schema

FACT_COLS = {
    0: ["orderdate", "quantity", "discount", "extprice"],
    1: ["orderdate", "quantity", "discount", "extprice", "partkey", "revenue"],
    2: ["orderdate", "quantity", "discount", "extprice", "partkey", "custkey", "suppkey", "revenue",
        "supplycost"],
}
FACT_COLS[5] = FACT_COLS[2]
FACT_COLS[7] = FACT_COLS[2]

# String widths of config 5's geography columns (bytes, NUL-padded).
CITY_W, NATION_W, REGION_W = 10, 15, 12


def int_schema(n: int) -> ObjectInfo:
    return create_schema([ValType.Int32] * n, [4] * n)


def schema_of(cols: list) -> ObjectInfo:
    """The schema of host columns: int32 / int64, or String of width w for 'S<w>' bytes."""
    types, sizes = [], []
    for c in cols:
        dt = np.asarray(c).dtype
        if dt.kind == "S":
            types.append(ValType.String)
            sizes.append(dt.itemsize)
        else:
            types.append(ValType.Int64 if dt == np.int64 else ValType.Int32)
            sizes.append(dt.itemsize)
    return create_schema(types, sizes)


def city_name(c: int) -> str:
    return f"CT{c:03d}" + "xyz"[: c % 4]


def nation_name(n: int) -> str:
    return f"NAT{n:02d}-" + "nation"[: n % 7]


def region_name(r: int) -> str:
    return f"RG{r}-" + "region"[: r + 1]


def geo_strings(table: dict) -> list[np.ndarray]:
    """City / nation / region codes of a geography table as synthetic
    fixed-width names of varied lengths (no two share a prefix that StrCmp
    would take for equality)."""
    def names(codes, fmt, width):
        uniq = np.unique(codes)
        lut = np.array([fmt(int(u)).encode() for u in uniq], dtype=f"S{width}")
        return lut[np.searchsorted(uniq, codes)]
    return [names(table["city"], city_name, CITY_W), names(table["nation"], nation_name, NATION_W),
            names(table["region"], region_name, REGION_W)]


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
    device_fact: bool = True                        # the library can generate the fact table

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
        return 4 * {0: 4, 1: 3, 2: 5, 5: 5, 7: 6}[self.config]

    def dim_schema(self, name: str) -> ObjectInfo:
        return schema_of(self.dims[name])


def make(config: int, *, fact_rows: int | None = None, seed: int = dg.DEFAULT_SEED,
         tuple_per_bulk: int | None = None, n_part: int | None = None, n_cust: int | None = None,
         n_supp: int | None = None, qseed: int | None = None) -> Workload:
    qs = seed if qseed is None else qseed

    def dflt(v, d):
        return d if v is None else v

    if config == 6:
        return make_string_edges(dflt(fact_rows, 50_000), dflt(tuple_per_bulk, 20_000), seed)

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
    elif config == 5:
        w = Workload(5, dflt(fact_rows, 600_000_000), dflt(tuple_per_bulk, 3_000_000), seed,
                     n_part=dflt(n_part, 1_400_000), n_cust=dflt(n_cust, 3_000_000),
                     n_supp=dflt(n_supp, 200_000))
        r, r2, y = dg.draw(qs, 5, 0, 4), dg.draw(qs, 6, 0, 4), dg.draw(qs, 7, 1992, 1996)
        w.params = {"c_region": region_name(r), "s_region": region_name(r2), "year_lo": y}
        dt = dg.date_table()
        ct = dg.customer_table(w.n_cust, seed)
        st = dg.supplier_table(w.n_supp, seed)
        w.dims = {"date": [dt["datekey"], dt["year"], dt["month"]],
                  "customer": [ct["key"]] + geo_strings(ct),
                  "supplier": [st["key"]] + geo_strings(st)}
        nat = [(ValType.Int32, 4), (ValType.String, NATION_W)]
        w.dim_pipelines = [
            dim_pipeline("q5_date", "date", int_schema(3), "$(0.0),$(0.1)", f"$(0.1)>={y} && $(0.1)<={y + 2}"),
            dim_pipeline("q5_cust", "customer", w.dim_schema("customer"), "$(0.0),$(0.2)",
                         f'StrCmp($(0.3),"{region_name(r)}",{REGION_W})==0', out_cols=nat),
            dim_pipeline("q5_supp", "supplier", w.dim_schema("supplier"), "$(0.0),$(0.2)",
                         f'StrCmp($(0.3),"{region_name(r2)}",{REGION_W})==0', out_cols=nat),
        ]
        w.query = fact_pipeline("q5", "lineorder", w.fact_schema(), ["q5_date", "q5_cust", "q5_supp"],
                                [("$(0.0)", "$(1.0)"), ("$(0.5)", "$(2.0)"), ("$(0.6)", "$(3.0)")],
                                "$(2.1),$(3.1),$(1.1)", "$(0.7)-$(0.8)")
        w.key_num = 3
    elif config == 7:
        # Joined projection (no ReduceBy) over the four-dimension schema: the
        # rows of a discount band whose date, customer and supplier keys all
        # match, with columns from the fact table and every joined object.
        w = make(2, fact_rows=dflt(fact_rows, 6_000_000), seed=seed, tuple_per_bulk=tuple_per_bulk,
                 n_part=n_part, n_cust=n_cust, n_supp=n_supp, qseed=qs)
        w.config = 7
        w.query = join_map_pipeline("q7", "lineorder", w.fact_schema(), ["q2_date", "q2_cust", "q2_supp"],
                                    [("$(0.0)", "$(1.0)"), ("$(0.5)", "$(2.0)"), ("$(0.6)", "$(3.0)")],
                                    "$(0.0),$(1.1),$(2.1),$(3.1),$(0.7)-$(0.8),$(0.5)",
                                    predication="$(0.2)<=4")
        w.key_num = -1  # no ReduceBy: the result is rows (read_all)
    else:
        raise ValueError(f"no config {config}")
    return w


# ------------------------------------------------------------------ batched queries
_DATE_YEAR = None


def _year_days(y0: int, y1: int) -> int:
    global _DATE_YEAR
    if _DATE_YEAR is None:
        _DATE_YEAR = dg.date_table()["year"]
    return int(np.count_nonzero((_DATE_YEAR >= y0) & (_DATE_YEAR <= y1)))


def _u01(seed: int, stream: int) -> float:
    return dg.draw(seed, stream, 0, (1 << 30) - 1) / float(1 << 30)


@dataclass
class BatchQuery:
    shape: int                 # 0, 1, 2: shaped like configs 0, 1, 2
    row0: int                  # the query reads fact rows [row0, row0 + nrows)
    nrows: int
    selectivity: float         # drawn target fraction of rows that pass
    pipe: PipelineInfo
    key_num: int


@dataclass
class BatchWorkload:
    fact: Workload                                   # the config-2 fact table and its dimensions
    dim_pipelines: list = field(default_factory=list)  # distinct dimension pipelines, shared
    queries: list = field(default_factory=list)


def make_batch(nq: int = 256, *, fact_rows: int | None = None, seed: int = dg.DEFAULT_SEED,
               qseed: int | None = None, tuple_per_bulk: int | None = None, min_rows: int = 1_000_000,
               n_part: int | None = None, n_cust: int | None = None, n_supp: int | None = None) -> BatchWorkload:
    """`nq` seeded queries shaped like configs 0-2, each with its own predicate
    constants, over the config-2 fact table (9 columns):

      row range   log-uniform length in [min_rows, fact_rows], uniform start
      selectivity log-uniform in [1e-4, 0.5]: a fact-side extprice window
                  passes min(1, target / p) of the rows, p being the expected
                  pass rate of the shape's own dimension and fact predicates

    Fact rows are the view "lo_q<i>" of "lineorder"; dimension pipelines with
    equal text are shared between queries."""
    qs = seed if qseed is None else qseed
    base = make(2, fact_rows=fact_rows, seed=seed, tuple_per_bulk=tuple_per_bulk, n_part=n_part,
                n_cust=n_cust, n_supp=n_supp, qseed=qs)
    pt = dg.part_table(base.n_part, seed)
    base.dims["part"] = [pt["partkey"], pt["category"], pt["brand"]]
    bw = BatchWorkload(base)
    dims = {}

    def dim(name, table, ncols, proj, pred):
        if name not in dims:
            dims[name] = dim_pipeline(name, table, int_schema(ncols), proj, pred)
            bw.dim_pipelines.append(dims[name])
        return name

    n = base.fact_rows
    lo_rows = max(1, min(min_rows, n))
    ext_lo, ext_hi = dg.RANGES["extprice"]
    schema = base.fact_schema()
    for i in range(nq):
        st = 10_000 + 16 * i
        shape = dg.draw(qs, st, 0, 2)
        length = int(round(np.exp(np.log(lo_rows) + _u01(qs, st + 1) * (np.log(n) - np.log(lo_rows)))))
        length = max(1, min(n, length))
        row0 = dg.draw(qs, st + 2, 0, n - length)
        sel = float(np.exp(np.log(1e-4) + _u01(qs, st + 3) * (np.log(0.5) - np.log(1e-4))))
        if shape == 0:
            y, d, q = dg.draw(qs, st + 4, 1992, 1998), dg.draw(qs, st + 5, 0, 8), dg.draw(qs, st + 6, 20, 35)
            p = _year_days(y, y) / dg.N_DATE * 3 / 11 * (q - 1) / 50
            dims_used = [dim(f"b_date_y{y}", "date", 3, "$(0.0),$(0.1)", f"$(0.1)=={y}")]
            joins = [("$(0.0)", "$(1.0)")]
            keys, metric, key_num = "", "$(0.3)*$(0.2)", 0
            pred = [f"$(0.2)>={d}", f"$(0.2)<={d + 2}", f"$(0.1)<{q}"]
        elif shape == 1:
            c = dg.draw(qs, st + 4, 0, 24)
            p = 1 / 25
            dims_used = [dim("b_date", "date", 3, "$(0.0),$(0.1)", None),
                         dim(f"b_part_c{c}", "part", 3, "$(0.0),$(0.2)", f"$(0.1)=={c}")]
            joins = [("$(0.0)", "$(1.0)"), ("$(0.4)", "$(2.0)")]
            keys, metric, key_num = "$(1.1),$(2.1)", "$(0.7)", 2
            pred = []
        else:
            r, r2, y = dg.draw(qs, st + 4, 0, 4), dg.draw(qs, st + 5, 0, 4), dg.draw(qs, st + 6, 1992, 1996)
            p = _year_days(y, y + 2) / dg.N_DATE / 25
            dims_used = [dim(f"b_date_w{y}", "date", 3, "$(0.0),$(0.1)", f"$(0.1)>={y} && $(0.1)<={y + 2}"),
                         dim(f"b_cust_r{r}", "customer", 4, "$(0.0),$(0.2)", f"$(0.3)=={r}"),
                         dim(f"b_supp_r{r2}", "supplier", 4, "$(0.0),$(0.2)", f"$(0.3)=={r2}")]
            joins = [("$(0.0)", "$(1.0)"), ("$(0.5)", "$(2.0)"), ("$(0.6)", "$(3.0)")]
            keys, metric, key_num = "$(2.1),$(3.1),$(1.1)", "$(0.7)-$(0.8)", 3
            pred = []
        frac = min(1.0, sel / p)
        if frac < 1.0:
            span = ext_hi - ext_lo + 1
            width = max(1, int(round(frac * span)))
            w0 = ext_lo + dg.draw(qs, st + 7, 0, span - width)
            pred += [f"$(0.3)>={w0}", f"$(0.3)<={w0 + width - 1}"]
        pipe = fact_pipeline(f"bq{i}", f"lo_q{i}", schema, dims_used, joins, keys, metric,
                             predication=" && ".join(pred) or None)
        bw.queries.append(BatchQuery(shape, row0, length, sel, pipe, key_num))
    return bw


def load_batch(engine, bw: BatchWorkload, generate_on_device: bool = True, build_dims: bool = True):
    """Dimensions, the fact table, one view per query and (build_dims) the
    shared dimension pipelines' outputs."""
    load_engine(engine, bw.fact, generate_on_device=generate_on_device)
    for i, q in enumerate(bw.queries):
        engine.view(f"lo_q{i}", "lineorder", q.row0, q.nrows)
    if build_dims:
        for p in bw.dim_pipelines:
            engine.run(p)


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
    if generate_on_device and w.device_fact:
        gen_fact_on_device(engine, w, fact_id, row0)
    else:
        engine.put(fact_id, w.fact_host(row0, w.fact_rows))


def run_engine(engine, w: Workload):
    for p in w.dim_pipelines:
        engine.run(p)
    engine.run(w.query)
    return engine.result(w.query.id, w.key_num)


def ssb_like_text(rows: int, ncols: int, seed: int, width: int = 10) -> tuple[bytes, list]:
    """SSB-like text for the Loader: `rows` lines of `ncols` right-aligned
    decimals padded with spaces to `width` bytes, '|' after each field and
    '\\n' after each line ((width + 1) * ncols + 1 bytes a line).  Returns
    the text and the int64 columns it holds."""
    rng = np.random.default_rng(seed)
    vals = rng.integers(-10 ** 8, 10 ** 9, size=(rows, ncols), dtype=np.int64)
    buf = np.full((rows, ncols, width + 1), ord(" "), np.uint8)
    buf[:, :, width] = ord("|")
    a = np.abs(vals)
    for d in range(width - 1, -1, -1):
        digit = (a % 10).astype(np.uint8) + ord("0")
        show = (a > 0) | (d == width - 1)
        buf[:, :, d] = np.where(show, digit, buf[:, :, d])
        a //= 10
    # the minus sign before the first digit
    ndig = np.maximum(1, np.floor(np.log10(np.maximum(np.abs(vals), 1))).astype(int) + 1)
    neg = vals < 0
    r, c = np.nonzero(neg)
    buf[r, c, width - 1 - ndig[r, c]] = ord("-")
    lines = np.concatenate([buf.reshape(rows, -1), np.full((rows, 1), ord("\n"), np.uint8)], axis=1)
    return lines.tobytes(), [vals[:, k] for k in range(ncols)]


# ------------------------------------------------------------------ string edge cases
TAG_NAMES = [b"", b"AM", b"AMER", b"AMERICAN", b"AMERICA", b"Aa", b"BB", b"ZZZZZZZZ", b"\xe9t\xe9", b"amer",
             b"AMX", b"A"]


@dataclass
class StringEdgeWorkload(Workload):
    """String semantics the reference's generated code has, on a small star:
    tag (key, name S8, group S6) and a fact table (tagkey, mode S5, value).

      q6_tag   Filter StrCmp(name, "AMERICA", 8) == 0 -- true for "", "A",
               "AM", "AMER", "AMERICA" and "AMERICAN" (StrCmp stops at either
               NUL, com/cpp/cpu-runtime.hpp:37-45) -- or >= "B", == "Aa", or
               below "A" (signed chars: "\xe9t\xe9" is, "" is not);
               Map key, name (S8), group cut to S4 (StrCopy of 4 bytes)
      q6       Filter StrCmp(mode, "RAIL", 5) != 0 on the fact table; join
               tag; GROUP BY name, group, mode -- Hash keys, where "Aa" and
               "BB" collide (seed 31) and merge as in the reference
    """

    device_fact: bool = False

    def fact_schema(self) -> ObjectInfo:
        return create_schema([ValType.Int32, ValType.String, ValType.Int32], [4, 5, 4])

    def fact_host(self, row0: int, n: int) -> list[np.ndarray]:
        tk = dg.uniform(self.seed, 91, 0, len(TAG_NAMES) - 1, row0, n).astype(np.int32)
        modes = np.array([b"RAIL", b"AIR", b"SHIP", b"TRUCK", b"RAILS", b""], dtype="S5")
        mode = modes[dg.uniform(self.seed, 92, 0, len(modes) - 1, row0, n)]
        val = dg.uniform(self.seed, 93, -1000, 100_000, row0, n).astype(np.int32)
        return [tk, mode, val]

    def fact_bytes_per_row(self) -> int:
        return 12


def make_string_edges(fact_rows: int = 50_000, tuple_per_bulk: int = 20_000, seed: int = dg.DEFAULT_SEED):
    w = StringEdgeWorkload(6, fact_rows, tuple_per_bulk, seed)
    # group cut to 4 bytes pairs the tags (k + 1) // 2: "Aa" (5) and "BB" (6) share it
    groups = [f"G{((k + 1) // 2) % 3}#{((k + 1) // 2) % 2}{k:02d}".encode() for k in range(len(TAG_NAMES))]
    w.dims = {"tag": [np.arange(len(TAG_NAMES), dtype=np.int32), np.array(TAG_NAMES, dtype="S8"),
                      np.array(groups, dtype="S6")]}
    w.dim_pipelines = [dim_pipeline("q6_tag", "tag", w.dim_schema("tag"), "$(0.0),$(0.1),$(0.2)",
                                    'StrCmp($(0.1),"AMERICA",8)==0 || StrCmp($(0.1),"B",8)>=0 || '
                                    'StrCmp($(0.1),"Aa",8)==0 || StrCmp($(0.1),"A",8)<0',
                                    out_cols=[(ValType.Int32, 4), (ValType.String, 8), (ValType.String, 4)])]
    w.query = fact_pipeline("q6", "lineorder", w.fact_schema(), ["q6_tag"], [("$(0.0)", "$(1.0)")],
                            "$(1.1),$(1.2),$(0.1)", "$(0.2)", predication='StrCmp($(0.1),"RAIL",5)!=0')
    w.key_num = 3
    return w
