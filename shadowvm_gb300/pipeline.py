"""Builders for PipelineInfo, mirroring the reference's two front ends:

* `PipelineTest` -- the C++ test harness (test/test.hpp:78-149): AddOperator /
  SetMode on a PipelineInfo, plus `run()` on an Engine in place of
  PipelineTest::Run (which needs the reference's JIT).
* `PipelineBuilder` -- the Java DSL (java_vRDD/src/main/java/ShadowVM/
  PipelineBuilder.java:99-147): filter / map / joinWith / reduceBy / sink with
  `$name` column names rewritten to `$(table.col)` longest-name first
  (PipelineBuilder.java:57-97).
"""
from __future__ import annotations

import re
from dataclasses import dataclass, field

from .proto import ObjectInfo, OperatorInfo, OpType, PipelineInfo, ValType, create_schema


def str_split(s: str, sep: str) -> list[str]:
    """com/cpp/com.cu:79-93 (StrSplit): no trailing empty piece."""
    out, p1 = [], 0
    p2 = s.find(sep)
    while p2 != -1:
        out.append(s[p1:p2])
        p1 = p2 + len(sep)
        p2 = s.find(sep, p1)
    if p1 != len(s):
        out.append(s[p1:])
    return out


class PipelineTest:
    """test/test.hpp:78-149."""

    def __init__(self, pid: str):
        self.pipe_info = PipelineInfo(id=pid)

    def add_operator(self, typ: OpType, args: dict, output: ObjectInfo | None):
        self.pipe_info.workflow.append(OperatorInfo(id=self.pipe_info.id, type=OpType(typ),
                                                    args=dict(args), output=output))
        return self

    def add_pre(self, *ids: str):
        self.pipe_info.pre_pipeline_id.extend(ids)
        return self

    def set_mode(self, codegen: bool, debug: bool, is_gpu: bool = False):
        self.pipe_info.codegen, self.pipe_info.debug, self.pipe_info.isGPU = codegen, debug, is_gpu
        return self

    def run(self, engine):
        engine.run(self.pipe_info)
        return self.pipe_info.id


I32 = ValType.Int32
I64 = ValType.Int64
STR = ValType.String


def dim_pipeline(pid: str, source: str, src_schema: ObjectInfo, select: str, predication: str | None,
                 hash_col_size: int = 40, out_cols: list | None = None) -> PipelineInfo:
    """Dimension-side pipeline as the reference drivers write them
    (e.g. example/run_SSB_Q31.cu:11-25): Source -> [Filter] -> Map -> Sink,
    output = the selected columns (int32, or out_cols' (ValType, val_size)
    each, e.g. String copies) plus the trailing hash-table column."""
    n = len(str_split(select, ","))
    cols = out_cols or [(I32, 4)] * n
    out = create_schema([t for t, _ in cols] + [STR], [z for _, z in cols] + [hash_col_size])
    t = PipelineTest(pid).add_pre(source)
    t.add_operator(OpType.Source, {"type": "object"}, src_schema)
    if predication:
        t.add_operator(OpType.Filter, {"predication": predication}, out)
    t.add_operator(OpType.Map, {"select": select}, out)
    t.add_operator(OpType.Sink, {}, out)
    return t.pipe_info


def fact_pipeline(pid: str, source: str, src_schema: ObjectInfo, dims: list[str],
                  joins: list[tuple[str, str]], dim_keys: str, metric: str,
                  predication: str | None = None, metric_type: ValType = I64) -> PipelineInfo:
    """Fact pipeline: Source -> [Filter] -> JoinWith... -> ReduceBy -> Sink
    (example/run_SSB_Q31.cu:77-102).  Sink: int32 keys, one column per metric."""
    nk = len(str_split(dim_keys, ","))
    nm = len(str_split(metric, ","))
    out = create_schema([I32] * nk + [metric_type] * nm, [4] * nk + [8 if metric_type == I64 else 4] * nm)
    t = PipelineTest(pid).add_pre(source, *dims)
    t.add_operator(OpType.Source, {"type": "object"}, src_schema)
    if predication:
        t.add_operator(OpType.Filter, {"predication": predication}, out)
    for lk, rk in joins:
        t.add_operator(OpType.JoinWith, {"lkey": lk, "rkey": rk}, out)
    t.add_operator(OpType.ReduceBy, {"dim": dim_keys, "metric": metric}, out)
    t.add_operator(OpType.Sink, {}, out)
    return t.pipe_info


def join_map_pipeline(pid: str, source: str, src_schema: ObjectInfo, dims: list[str],
                      joins: list[tuple[str, str]], select: str, predication: str | None = None) -> PipelineInfo:
    """Joined projection: Source -> [Filter] -> JoinWith... -> Map -> Sink, no
    ReduceBy (the reference generates its join block, then its select block,
    codegen/codegen.cpp:121-180).  Sink: one int32 column per expression."""
    n = len(str_split(select, ","))
    out = create_schema([I32] * n, [4] * n)
    t = PipelineTest(pid).add_pre(source, *dims)
    t.add_operator(OpType.Source, {"type": "object"}, src_schema)
    if predication:
        t.add_operator(OpType.Filter, {"predication": predication}, out)
    for lk, rk in joins:
        t.add_operator(OpType.JoinWith, {"lkey": lk, "rkey": rk}, out)
    t.add_operator(OpType.Map, {"select": select}, out)
    t.add_operator(OpType.Sink, {}, out)
    return t.pipe_info


# ------------------------------------------------------------------ Java DSL mirror
@dataclass
class Table:
    """A named object with named columns (ObjectSchema in the Java front end).
    A column named None has no name; one named "" is known as `$UNKNOWN`
    (PipelineBuilder.java:60-66)."""
    id: str
    columns: list[str | None]
    schema: ObjectInfo = field(default_factory=ObjectInfo)


def _java_split(s: str, regex: str) -> list[str]:
    """java.lang.String.split(regex): trailing empty pieces dropped."""
    parts = re.split(regex, s)
    while len(parts) > 1 and parts[-1] == "":
        parts.pop()
    return parts


class PipelineBuilder:
    """java_vRDD/.../PipelineBuilder.java: the operator DSL."""

    def __init__(self, pid: str, source: Table, output: ObjectInfo):
        self.info = PipelineInfo(id=pid)
        self.output = output
        self.out_names: list[str | None] = [None] * len(output.column_list)  # set by map()
        self.tables: list[Table] = []
        self.names: dict[str, str] = {}
        self._add_table(source)
        self.info.workflow.append(OperatorInfo(id=pid, type=OpType.Source, args={"type": "object"},
                                               output=source.schema))

    def _add_table(self, t: Table):
        k = len(self.tables)
        self.tables.append(t)
        self.info.pre_pipeline_id.append(t.id)
        for c, name in enumerate(t.columns):
            if name is not None:  # a later table's column of the same name wins
                self.names["$" + name if name else "$UNKNOWN"] = f"$({k}.{c})"

    def replace(self, expr: str) -> str:
        """PipelineBuilder.replaceExpression: plain text replacement of every
        known `$name`, names in descending order (a TreeSet walked backwards),
        so a name goes before any shorter name that prefixes it."""
        for key in sorted(self.names, reverse=True):
            expr = expr.replace(key, self.names[key])
        return expr

    def _op(self, typ: OpType, args: dict):
        self.info.workflow.append(OperatorInfo(id=self.info.id, type=typ, args=args, output=self.output))
        return self

    def filter(self, cond: str):
        return self._op(OpType.Filter, {"predication": self.replace(cond)})

    def map(self, *cols: str):
        """Also names output column i as the DSL does (PipelineBuilder.java:
        106-117): the text after the `$`, or, when the rewritten expression
        splits on the regex "/." (a '/' and the character after it), the
        second piece."""
        out = []
        for i, c in enumerate(cols):
            new = self.replace(c)
            parts = _java_split(new[1:], "/.")
            if i < len(self.out_names):
                self.out_names[i] = c[1:] if len(parts) == 1 else parts[1]
            out.append(new)
        return self._op(OpType.Map, {"select": ",".join(out)})

    def join_with(self, table: Table, lkey: str, rkey: str):
        self._add_table(table)
        return self._op(OpType.JoinWith, {"lkey": self.replace(lkey), "rkey": self.replace(rkey)})

    def reduce_by(self, dim: str, metric: str):
        return self._op(OpType.ReduceBy, {"dim": self.replace(dim), "metric": self.replace(metric)})

    def sink(self) -> PipelineInfo:
        self._op(OpType.Sink, {})
        return self.info

    def table(self) -> Table:
        """This pipeline's output as a table another builder can join: its id
        and the column names map() gave (Pipeline.schema() in the DSL)."""
        return Table(self.info.id, list(self.out_names), self.output)
