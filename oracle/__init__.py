"""ORACLE -- test infrastructure, never the product.

A CPU restatement of the reference's query path used to check the GPU library:
``codegen.py`` emits the reference's generated host loop for a pipeline,
``driver.cpp`` runs it bulk by bulk the way core/pipeline.cu does, and
``sql_exact.py`` is an independent NumPy evaluation of the same SQL.

Two builds of the generated-code path exist:

* ``mode="port"``: codegen.py's text compiled against ``svm_port_runtime.h``
  (this repository's restatement of the reference runtime).  Builds anywhere
  with g++; it is the CPU baseline timed by ``bench.py``.
* ``mode="ref"``: the reference's OWN CodeGen (``oracle/_ref/ref_codegen``)
  compiled against the reference's own runtime headers (``oracle/_ref``, built
  by ``build_ref.sh`` from the reference tree; x86 only).  Used to pin the port
  and to generate the committed golden fixtures.

Only ``tests/``, ``__graft_entry__.smoke`` and ``bench.py``'s CPU legs may
import this package.
"""
from __future__ import annotations

import ctypes
import hashlib
import os
import subprocess
import threading
from dataclasses import dataclass

import numpy as np

from shadowvm_gb300.proto import ObjectInfo, OpType, PipelineInfo, ValType

from . import codegen

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF = os.path.join(HERE, "_ref")
# The reference source tree: SVM_REFERENCE_DIR, else a directory named
# "reference" beside the repository.
REFERENCE_TREE = os.environ.get("SVM_REFERENCE_DIR") or os.path.normpath(os.path.join(HERE, "..", "..", "reference"))

_lock = threading.Lock()
_libs: dict[str, ctypes.CDLL] = {}
_fns: dict[str, ctypes._CFuncPtr] = {}

CXX_FLAGS = ["-w", "-O2", "-std=c++11", "-fPIC", "-shared"]  # codegen/compiler.cpp:30


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{r.stderr[-4000:]}")


def build_port() -> str:
    """Compile the driver against the port runtime; returns the library path."""
    os.makedirs(os.path.join(BUILD, "q"), exist_ok=True)
    out = os.path.join(BUILD, "libsvm_oracle_port.so")
    src = [os.path.join(HERE, "driver.cpp"), os.path.join(HERE, "svm_port_runtime.h")]
    if not os.path.exists(out) or os.path.getmtime(out) < max(os.path.getmtime(s) for s in src):
        _run(["g++", "-O2", "-std=c++11", "-fPIC", "-shared", "-pthread", f"-I{HERE}",
              '-DSVM_ORACLE_RUNTIME="svm_port_runtime.h"', src[0], "-o", out + ".tmp"])
        os.replace(out + ".tmp", out)
    return out


def build_loader() -> str:
    """Compile the Loader restatement (loader.c); returns the library path."""
    os.makedirs(BUILD, exist_ok=True)
    out = os.path.join(BUILD, "libsvm_oracle_loader.so")
    src = os.path.join(HERE, "loader.c")
    if not os.path.exists(out) or os.path.getmtime(out) < os.path.getmtime(src):
        _run(["gcc", "-O2", "-fPIC", "-shared", src, "-o", out + ".tmp"])
        os.replace(out + ".tmp", out)
    return out


def load_text(text: bytes, types: list, col_delim: str = "|", row_delim: str = "\n", cap_rows: int | None = None):
    """The reference Loader over `text` (restated in loader.c): returns
    (rows, [column arrays]); raises ValueError for an item over 4095 bytes."""
    lib = ctypes.CDLL(build_loader())
    f = lib.svm_oracle_load_text
    f.restype = ctypes.c_longlong
    f.argtypes = [ctypes.c_char_p, ctypes.c_ulonglong, ctypes.c_char, ctypes.c_char, ctypes.c_int,
                  ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_void_p), ctypes.c_ulonglong]
    if cap_rows is None:
        cap_rows = text.count(row_delim.encode())
    cols = [np.zeros(cap_rows + 1, np.int64 if int(t) == 3 else np.int32) for t in types]
    ptrs = (ctypes.c_void_p * len(cols))(*[c.ctypes.data for c in cols])
    tt = (ctypes.c_int * len(types))(*[int(t) for t in types])
    n = f(text, len(text), col_delim.encode(), row_delim.encode(), len(types), tt, ptrs, cap_rows)
    if n < 0:
        raise ValueError("an item longer than 4095 bytes")
    return n, [c[:min(n, cap_rows)] for c in cols]


def ref_available() -> bool:
    return os.path.exists(os.path.join(REF, "libsvm_oracle_ref.so")) and \
        os.path.exists(os.path.join(REF, "ref_codegen"))


def build_ref() -> str:
    """Build oracle/_ref from the reference tree (x86, reference present)."""
    _run(["bash", os.path.join(HERE, "build_ref.sh")])
    return REF


def _driver(mode: str) -> ctypes.CDLL:
    with _lock:
        if mode in _libs:
            return _libs[mode]
        path = build_port() if mode == "port" else os.path.join(REF, "libsvm_oracle_ref.so")
        lib = ctypes.CDLL(path)
        vp, u64, i32 = ctypes.c_void_p, ctypes.c_ulonglong, ctypes.c_int
        lib.svmo_object_new.restype = vp
        lib.svmo_object_new.argtypes = [i32, ctypes.POINTER(i32), ctypes.POINTER(u64)]
        lib.svmo_object_free.argtypes = [vp]
        lib.svmo_object_add_bulk.restype = i32
        lib.svmo_object_add_bulk.argtypes = [vp, u64, u64]
        lib.svmo_object_nbulks.restype = i32
        lib.svmo_object_nbulks.argtypes = [vp]
        lib.svmo_bulk_column.restype = vp
        lib.svmo_bulk_column.argtypes = [vp, i32, i32]
        lib.svmo_bulk_tuple_count.restype = u64
        lib.svmo_bulk_tuple_count.argtypes = [vp, i32]
        lib.svmo_run_pipeline.restype = vp
        lib.svmo_run_pipeline.argtypes = [
            vp, vp, i32, ctypes.POINTER(vp), i32, ctypes.POINTER(i32), ctypes.POINTER(i32),
            i32, ctypes.POINTER(i32), ctypes.POINTER(u64), u64, i32, i32, i32, i32,
            ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), ctypes.POINTER(i32)]
        _libs[mode] = lib
        return lib


# ------------------------------------------------------------------ objects
_NP = {ValType.Int32: np.int32, ValType.Int64: np.int64, ValType.Int16: np.int16}


def _dtype(col) -> np.dtype:
    """NumPy type of a column: its int type, or val_size raw bytes for a String."""
    if col.type == ValType.String:
        return np.dtype(f"S{int(col.val_size)}")
    return np.dtype(_NP[col.type])


def _view(addr: int, dtype, n: int) -> np.ndarray:
    if n == 0:
        return np.zeros(0, dtype)
    buf = (ctypes.c_char * (n * np.dtype(dtype).itemsize)).from_address(addr)
    return np.frombuffer(buf, dtype=dtype, count=n)


class Obj:
    """A reference-style object: bulks of columns in the driver's memory."""

    def __init__(self, schema: ObjectInfo, mode: str, handle=None):
        self.schema = schema
        self.mode = mode
        self.lib = _driver(mode)
        n = len(schema.column_list)
        types = (ctypes.c_int * n)(*[int(c.type) for c in schema.column_list])
        sizes = (ctypes.c_ulonglong * n)(*[int(c.val_size) for c in schema.column_list])
        self.h = handle if handle is not None else self.lib.svmo_object_new(n, types, sizes)
        if not self.h:
            raise ValueError("bad schema")

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self.lib.svmo_object_free(h)
            self.h = None

    @classmethod
    def from_columns(cls, cols: list[np.ndarray], schema: ObjectInfo, tuple_per_bulk: int, mode: str):
        """Split equal-length int columns into bulks of tuple_per_bulk rows
        (an empty table has no bulks, like an object with no data)."""
        o = cls(schema, mode)
        n = len(cols[0]) if cols else 0
        for b0 in range(0, n, tuple_per_bulk):
            cnt = min(tuple_per_bulk, n - b0)
            b = o.lib.svmo_object_add_bulk(o.h, tuple_per_bulk, cnt)
            if b < 0:
                raise MemoryError("oracle bulk allocation failed")
            for c, arr in enumerate(cols):
                t = _dtype(schema.column_list[c])
                dst = _view(o.lib.svmo_bulk_column(o.h, b, c), t, cnt)
                dst[:] = np.asarray(arr[b0:b0 + cnt], dtype=t)
        return o

    def nbulks(self) -> int:
        return self.lib.svmo_object_nbulks(self.h)

    def column(self, bulk: int, col: int) -> np.ndarray:
        t = _dtype(self.schema.column_list[col])
        n = self.lib.svmo_bulk_tuple_count(self.h, bulk)
        return _view(self.lib.svmo_bulk_column(self.h, bulk, col), t, n).copy()

    def concat(self, col: int) -> np.ndarray:
        return np.concatenate([self.column(b, col) for b in range(self.nbulks())]) if self.nbulks() else \
            np.zeros(0, _dtype(self.schema.column_list[col]))


# ------------------------------------------------------------------ codegen
def ref_codegen(info: PipelineInfo, ref_infos: list[ObjectInfo]) -> str:
    """Generated host code from the reference's own CodeGen (oracle/_ref)."""
    def sch(o: ObjectInfo) -> str:
        return "\t".join(f"{int(c.type)}:{int(c.val_size)}" for c in o.column_list)
    src = [op.output for op in info.workflow if op.type == OpType.Source][0]
    sink = [op.output for op in info.workflow if op.type == OpType.Sink][0]
    lines = [f"id\t{info.id}", f"schema\t0\t{sch(src)}"]
    lines += [f"schema\t{k + 1}\t{sch(o)}" for k, o in enumerate(ref_infos)]
    lines.append(f"out\t{sch(sink)}")
    for op in info.workflow:
        if op.type == OpType.Filter:
            lines.append(f"filter\t{op.args['predication']}")
        elif op.type == OpType.Map:
            lines.append(f"select\t{op.args['select']}")
        elif op.type == OpType.ReduceBy:
            lines.append(f"reduce\t{op.args.get('dim', '')}\t{op.args['metric']}")
        elif op.type == OpType.JoinWith:
            lines.append(f"join\t{op.args['lkey']}\t{op.args['rkey']}")
    r = subprocess.run([os.path.join(REF, "ref_codegen")], input="\n".join(lines) + "\n",
                       capture_output=True, text=True, check=True)
    return r.stdout


def port_codegen(info: PipelineInfo, ref_infos: list[ObjectInfo], includes=None) -> str:
    bp = codegen.bind(info, ref_infos)
    return codegen.export_host_code([codegen.gen_host_function(bp)],
                                    codegen.REFERENCE_INCLUDES if includes is None else includes)


def compile_query(code: str, mode: str) -> str:
    """Compile generated host code with the reference's flags; cached by hash."""
    d = os.path.join(BUILD if mode == "port" else REF, "q")
    os.makedirs(d, exist_ok=True)
    key = code
    if mode == "port":  # a changed runtime header recompiles
        with open(os.path.join(HERE, "svm_port_runtime.h")) as f:
            key += f.read()
    h = hashlib.sha1(key.encode()).hexdigest()[:20]
    so = os.path.join(d, f"q{h}.so")
    if not os.path.exists(so):
        src = os.path.join(d, f"q{h}.cpp")
        with open(src, "w") as f:
            f.write(code)
        inc = HERE if mode == "port" else os.path.join(REFERENCE_TREE, "com", "cpp")
        _run(["g++", *CXX_FLAGS, f"-I{inc}", src, "-o", so + ".tmp"])
        os.replace(so + ".tmp", so)
    return so


def query_function(info: PipelineInfo, ref_infos: list[ObjectInfo], mode: str):
    if mode == "port":
        code = port_codegen(info, ref_infos, codegen.PORT_INCLUDES)
    else:
        code = ref_codegen(info, ref_infos)
    so = compile_query(code, mode)
    with _lock:
        if so not in _fns:
            lib = ctypes.CDLL(so)
            _libs["q:" + so] = lib
            _fns[so] = getattr(lib, info.id)
        return _fns[so]


# ------------------------------------------------------------------ run
@dataclass
class RunStats:
    open_ms: float
    compute_ms: float


def run_pipeline(info: PipelineInfo, source: Obj, refs: list[Obj], tuple_per_bulk: int,
                 threads: int = 1, mode: str = "port") -> tuple[Obj, RunStats]:
    """One pipeline through generated code, as PipelineTest::Run (test/test.hpp:122-146)."""
    bp = codegen.bind(info, [r.schema for r in refs])
    fn = query_function(info, [r.schema for r in refs], mode)
    lib = _driver(mode)
    nref = len(refs)
    ref_arr = (ctypes.c_void_p * max(nref, 1))(*[r.h for r in refs])
    nj = len(bp.join_rkey)
    jo = (ctypes.c_int * max(nj, 1))(*[k.obj for k in bp.join_rkey])
    jc = (ctypes.c_int * max(nj, 1))(*[k.col for k in bp.join_rkey])
    out = bp.output_info
    no = len(out.column_list)
    ot = (ctypes.c_int * no)(*[int(c.type) for c in out.column_list])
    os_ = (ctypes.c_ulonglong * no)(*[int(c.val_size) for c in out.column_list])
    om, cm, st = ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
    h = lib.svmo_run_pipeline(ctypes.cast(fn, ctypes.c_void_p), source.h, nref, ref_arr, nj, jo, jc,
                              no, ot, os_, tuple_per_bulk, int(bp.is_reduce), len(bp.reduce_key),
                              len(bp.metric_exp), threads, ctypes.byref(om), ctypes.byref(cm),
                              ctypes.byref(st))
    if not h:
        raise RuntimeError(f"oracle pipeline {info.id} failed with status {st.value}")
    return Obj(out, mode, handle=h), RunStats(om.value, cm.value)


def merge_groups(sink: Obj, key_num: int, metric_num: int):
    """Merge the per-bulk reduced runs and sort by key (the documented
    deviation from core/pipeline.cu:322-328, which keeps one run per bulk).
    Returns (keys int32 [g, key_num], sums int64 [g, metric_num])."""
    ks = [sink.concat(k).astype(np.int64) for k in range(key_num)]
    ms = [sink.concat(key_num + m) for m in range(metric_num)]
    wide = [sink.schema.column_list[key_num + m].val_size == 8 for m in range(metric_num)]
    if sink.nbulks() == 0:
        return np.zeros((0, key_num), np.int32), np.zeros((0, metric_num), np.int64)
    if key_num == 0:
        sums = []
        for m in range(metric_num):
            s = int(ms[m].astype(np.int64).sum(dtype=np.int64)) if len(ms[m]) else 0
            sums.append(s if wide[m] else int(np.int64(s).astype(np.int32)))
        return np.zeros((1, 0), np.int32), np.array([sums], np.int64)
    if len(ks[0]) == 0:
        return np.zeros((0, key_num), np.int32), np.zeros((0, metric_num), np.int64)
    kmat = np.stack(ks, axis=1)
    uniq, inv = np.unique(kmat, axis=0, return_inverse=True)
    inv = inv.reshape(-1)
    sums = np.zeros((len(uniq), metric_num), np.int64)
    for m in range(metric_num):
        with np.errstate(over="ignore"):
            np.add.at(sums[:, m], inv, ms[m].astype(np.int64))
        if not wide[m]:
            sums[:, m] = sums[:, m].astype(np.int32)
    return uniq.astype(np.int32), sums


# ------------------------------------------------------------------ workloads
def run_workload(w, mode: str = "port", threads: int = 1, fact: list | None = None):
    """A whole workload (shadowvm_gb300.workloads) through the generated-code
    path: the dimension pipelines, then the fact pipeline, as the reference's
    drivers run them (example/run_SSB_Q31.cu:77-107).  Returns
    ((keys, sums), RunStats of the fact pipeline)."""
    from shadowvm_gb300.workloads import schema_of
    tpb = w.tuple_per_bulk
    objs = {name: Obj.from_columns(cols, schema_of(cols), tpb, mode) for name, cols in w.dims.items()}
    fact = w.fact_host(0, w.fact_rows) if fact is None else fact
    objs["lineorder"] = Obj.from_columns(fact, w.fact_schema(), tpb, mode)
    for p in w.dim_pipelines:
        out, _ = run_pipeline(p, objs[p.pre_pipeline_id[0]], [], tpb, threads, mode)
        objs[p.id] = out
    q = w.query
    sink, stats = run_pipeline(q, objs[q.pre_pipeline_id[0]], [objs[i] for i in q.pre_pipeline_id[1:]],
                               tpb, threads, mode)
    return merge_groups(sink, w.key_num, w.metric_num), stats


def run_workload_rows(w, mode: str = "port", threads: int = 1, fact: list | None = None):
    """A workload whose fact pipeline has no ReduceBy (a joined projection):
    its output columns, rows in order bulk by bulk as the reference's
    TransformTask writes them (core/pipeline.cu:262-344)."""
    from shadowvm_gb300.workloads import schema_of
    tpb = w.tuple_per_bulk
    objs = {name: Obj.from_columns(cols, schema_of(cols), tpb, mode) for name, cols in w.dims.items()}
    fact = w.fact_host(0, w.fact_rows) if fact is None else fact
    objs["lineorder"] = Obj.from_columns(fact, w.fact_schema(), tpb, mode)
    for p in w.dim_pipelines:
        out, _ = run_pipeline(p, objs[p.pre_pipeline_id[0]], [], tpb, threads, mode)
        objs[p.id] = out
    q = w.query
    sink, _ = run_pipeline(q, objs[q.pre_pipeline_id[0]], [objs[i] for i in q.pre_pipeline_id[1:]],
                           tpb, threads, mode)
    ncols = len([op.output for op in q.workflow if op.type == OpType.Sink][0].column_list)
    return [sink.concat(c) for c in range(ncols)]


def exact_workload_rows(w, fact: list | None = None):
    """The joined projection through sql_exact (every dimension row joinable)."""
    from . import sql_exact
    objs = {name: list(cols) for name, cols in w.dims.items()}
    for p in w.dim_pipelines:
        objs[p.id] = sql_exact.run_select(p, objs[p.pre_pipeline_id[0]])
    q = w.query
    fact = w.fact_host(0, w.fact_rows) if fact is None else fact
    return sql_exact.run_join_select(q, fact, [objs[i] for i in q.pre_pipeline_id[1:]])


def exact_workload(w, fact: list | None = None):
    """The same workload through sql_exact (every dimension row joinable)."""
    from . import sql_exact
    objs = {name: list(cols) for name, cols in w.dims.items()}
    for p in w.dim_pipelines:
        objs[p.id] = sql_exact.run_select(p, objs[p.pre_pipeline_id[0]])
    q = w.query
    fact = w.fact_host(0, w.fact_rows) if fact is None else fact
    return sql_exact.run_reduce(q, fact, [objs[i] for i in q.pre_pipeline_id[1:]])
