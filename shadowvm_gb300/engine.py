"""Python host API over the C ABI: a data-plane context (`Engine`), its object
store, and pipeline execution.  The reference equivalents are the
ObjectStore / cached_obj map and ShadowVMService::RunPipelineCMD
(object/store.cpp:49-91, service/service.cu:25-63)."""
from __future__ import annotations

import ctypes

import numpy as np

from . import capi
from .proto import OpType, PipelineInfo, ValType


class Engine:
    """One data-plane context on one GPU."""

    def __init__(self, device: int = 0, tuple_per_bulk: int = 2_000_000, join_mode: str = "ref_compat",
                 hbm_budget_bytes: int = 0, hash_char_signed: bool = True, batch_policy: str = "auto",
                 autotune: bool = True):
        self.lib = capi.load()
        cfg = capi.svm_config()
        self.lib.svm_config_default(ctypes.byref(cfg))
        cfg.device = device
        cfg.tuple_per_bulk = tuple_per_bulk
        cfg.join_mode = {"ref_compat": capi.JOIN_REF_COMPAT, "exact": capi.JOIN_EXACT}[join_mode]
        cfg.hbm_budget_bytes = hbm_budget_bytes
        cfg.hash_char_signed = int(hash_char_signed)
        cfg.batch_policy = {"auto": 0, "always": 1, "never": 2}[batch_policy]
        cfg.autotune = int(autotune)
        h = ctypes.c_void_p()
        st = self.lib.svm_init(ctypes.byref(cfg), ctypes.byref(h))
        if st != capi.OK:
            raise capi.SvmError(st, "svm_init failed (is a CUDA device visible?)")
        self.h = h
        self.tuple_per_bulk = tuple_per_bulk
        self.join_mode = join_mode
        self._host_cols = {}  # host-resident objects' arrays, kept alive while the objects exist

    def close(self):
        if getattr(self, "h", None):
            self.lib.svm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ------------------------------------------------------------ plumbing
    def _check(self, st: int):
        if st != capi.OK:
            raise capi.SvmError(st, (self.lib.svm_last_error(self.h) or b"").decode())

    @property
    def stream(self) -> int:
        return self.lib.svm_stream(self.h)

    def bytes_in_use(self) -> int:
        return self.lib.svm_bytes_in_use(self.h)

    # ------------------------------------------------------------ objects
    def put(self, oid: str, columns, on_device: bool = False, nrows: int | None = None):
        """Store host arrays (int32/int64 numpy, or fixed-width bytes 'S<w>'
        for String columns of width w) or device pointers as object `oid`.
        A None column is left zeroed (int32; pass nrows when every column is None)."""
        n = len(columns)
        if on_device:
            ptrs = [ctypes.c_void_p(int(c[0])) for c in columns]  # (ptr, dtype, nrows)
            types = [capi_type(c[1]) for c in columns]
            nrows = int(columns[0][2]) if n else 0
            keep = None
        else:
            keep = [None if c is None else np.ascontiguousarray(c) for c in columns]
            types = [int(ValType.String) if c is not None and c.dtype.kind == "S" else
                     capi_type(np.int32 if c is None else c.dtype) for c in keep]
            lens = {len(c) for c in keep if c is not None}
            if len(lens) > 1:
                raise ValueError("columns differ in length")
            nrows = lens.pop() if lens else (nrows or 0)
            ptrs = [ctypes.c_void_p(None if c is None else c.ctypes.data) for c in keep]
        pa = (ctypes.c_void_p * n)(*ptrs)
        if not on_device and any(c is not None and c.dtype.kind == "S" for c in keep):
            descs = (capi.svm_column_desc * n)(*[
                capi.svm_column_desc(int(ValType.String), c.dtype.itemsize) if c is not None and c.dtype.kind == "S"
                else capi.svm_column_desc(t, 8 if t == int(ValType.Int64) else 4) for c, t in zip(keep, types)])
            self._check(self.lib.svm_object_put_columns(self.h, oid.encode(), n, descs, nrows, pa, 0))
            return
        t = (ctypes.c_int * n)(*types)
        self._check(self.lib.svm_object_put(self.h, oid.encode(), n, t, nrows, pa, int(on_device)))
        self._host_cols.pop(oid, None)
        del keep

    def put_host(self, oid: str, columns):
        """Store page-locked host arrays (int32/int64 numpy views of pinned
        memory, e.g. a pinned torch tensor's .numpy()) as object `oid`, read
        in place (svm_object_put_host).  The arrays are kept referenced until
        the object is dropped or replaced; a None column is absent."""
        n = len(columns)
        lens = {len(c) for c in columns if c is not None}
        if len(lens) > 1:
            raise ValueError("columns differ in length")
        nrows = lens.pop() if lens else 0
        for c in columns:
            if c is not None and not c.flags["C_CONTIGUOUS"]:
                raise ValueError("host-resident columns must be contiguous")
        types = (ctypes.c_int * n)(*[capi_type(np.int32 if c is None else c.dtype) for c in columns])
        pa = (ctypes.c_void_p * n)(*[ctypes.c_void_p(None if c is None else c.ctypes.data) for c in columns])
        self._check(self.lib.svm_object_put_host(self.h, oid.encode(), n, types, nrows, pa))
        self._host_cols[oid] = list(columns)

    def create(self, oid: str, ncols: int, nrows: int, dtype=np.int32):
        t = (ctypes.c_int * ncols)(*([capi_type(np.dtype(dtype))] * ncols))
        self._check(self.lib.svm_object_put(self.h, oid.encode(), ncols, t, nrows, None, 0))

    def gen_uniform(self, oid: str, col: int, seed: int, stream: int, lo: int, hi: int, lookup=None,
                    row0: int = 0):
        """Device-side datagen.uniform(seed, stream, lo, hi, row0, nrows) (optionally
        mapped through `lookup`)."""
        lut = None
        if lookup is not None:
            arr = np.ascontiguousarray(lookup, dtype=np.int32)
            assert len(arr) == hi - lo + 1
            lut = arr.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        self._check(self.lib.svm_object_gen_uniform(self.h, oid.encode(), col, seed & (2**64 - 1),
                                                    stream, row0, lo, hi, lut))

    def kernel_launches(self) -> int:
        return self.lib.svm_kernel_launches()

    def view(self, oid: str, base: str, row0: int, nrows: int):
        self._check(self.lib.svm_object_view(self.h, oid.encode(), base.encode(), row0, nrows))

    def info(self, oid: str) -> tuple[int, int]:
        nc, nr = ctypes.c_int(), ctypes.c_ulonglong()
        self._check(self.lib.svm_object_info(self.h, oid.encode(), ctypes.byref(nc), ctypes.byref(nr)))
        return nc.value, nr.value

    def types(self, oid: str) -> list[int]:
        nc, _ = self.info(oid)
        t = (ctypes.c_int * max(nc, 1))()
        self._check(self.lib.svm_object_types(self.h, oid.encode(), t, nc))
        return list(t)[:nc]

    def columns(self, oid: str) -> list[tuple[int, int]]:
        """(ValType, val_size) of each column (a String column's width in bytes)."""
        nc, _ = self.info(oid)
        d = (capi.svm_column_desc * max(nc, 1))()
        self._check(self.lib.svm_object_columns(self.h, oid.encode(), d, nc))
        return [(d[k].type, d[k].val_size) for k in range(nc)]

    def read(self, oid: str, col: int, row0: int = 0, n: int | None = None) -> np.ndarray:
        """Rows of one column: int32 / int64, or 'S<w>' bytes for a String column."""
        _, nr = self.info(oid)
        n = nr - row0 if n is None else n
        t, w = self.columns(oid)[col]
        dt = np.dtype(f"S{w}") if t == ValType.String else np.int64 if t == ValType.Int64 else np.int32
        out = np.empty(n, dt)
        self._check(self.lib.svm_object_read(self.h, oid.encode(), col, row0, n,
                                             out.ctypes.data_as(ctypes.c_void_p)))
        return out

    def read_all(self, oid: str) -> list[np.ndarray]:
        nc, _ = self.info(oid)
        return [self.read(oid, c) for c in range(nc)]

    def load_text(self, oid: str, text, types: list, col_delim: str = "|", row_delim: str = "\n",
                  device_ptr: int | None = None, nbytes: int | None = None) -> int:
        """Delimited text -> object `oid` on the device, as the reference's
        Loader operator parses it; returns rows.  `text` is host bytes (or a
        buffer), or pass device_ptr / nbytes for text already on the device."""
        t = (ctypes.c_int * len(types))(*[int(x) for x in types])
        n = ctypes.c_ulonglong()
        if device_ptr is not None:
            ptr, size, on_dev = ctypes.c_void_p(device_ptr), nbytes, 1
        else:
            buf = np.frombuffer(memoryview(text), np.uint8) if not isinstance(text, np.ndarray) else text
            ptr, size, on_dev = buf.ctypes.data_as(ctypes.c_void_p), buf.nbytes, 0
        self._check(self.lib.svm_object_load_text(self.h, oid.encode(), len(types), t, ptr, size, on_dev,
                                                  col_delim.encode(), row_delim.encode(), ctypes.byref(n)))
        return n.value

    def read_objects(self, oids: list[str], types: list[list[int]]) -> list[list[np.ndarray]]:
        """Whole objects in one device pass (svm_objects_read); types[k] lists
        object k's column types (ValType.Int32 / Int64)."""
        n = len(oids)
        if n == 0:
            return []
        ids = (ctypes.c_char_p * n)(*[o.encode() for o in oids])
        rows = (ctypes.c_ulonglong * n)()
        need = ctypes.c_ulonglong()
        self._check(self.lib.svm_objects_read(self.h, n, ids, None, 0, rows, ctypes.byref(need)))
        buf = np.empty(max(need.value, 8), np.uint8)
        self._check(self.lib.svm_objects_read(self.h, n, ids, buf.ctypes.data_as(ctypes.c_void_p), buf.nbytes, rows,
                                              ctypes.byref(need)))
        out, off = [], 0
        for k in range(n):
            cols = []
            for t in types[k]:
                dt = np.int64 if t == ValType.Int64 else np.int32
                nb = rows[k] * np.dtype(dt).itemsize
                cols.append(buf[off:off + nb].view(dt).copy())
                off += (nb + 7) & ~7
            out.append(cols)
        return out

    def device_ptr(self, oid: str, col: int) -> int:
        p = ctypes.c_void_p()
        self._check(self.lib.svm_object_device_ptr(self.h, oid.encode(), col, ctypes.byref(p)))
        return p.value

    def drop(self, oid: str):
        self._check(self.lib.svm_object_drop(self.h, oid.encode()))
        self._host_cols.pop(oid, None)

    # ------------------------------------------------------------ pipelines
    def run(self, pipe):
        """RunPipelineCMD: the output is stored as object `pipe.id`.  `pipe` is
        a PipelineInfo or a Prepared one (marshalled once, run many times)."""
        p = pipe if isinstance(pipe, Prepared) else Prepared([pipe])
        self._check(self.lib.svm_run_pipeline(self.h, ctypes.byref(p.arr[0])))

    def run_batch(self, pipes):
        """Many pipelines in one call (svm_run_batch); a list of PipelineInfo
        or a Prepared batch."""
        p = pipes if isinstance(pipes, Prepared) else Prepared(pipes)
        self._check(self.lib.svm_run_batch(self.h, p.n, p.arr))

    def batch_begin(self, pipes, host_results: bool = False) -> "Fold":
        """Enqueues a fold without waiting for its device work
        (svm_batch_begin); complete it with Fold.wait / Fold.release."""
        p = pipes if isinstance(pipes, Prepared) else Prepared(pipes)
        h = ctypes.c_void_p()
        self._check(self.lib.svm_batch_begin(self.h, p.n, p.arr, int(host_results), ctypes.byref(h)))
        return Fold(self, h, p)

    def footprint(self, pipe) -> int:
        """Device bytes running `pipe` needs beyond what is resident (plans it;
        joined dimension tables are built and cached)."""
        p = pipe if isinstance(pipe, Prepared) else Prepared([pipe])
        b = ctypes.c_ulonglong()
        self._check(self.lib.svm_pipeline_footprint(self.h, ctypes.byref(p.arr[0]), ctypes.byref(b)))
        return b.value

    def result(self, oid: str, key_num: int) -> tuple[np.ndarray, np.ndarray]:
        """A reduce pipeline's output: keys int32 [g, key_num], sums int64 [g, m]."""
        cols = self.read_all(oid)
        g = len(cols[0]) if cols else 0
        keys = np.stack(cols[:key_num], axis=1).astype(np.int32) if key_num else np.zeros((g, 0), np.int32)
        mets = np.stack([c.astype(np.int64) for c in cols[key_num:]], axis=1) if len(cols) > key_num else \
            np.zeros((g, 0), np.int64)
        return keys, mets

    # ------------------------------------------------------------ profiling
    def pin_launch(self, rows_per_lane: int = -1, ring_stages: int = 0, tables_staged: int = -1,
                   blocks_per_sm: int = 0):
        """Narrows the fused scan's launch configurations (svm_pin_launch);
        the defaults lift every pin."""
        self._check(self.lib.svm_pin_launch(self.h, rows_per_lane, blocks_per_sm, ring_stages, tables_staged))

    def pin_list_after(self, list_after: int = -1):
        """Narrows the compiled scan's row-list form (svm_pin_list_after):
        -1 any, 0..2 the step after which later steps run over a list of
        the live rows, 3 none, 4 a list after step 0 with steps 1 and 2
        over it in one pass."""
        self._check(self.lib.svm_pin_list_after(self.h, list_after))

    def pin_batch_launch(self, consumer_warps: int = 0, ring_stages: int = 0):
        """Narrows the merged batch kernel's launch configurations
        (svm_pin_batch_launch); the defaults lift every pin."""
        self._check(self.lib.svm_pin_batch_launch(self.h, consumer_warps, ring_stages))

    def last_launch(self) -> dict:
        """The last fused scan's launch configuration (svm_last_launch)."""
        import json
        buf = ctypes.create_string_buffer(1024)
        self._check(self.lib.svm_last_launch(self.h, buf, len(buf)))
        return json.loads(buf.value.decode()) if buf.value else {}

    def test_device_wait(self, wait_polls: int = 0, stall_copies: bool = False):
        """Test hook: the fused scan's mbarrier poll limit (0 = default) and
        whether its copy warp issues no copies (svm_test_device_wait)."""
        self._check(self.lib.svm_test_device_wait(self.h, wait_polls, int(stall_copies)))

    def profile(self, on: bool = True):
        self._check(self.lib.svm_profile_enable(self.h, int(on)))

    def profile_reset(self):
        self._check(self.lib.svm_profile_reset(self.h))

    def profile_read(self, cls: int) -> tuple[int, float]:
        n, ms = ctypes.c_ulonglong(), ctypes.c_double()
        self._check(self.lib.svm_profile_read(self.h, cls, ctypes.byref(n), ctypes.byref(ms)))
        return n.value, ms.value


def capi_type(dtype) -> int:
    dt = np.dtype(dtype)
    if dt == np.int32:
        return int(ValType.Int32)
    if dt == np.int64:
        return int(ValType.Int64)
    raise TypeError(f"unsupported column dtype {dt}")


class Fold:
    """A fold in flight (svm_batch_begin .. svm_batch_release)."""

    def __init__(self, engine: "Engine", handle: ctypes.c_void_p, prepared: "Prepared"):
        self.engine = engine
        self.h = handle
        self.prepared = prepared  # the marshalled pipelines stay alive while the fold is in flight
        self.rows = None
        self.needed = 0

    def wait(self) -> list[int]:
        """Blocks until the fold's device work is done; stores its results as
        objects; returns each pipeline's row count (input order)."""
        n = self.prepared.n
        rows = (ctypes.c_ulonglong * max(n, 1))()
        need = ctypes.c_ulonglong()
        self.engine._check(self.engine.lib.svm_batch_wait(self.engine.h, self.h, rows, ctypes.byref(need)))
        self.rows = [rows[i] for i in range(n)]
        self.needed = need.value
        return self.rows

    def release(self, types: list[list[int]] | None = None) -> list[list[np.ndarray]] | None:
        """Frees the fold; with `types` (each pipeline's column types, after a
        successful wait of a fold begun with host_results) returns every
        result's columns, copied from the fold's staging."""
        if self.h is None:
            return None
        lib, eh = self.engine.lib, self.engine.h
        if types is None or self.rows is None:
            st = lib.svm_batch_release(eh, self.h, None, 0)
            self.h = None
            self.engine._check(st)
            return None
        buf = np.empty(max(self.needed, 8), np.uint8)
        st = lib.svm_batch_release(eh, self.h, buf.ctypes.data_as(ctypes.c_void_p), buf.nbytes)
        self.h = None
        self.engine._check(st)
        out, off = [], 0
        for k, ts in enumerate(types):
            cols = []
            for t in ts:
                dt = np.int64 if t == ValType.Int64 else np.int32
                nb = self.rows[k] * np.dtype(dt).itemsize
                cols.append(buf[off:off + nb].view(dt).copy())
                off += (nb + 7) & ~7
            out.append(cols)
        return out

    def __del__(self):
        try:
            if self.h is not None:
                self.engine.lib.svm_batch_release(self.engine.h, self.h, None, 0)
        except Exception:
            pass


class Prepared:
    """Pipelines marshalled into C-ABI structs once (as a server decodes a
    request once), reusable across run / run_batch calls."""

    def __init__(self, pipes: list[PipelineInfo]):
        self.keep = []
        self.n = len(pipes)
        self.arr = (capi.svm_pipeline * max(self.n, 1))(*[marshal(p, self.keep) for p in pipes])


# Marshalled operator and pre_pipeline_id arrays by pipeline content (its
# operators and inputs, not its id): a server sees the same query text again
# and again under new ids, and building the ctypes arrays is most of the
# cost of marshalling.  The arrays are read-only to the library, so requests
# share them; the cache keeps them alive.
_MARSHAL_CACHE: dict = {}
_MARSHAL_CACHE_MAX = 4096


def _content_key(pipe: PipelineInfo):
    return (tuple((int(op.type), tuple(sorted(op.args.items())),
                   tuple((int(c.type), int(c.val_size)) for c in op.output.column_list)
                   if op.output is not None else None) for op in pipe.workflow),
            tuple(pipe.pre_pipeline_id))


def marshal(pipe: PipelineInfo, keep: list) -> capi.svm_pipeline:
    """PipelineInfo -> svm_pipeline; `keep` holds the buffers alive."""
    key = _content_key(pipe)
    hit = _MARSHAL_CACHE.get(key)
    if hit is None:
        hit = _marshal_ops(pipe)
        if len(_MARSHAL_CACHE) >= _MARSHAL_CACHE_MAX:
            _MARSHAL_CACHE.clear()
        _MARSHAL_CACHE[key] = hit
    ops, nops, pre, npre = hit
    pid = pipe.id.encode()
    keep += [hit, pid]
    return capi.svm_pipeline(pid, nops, ops, npre, pre)


def _marshal_ops(pipe: PipelineInfo):
    keep = []
    ops = (capi.svm_operator * max(len(pipe.workflow), 1))()
    for i, op in enumerate(pipe.workflow):
        items = sorted(op.args.items())
        args = (capi.svm_arg * max(len(items), 1))(*[capi.svm_arg(k.encode(), v.encode()) for k, v in items])
        cols = op.output.column_list if op.output is not None else []
        out = (capi.svm_column_desc * max(len(cols), 1))(
            *[capi.svm_column_desc(int(c.type), int(c.val_size)) for c in cols])
        keep += [args, out]
        ops[i] = capi.svm_operator(int(op.type), len(items), args, len(cols), out)
    pre = (ctypes.c_char_p * max(len(pipe.pre_pipeline_id), 1))(*[s.encode() for s in pipe.pre_pipeline_id])
    ops._keep = keep  # the operators' argument and column arrays live as long as the operator array
    return ops, len(pipe.workflow), pre, len(pipe.pre_pipeline_id)


def reduce_shape(pipe: PipelineInfo) -> tuple[int, int]:
    """(key_num, metric_num) of a ReduceBy pipeline, split as the reference does."""
    from .pipeline import str_split
    for op in pipe.workflow:
        if op.type == OpType.ReduceBy:
            return len(str_split(op.args.get("dim", ""), ",")), len(str_split(op.args["metric"], ","))
    return 0, 0
