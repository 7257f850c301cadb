"""The ShadowVM wire messages (com/svm.proto:49-159) as plain dataclasses, with a
self-contained proto3 wire codec.

The data plane speaks exactly the reference's messages -- ``PipelineInfo``
(svm.proto:137-144) in, ``Ret`` (152-155) out, on the method
``/ShadowVM.ShadowVMAPI/RunPipelineCMD`` (157-159) -- so a Java/Spark control
plane built against svm.proto talks to it unchanged.  The codec here is written
against the public protobuf encoding rules (varints, length-delimited fields,
packed repeated scalars, maps as repeated key/value entries); it needs neither
protoc nor the protobuf runtime, which the GPU hosts do not have.
"""
from __future__ import annotations

import enum
from dataclasses import dataclass, field


class ValType(enum.IntEnum):          # svm.proto:62-72
    Byte = 0
    Int16 = 1
    Int32 = 2
    Int64 = 3
    Float16 = 4
    Float32 = 5
    Float64 = 6
    String = 7
    Tensor = 8


class StoType(enum.IntEnum):          # svm.proto:49-54
    Disk = 0
    HostMem = 1
    DeviceMem = 2
    SharedMem = 3


class OpType(enum.IntEnum):           # svm.proto:102-111 (OperatorInfo.Type)
    Source = 0
    Loader = 1
    Filter = 2
    Map = 3
    ReduceBy = 4
    SortBy = 5
    JoinWith = 6
    Sink = 7


class Preference(enum.IntEnum):       # svm.proto:112-116
    CPU = 0
    GPU = 1
    NO = 2


@dataclass
class ColumnInfo:                     # svm.proto:73-79
    id: str = ""
    type: ValType = ValType.Byte
    isnull: bool = False
    dim: list[int] = field(default_factory=list)
    val_size: int = 0


@dataclass
class ObjectInfo:                     # svm.proto:81-87
    id: str = ""
    host: str = ""
    column_list: list[ColumnInfo] = field(default_factory=list)
    storage: StoType = StoType.Disk
    path: str = ""


@dataclass
class DependencyInfo:                 # svm.proto:89-98
    pre_object: ObjectInfo | None = None
    type: int = 0
    shard_id: int = 0


@dataclass
class OperatorInfo:                   # svm.proto:101-123
    id: str = ""
    type: OpType = OpType.Source
    input: list[DependencyInfo] = field(default_factory=list)
    args: dict[str, str] = field(default_factory=dict)
    output: ObjectInfo | None = None
    perf: Preference = Preference.CPU


@dataclass
class PipelineInfo:                   # svm.proto:137-144
    id: str = ""
    workflow: list[OperatorInfo] = field(default_factory=list)
    pre_pipeline_id: list[str] = field(default_factory=list)
    codegen: bool = False
    debug: bool = False
    isGPU: bool = False


@dataclass
class Ret:                            # svm.proto:152-155
    success: bool = False
    info: str = ""


def create_schema(types, sizes, storage: StoType = StoType.HostMem) -> ObjectInfo:
    """Same as the reference test helper CreateSchema (test/test.hpp:17-27)."""
    assert len(types) == len(sizes)
    return ObjectInfo(column_list=[ColumnInfo(type=ValType(t), val_size=int(s))
                                   for t, s in zip(types, sizes)], storage=storage)


# ------------------------------------------------------------------ encoding
def _varint(v: int) -> bytes:
    v &= 0xFFFFFFFFFFFFFFFF            # negative int32/int64 encode as 10-byte two's complement
    out = bytearray()
    while True:
        b = v & 0x7F
        v >>= 7
        if v:
            out.append(b | 0x80)
        else:
            out.append(b)
            return bytes(out)


def _key(num: int, wt: int) -> bytes:
    return _varint((num << 3) | wt)


def _ld(num: int, payload: bytes) -> bytes:
    return _key(num, 2) + _varint(len(payload)) + payload


def _str(num: int, s: str) -> bytes:
    return _ld(num, s.encode()) if s else b""


def _int(num: int, v: int) -> bytes:
    return _key(num, 0) + _varint(int(v)) if v else b""


def _enc_column(c: ColumnInfo) -> bytes:
    b = _str(1, c.id) + _int(2, c.type) + _int(3, 1 if c.isnull else 0)
    if c.dim:
        b += _ld(4, b"".join(_varint(d) for d in c.dim))
    return b + _int(5, c.val_size)


def _enc_object(o: ObjectInfo) -> bytes:
    b = _str(1, o.id) + _str(2, o.host)
    for c in o.column_list:
        b += _ld(3, _enc_column(c))
    return b + _int(4, o.storage) + _str(5, o.path)


def _enc_dep(d: DependencyInfo) -> bytes:
    b = _ld(1, _enc_object(d.pre_object)) if d.pre_object is not None else b""
    return b + _int(2, d.type) + _int(3, d.shard_id)


def _enc_operator(op: OperatorInfo) -> bytes:
    b = _str(1, op.id) + _int(2, op.type)
    for d in op.input:
        b += _ld(3, _enc_dep(d))
    for k in sorted(op.args):
        b += _ld(4, _str(1, k) + _str(2, op.args[k]))
    if op.output is not None:
        b += _ld(5, _enc_object(op.output))
    return b + _int(6, op.perf)


def encode_pipeline(p: PipelineInfo) -> bytes:
    b = _str(1, p.id)
    for op in p.workflow:
        b += _ld(2, _enc_operator(op))
    for s in p.pre_pipeline_id:
        b += _ld(3, s.encode())
    return b + _int(4, p.codegen) + _int(5, p.debug) + _int(6, p.isGPU)


def encode_ret(r: Ret) -> bytes:
    return _int(1, 1 if r.success else 0) + _str(2, r.info)


# ------------------------------------------------------------------ decoding
class DecodeError(ValueError):
    pass


def _read_varint(buf: bytes, i: int) -> tuple[int, int]:
    shift = 0
    v = 0
    while True:
        if i >= len(buf):
            raise DecodeError("truncated varint")
        b = buf[i]
        i += 1
        v |= (b & 0x7F) << shift
        if not b & 0x80:
            return v, i
        shift += 7
        if shift >= 70:
            raise DecodeError("varint too long")


def _fields(buf: bytes):
    """Yield (field number, wire type, value) with value an int or bytes."""
    i = 0
    while i < len(buf):
        k, i = _read_varint(buf, i)
        num, wt = k >> 3, k & 7
        if wt == 0:
            v, i = _read_varint(buf, i)
        elif wt == 1:
            v, i = int.from_bytes(buf[i:i + 8], "little"), i + 8
        elif wt == 2:
            n, i = _read_varint(buf, i)
            if i + n > len(buf):
                raise DecodeError("truncated length-delimited field")
            v, i = bytes(buf[i:i + n]), i + n
        elif wt == 5:
            v, i = int.from_bytes(buf[i:i + 4], "little"), i + 4
        else:
            raise DecodeError(f"unsupported wire type {wt}")
        if i > len(buf):
            raise DecodeError("truncated field")
        yield num, wt, v


def _s64(v: int) -> int:
    return v - (1 << 64) if v >= 1 << 63 else v


def _dec_column(buf: bytes) -> ColumnInfo:
    c = ColumnInfo()
    for num, wt, v in _fields(buf):
        if num == 1 and wt == 2:
            c.id = v.decode()
        elif num == 2 and wt == 0:
            c.type = ValType(v) if v in ValType._value2member_map_ else v
        elif num == 3 and wt == 0:
            c.isnull = bool(v)
        elif num == 4:
            if wt == 2:
                j = 0
                while j < len(v):
                    d, j = _read_varint(v, j)
                    c.dim.append(_s64(d))
            else:
                c.dim.append(_s64(v))
        elif num == 5 and wt == 0:
            c.val_size = _s64(v)
    return c


def _dec_object(buf: bytes) -> ObjectInfo:
    o = ObjectInfo()
    for num, wt, v in _fields(buf):
        if num == 1 and wt == 2:
            o.id = v.decode()
        elif num == 2 and wt == 2:
            o.host = v.decode()
        elif num == 3 and wt == 2:
            o.column_list.append(_dec_column(v))
        elif num == 4 and wt == 0:
            o.storage = StoType(v) if v in StoType._value2member_map_ else v
        elif num == 5 and wt == 2:
            o.path = v.decode()
    return o


def _dec_operator(buf: bytes) -> OperatorInfo:
    op = OperatorInfo()
    for num, wt, v in _fields(buf):
        if num == 1 and wt == 2:
            op.id = v.decode()
        elif num == 2 and wt == 0:
            op.type = OpType(v) if v in OpType._value2member_map_ else v
        elif num == 3 and wt == 2:
            d = DependencyInfo()
            for n2, w2, v2 in _fields(v):
                if n2 == 1 and w2 == 2:
                    d.pre_object = _dec_object(v2)
                elif n2 == 2 and w2 == 0:
                    d.type = v2
                elif n2 == 3 and w2 == 0:
                    d.shard_id = _s64(v2)
            op.input.append(d)
        elif num == 4 and wt == 2:
            k = val = ""
            for n2, w2, v2 in _fields(v):
                if n2 == 1 and w2 == 2:
                    k = v2.decode()
                elif n2 == 2 and w2 == 2:
                    val = v2.decode()
            op.args[k] = val
        elif num == 5 and wt == 2:
            op.output = _dec_object(v)
        elif num == 6 and wt == 0:
            op.perf = Preference(v) if v in Preference._value2member_map_ else v
    return op


def decode_pipeline(buf: bytes) -> PipelineInfo:
    p = PipelineInfo()
    for num, wt, v in _fields(buf):
        if num == 1 and wt == 2:
            p.id = v.decode()
        elif num == 2 and wt == 2:
            p.workflow.append(_dec_operator(v))
        elif num == 3 and wt == 2:
            p.pre_pipeline_id.append(v.decode())
        elif num == 4 and wt == 0:
            p.codegen = bool(v)
        elif num == 5 and wt == 0:
            p.debug = bool(v)
        elif num == 6 and wt == 0:
            p.isGPU = bool(v)
    return p


def decode_ret(buf: bytes) -> Ret:
    r = Ret()
    for num, wt, v in _fields(buf):
        if num == 1 and wt == 0:
            r.success = bool(v)
        elif num == 2 and wt == 2:
            r.info = v.decode()
    return r
