"""The hand-written svm.proto codec (shadowvm_gb300/proto.py) against the
protobuf runtime itself: the messages of com/svm.proto:49-155 are restated
here as a descriptor (field numbers, types and labels as the .proto file
declares them), protobuf builds their classes, and bytes go both ways.  Our
encoder must produce exactly protobuf's deterministic serialisation, and our
decoder must read what protobuf writes, including fields we never set and
fields it does not know."""
import pytest

descriptor_pb2 = pytest.importorskip("google.protobuf.descriptor_pb2")
from google.protobuf import descriptor_pool, message_factory  # noqa: E402

from shadowvm_gb300 import proto  # noqa: E402
from shadowvm_gb300.pipeline import fact_pipeline  # noqa: E402
from shadowvm_gb300.proto import (ColumnInfo, DependencyInfo, ObjectInfo, OperatorInfo, OpType,  # noqa: E402
                                  PipelineInfo, Preference, Ret, StoType, ValType, create_schema)

F = descriptor_pb2.FieldDescriptorProto


def _messages():
    fd = descriptor_pb2.FileDescriptorProto(name="svm_wire_check.proto", package="ShadowVM", syntax="proto3")

    def enum(container, name, values):
        e = container.enum_type.add(name=name)
        for i, v in enumerate(values):
            e.value.add(name=v, number=i)

    def field(msg, name, num, ftype, type_name=None, repeated=False):
        f = msg.field.add(name=name, number=num, type=ftype,
                          label=F.LABEL_REPEATED if repeated else F.LABEL_OPTIONAL)
        if type_name:
            f.type_name = type_name

    enum(fd, "StoType", ["Disk", "HostMem", "DeviceMem", "SharedMem"])
    enum(fd, "ValType", ["Byte", "Int16", "Int32", "Int64", "Float16", "Float32", "Float64", "String", "Tensor"])
    col = fd.message_type.add(name="ColumnInfo")
    field(col, "id", 1, F.TYPE_STRING)
    field(col, "type", 2, F.TYPE_ENUM, ".ShadowVM.ValType")
    field(col, "isnull", 3, F.TYPE_BOOL)
    field(col, "dim", 4, F.TYPE_INT32, repeated=True)
    field(col, "val_size", 5, F.TYPE_INT64)
    obj = fd.message_type.add(name="ObjectInfo")
    field(obj, "id", 1, F.TYPE_STRING)
    field(obj, "host", 2, F.TYPE_STRING)
    field(obj, "column_list", 3, F.TYPE_MESSAGE, ".ShadowVM.ColumnInfo", repeated=True)
    field(obj, "storage", 4, F.TYPE_ENUM, ".ShadowVM.StoType")
    field(obj, "path", 5, F.TYPE_STRING)
    dep = fd.message_type.add(name="DependencyInfo")
    enum(dep, "Type", ["Whole", "HashPartition", "RangePartition"])
    field(dep, "pre_object", 1, F.TYPE_MESSAGE, ".ShadowVM.ObjectInfo")
    field(dep, "type", 2, F.TYPE_ENUM, ".ShadowVM.DependencyInfo.Type")
    field(dep, "shard_id", 3, F.TYPE_INT32)
    op = fd.message_type.add(name="OperatorInfo")
    enum(op, "Type", ["Source", "Loader", "Filter", "Map", "ReduceBy", "SortBy", "JoinWith", "Sink"])
    enum(op, "Preference", ["CPU", "GPU", "NO"])
    entry = op.nested_type.add(name="ArgsEntry")
    entry.options.map_entry = True
    field(entry, "key", 1, F.TYPE_STRING)
    field(entry, "value", 2, F.TYPE_STRING)
    field(op, "id", 1, F.TYPE_STRING)
    field(op, "type", 2, F.TYPE_ENUM, ".ShadowVM.OperatorInfo.Type")
    field(op, "input", 3, F.TYPE_MESSAGE, ".ShadowVM.DependencyInfo", repeated=True)
    field(op, "args", 4, F.TYPE_MESSAGE, ".ShadowVM.OperatorInfo.ArgsEntry", repeated=True)
    field(op, "output", 5, F.TYPE_MESSAGE, ".ShadowVM.ObjectInfo")
    field(op, "perf", 6, F.TYPE_ENUM, ".ShadowVM.OperatorInfo.Preference")
    pipe = fd.message_type.add(name="PipelineInfo")
    field(pipe, "id", 1, F.TYPE_STRING)
    field(pipe, "workflow", 2, F.TYPE_MESSAGE, ".ShadowVM.OperatorInfo", repeated=True)
    field(pipe, "pre_pipeline_id", 3, F.TYPE_STRING, repeated=True)
    field(pipe, "codegen", 4, F.TYPE_BOOL)
    field(pipe, "debug", 5, F.TYPE_BOOL)
    field(pipe, "isGPU", 6, F.TYPE_BOOL)
    ret = fd.message_type.add(name="Ret")
    field(ret, "success", 1, F.TYPE_BOOL)
    field(ret, "info", 2, F.TYPE_STRING)
    pool = descriptor_pool.DescriptorPool()
    pool.Add(fd)
    return {n: message_factory.GetMessageClass(pool.FindMessageTypeByName("ShadowVM." + n))
            for n in ("PipelineInfo", "Ret")}


M = _messages()


def _full_pipeline() -> PipelineInfo:
    """A fact pipeline as the drivers send it, plus every field the data
    plane itself never sets (hosts, paths, dims, dependencies, flags)."""
    p = fact_pipeline("q_wire", "lineorder", create_schema([ValType.Int32] * 3, [4] * 3), ["d1", "d2"],
                      [("$(0.0)", "$(1.0)"), ("$(0.1)", "$(2.0)")], "$(1.1),$(2.1)", "$(0.2)*3",
                      predication='$(0.2) > -7 && StrCmp($(0.1),"AMERICA",12)==0')
    p.codegen, p.debug, p.isGPU = True, False, True
    src = p.workflow[0]
    src.id = "src-op"
    src.perf = Preference.GPU
    src.args["path"] = "/data/lineorder"
    src.input.append(DependencyInfo(pre_object=ObjectInfo(id="lineorder", host="node-3", path="/tmp/x",
                                                          storage=StoType.DeviceMem), type=2, shard_id=-5))
    src.output.column_list.append(ColumnInfo(id="c_name", type=ValType.String, isnull=True, dim=[3, 0, 70000, -1],
                                             val_size=-25))
    src.output.host = "node-3"
    return p


def _official(p: PipelineInfo):
    m = M["PipelineInfo"](id=p.id, pre_pipeline_id=p.pre_pipeline_id, codegen=p.codegen, debug=p.debug,
                          isGPU=p.isGPU)

    def fill_obj(dst, o: ObjectInfo):
        dst.id, dst.host, dst.storage, dst.path = o.id, o.host, int(o.storage), o.path
        for c in o.column_list:
            dst.column_list.add(id=c.id, type=int(c.type), isnull=c.isnull, dim=c.dim, val_size=c.val_size)

    for op in p.workflow:
        mo = m.workflow.add(id=op.id, type=int(op.type), perf=int(op.perf))
        for k, v in op.args.items():
            mo.args[k] = v
        for d in op.input:
            md = mo.input.add(type=d.type, shard_id=d.shard_id)
            if d.pre_object is not None:
                fill_obj(md.pre_object, d.pre_object)
        if op.output is not None:
            fill_obj(mo.output, op.output)
    return m


def test_our_bytes_are_protobufs_deterministic_serialisation():
    p = _full_pipeline()
    ours = proto.encode_pipeline(p)
    m = M["PipelineInfo"].FromString(ours)
    assert m.SerializeToString(deterministic=True) == ours
    assert _official(p).SerializeToString(deterministic=True) == ours
    assert m.workflow[0].input[0].shard_id == -5
    assert list(m.workflow[0].output.column_list[-1].dim) == [3, 0, 70000, -1]
    assert m.workflow[0].output.column_list[-1].val_size == -25
    assert dict(m.workflow[1].args) == {"predication": '$(0.2) > -7 && StrCmp($(0.1),"AMERICA",12)==0'}


def test_we_decode_what_protobuf_writes():
    p = _full_pipeline()
    back = proto.decode_pipeline(_official(p).SerializeToString())
    assert back == p
    # the same with fields protobuf knows and we do not (a newer peer):
    # unknown numbers of every wire type are skipped
    m = _official(p)
    extra = bytes([0x48, 0x01,                              # field 9, varint
                   0x52, 0x03]) + b"abc" + bytes([          # field 10, length-delimited
                   0x5D, 1, 2, 3, 4,                        # field 11, fixed32
                   0x61, 1, 2, 3, 4, 5, 6, 7, 8])           # field 12, fixed64
    assert proto.decode_pipeline(m.SerializeToString() + extra) == p


def test_unpacked_repeated_ints_are_read():
    """proto3 writes repeated int32 packed, but parsers must accept the
    unpacked form too (a proto2 peer or an older writer)."""
    col = bytes([0x0A, 1]) + b"d" + bytes([0x20, 7, 0x20, 9]) + bytes([0x28, 4])
    obj = bytes([0x1A, len(col)]) + col
    op = bytes([0x10, int(OpType.Sink), 0x2A, len(obj)]) + obj
    p = proto.decode_pipeline(bytes([0x12, len(op)]) + op)
    c = p.workflow[0].output.column_list[0]
    assert (c.id, c.dim, c.val_size) == ("d", [7, 9], 4)


@pytest.mark.parametrize("ret", [Ret(True, "ShadowVM exec: q1"), Ret(False, "ShadowVM error: no object x"),
                                 Ret(False, "")])
def test_ret_both_ways(ret):
    ours = proto.encode_ret(ret)
    m = M["Ret"].FromString(ours)
    assert (m.success, m.info) == (ret.success, ret.info)
    assert m.SerializeToString(deterministic=True) == ours
    assert proto.decode_ret(M["Ret"](success=ret.success, info=ret.info).SerializeToString()) == ret
