"""The ShadowVM data-plane service: `/ShadowVM.ShadowVMAPI/RunPipelineCMD`
(com/svm.proto:157-159) on the same wire messages, in front of the GPU engine.

Semantics follow ShadowVMService::RunPipelineCMD (service/service.cu:25-63):
every pre_pipeline_id must name a cached object, else the RPC ends with
CANCELLED; on success the reply is Ret{success=true, info="ShadowVM exec: <id>"}
and the output stays server-side under the pipeline id (the wire has no
result-fetch RPC; results are read through the engine API).  Where the
reference would assert -- an expression outside the supported grammar, an
HBM budget overrun -- this service answers Ret{success=false, info=<why>},
which the Java client prints (java_vRDD/.../vRDD.scala:64-66).

Requests are not run one RPC at a time: a `BatchLoop` folds every reduce
pipeline that arrives while the GPU is busy into the next batched launch
(continuous batching, see serving.py).  grpcio is needed only here; the GPU
hosts do not have it, so the core never imports this module.
"""
from __future__ import annotations

import concurrent.futures as cf

from . import proto
from .capi import E_NOT_FOUND, SvmError

SERVICE = "ShadowVM.ShadowVMAPI"
METHOD = "RunPipelineCMD"
FULL_METHOD = f"/{SERVICE}/{METHOD}"


class DataPlane:
    """The RPC handler's logic, independent of grpc (tested without a server)."""

    def __init__(self, executor):
        # `executor` runs one PipelineInfo: serving.BatchLoop (batched) or an
        # object with .submit(pipe) -> Future; .known(id) -> bool.
        self.executor = executor

    def handle(self, pipe: proto.PipelineInfo) -> tuple[str, proto.Ret]:
        """Returns (grpc status name, reply)."""
        for pid in pipe.pre_pipeline_id:
            if not self.executor.known(pid):
                return "CANCELLED", proto.Ret(False, f"unknown pre_pipeline_id {pid}")
        try:
            self.executor.submit(pipe).result()
        except SvmError as e:
            if e.status == E_NOT_FOUND:
                return "CANCELLED", proto.Ret(False, e.message)
            return "OK", proto.Ret(False, f"ShadowVM error: {e}")
        return "OK", proto.Ret(True, f"ShadowVM exec: {pipe.id}")


def make_server(data_plane: DataPlane, endpoint: str = "0.0.0.0:50051", workers: int = 16):
    """A grpc server for the data plane (service/service.hpp:93-100 listens on 0.0.0.0:50051)."""
    import grpc

    def run(request: proto.PipelineInfo, context):
        status, ret = data_plane.handle(request)
        if status == "CANCELLED":
            context.abort(grpc.StatusCode.CANCELLED, ret.info)
        return ret

    handler = grpc.method_handlers_generic_handler(SERVICE, {
        METHOD: grpc.unary_unary_rpc_method_handler(
            run, request_deserializer=proto.decode_pipeline, response_serializer=proto.encode_ret)})
    server = grpc.server(cf.ThreadPoolExecutor(max_workers=workers))
    server.add_generic_rpc_handlers((handler,))
    port = server.add_insecure_port(endpoint)
    return server, port


class Client:
    """ShadowVMClient (service/service.hpp:37-70) over the same method."""

    def __init__(self, endpoint: str = "localhost:50051"):
        import grpc
        self.channel = grpc.insecure_channel(endpoint)
        self.call = self.channel.unary_unary(FULL_METHOD, request_serializer=proto.encode_pipeline,
                                             response_deserializer=proto.decode_ret)

    def run_pipeline_cmd(self, pipe: proto.PipelineInfo, timeout: float | None = None) -> proto.Ret:
        return self.call(pipe, timeout=timeout)

    def close(self):
        self.channel.close()
