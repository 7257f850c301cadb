"""RunPipelineCMD against the CUDA engine, end to end.

The golden case c2_small (the four-dimension star query at test scale, whose
result the reference's own generated code produced) is sent as the wire
messages a ShadowVM client sends: its three dimension pipelines, then the
fact pipeline, each one RunPipelineCMD into DataPlane(BatchLoop(Engine())).
Each reply must be Ret{success, "ShadowVM exec: <id>"}, the result cached
server-side under the fact pipeline's id must equal the golden rows bit for
bit, and a pipeline naming an object the server does not hold must end
CANCELLED.

Where grpcio is installed the requests go through a real gRPC server and
ShadowVMClient's method (service.Client); elsewhere (GPU hosts without
grpcio) each request is encoded to the wire bytes, decoded by the server's
own request deserializer and handed to the same RPC handler the server
registers, so everything but the HTTP/2 transport runs."""
import json
import os

import numpy as np
import pytest

from shadowvm_gb300 import proto, serving
from shadowvm_gb300 import workloads as W
from shadowvm_gb300.pipeline import fact_pipeline
from shadowvm_gb300.service import DataPlane

pytestmark = pytest.mark.gpu

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_results.json")))


class WireCaller:
    """The RPC handler behind the wire codec, as the grpc server runs it."""

    def __init__(self, dp):
        self.dp = dp

    def __call__(self, pipe):
        request = proto.decode_pipeline(proto.encode_pipeline(pipe))
        status, ret = self.dp.handle(request)
        return status, proto.decode_ret(proto.encode_ret(ret))


class GrpcCaller:
    def __init__(self, dp, grpc):
        from shadowvm_gb300.service import Client, make_server
        self.grpc = grpc
        self.server, port = make_server(dp, "127.0.0.1:0", workers=4)
        self.server.start()
        self.client = Client(f"127.0.0.1:{port}")

    def __call__(self, pipe):
        try:
            return "OK", self.client.run_pipeline_cmd(pipe, timeout=60)
        except self.grpc.RpcError as e:
            return e.code().name, None

    def close(self):
        self.client.close()
        self.server.stop(0)


def test_run_pipeline_cmd_reaches_the_gpu_and_matches_the_golden(engine_factory):
    case = GOLDEN["c2_small"]
    w = W.make(case["config"], **case["kwargs"])
    eng = engine_factory(tuple_per_bulk=w.tuple_per_bulk)
    W.load_engine(eng, w)
    try:
        import grpc
    except ImportError:
        grpc = None
    with serving.BatchLoop(eng) as loop:
        dp = DataPlane(loop)
        call = GrpcCaller(dp, grpc) if grpc is not None else WireCaller(dp)
        try:
            for p in w.dim_pipelines + [w.query]:
                status, ret = call(p)
                assert status == "OK" and ret.success, (status, ret)
                assert ret.info == f"ShadowVM exec: {p.id}"
            missing = fact_pipeline("q_missing", "lineorder", w.fact_schema(), ["no_such_dim"],
                                    [("$(0.0)", "$(1.0)")], "$(1.1)", "$(0.7)")
            status, _ = call(missing)
            assert status == "CANCELLED"
        finally:
            if grpc is not None:
                call.close()
    keys, sums = eng.result(w.query.id, w.key_num)
    rows = len(case["sums"])
    np.testing.assert_array_equal(keys, np.array(case["keys"], np.int32).reshape(rows, w.key_num))
    np.testing.assert_array_equal(sums, np.array(case["sums"], np.int64).reshape(rows, -1))
