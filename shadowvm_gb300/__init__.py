"""shadowvm_gb300: a GB300 (sm_103a) data plane for ShadowVM's query hot path --
fused fact-table filter, dimension hash-table build/probe and group-by
aggregation over device-resident columnar int32 tables -- behind the
reference's PipelineInfo / RunPipelineCMD interface and a plain C ABI
(include/svm_capi.h)."""
from .capi import SvmError
from .engine import Engine
from .pipeline import PipelineBuilder, PipelineTest
from .proto import ObjectInfo, OperatorInfo, OpType, PipelineInfo, Ret, ValType, create_schema

__all__ = ["Engine", "SvmError", "PipelineBuilder", "PipelineTest", "PipelineInfo", "OperatorInfo",
           "ObjectInfo", "OpType", "Ret", "ValType", "create_schema"]
