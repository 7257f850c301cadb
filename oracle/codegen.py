"""ORACLE (test infrastructure only): a restatement of the reference's code
generator for query pipelines.

It turns a PipelineInfo into the C++ source text of the reference's generated
*host* function -- the per-row loop the reference compiles with clang and runs
on the CPU -- so that text can be compiled (g++) and run by ``oracle/driver.cpp``
against either this repository's runtime restatement (``svm_port_runtime.h``)
or the reference's own runtime headers (``oracle/_ref``).  Each function below
names the reference function it follows.  The emitted text is meant to be
character-identical to the reference's; ``tests/test_oracle.py`` checks
that against the reference's own CodeGen compiled here (``oracle/ref_codegen_shim.cpp``).

Only the product's tests, ``bench.py``'s CPU legs and ``__graft_entry__.smoke``
use this module.
"""
from __future__ import annotations

from dataclasses import dataclass, field

from shadowvm_gb300.proto import ObjectInfo, OpType, PipelineInfo, ValType

# codegen/codegen.cpp:12-21 (CodeGen::ToNativeType)
NATIVE_TYPE = {
    ValType.Byte: "char", ValType.Int16: "short", ValType.Int32: "int",
    ValType.Int64: "long long", ValType.Float32: "float", ValType.Float64: "double",
    ValType.String: "char", ValType.Tensor: "char",
}


def native_type(t) -> str:
    # std::map::operator[] on a missing key yields an empty string.
    return NATIVE_TYPE.get(t, "")


def str_split(code: str, sep: str) -> list[str]:
    """com/cpp/com.cu:79-93 (StrSplit): no trailing empty piece."""
    ret = []
    pos1 = 0
    pos2 = code.find(sep)
    while pos2 != -1:
        ret.append(code[pos1:pos2])
        pos1 = pos2 + len(sep)
        pos2 = code.find(sep, pos1)
    if pos1 != len(code):
        ret.append(code[pos1:])
    return ret


def stoi(s: str) -> int:
    """std::stoi: skip leading whitespace, optional sign, then digits."""
    s = s.lstrip(" \t\n\r\f\v")
    j = 0
    if j < len(s) and s[j] in "+-":
        j += 1
    k = j
    while k < len(s) and s[k].isdigit():
        k += 1
    if k == j:
        raise ValueError(f"stoi: no conversion in {s!r}")
    return int(s[:k])


@dataclass
class KeyIndex:                  # com/cpp/define.hpp:60-66
    obj: int
    col: int


def gen_key_index(exp: str) -> KeyIndex:
    """codegen/codegen.cpp:231-238 (CodeGen::GenKeyIndex)."""
    p1 = exp.find("$(")
    p2 = exp.find(".", p1)
    p3 = exp.find(")", p2)
    obj = stoi(exp[p1 + 2:p2])
    col = stoi(exp[p2 + 1:p2 + 1 + (p3 - p1 - 1)])
    return KeyIndex(obj, col)


@dataclass
class BoundPipeline:
    """What core/pipeline.cu:11-80 (Pipeline::Pipeline) binds out of a PipelineInfo,
    plus the joined objects' schemas appended as test/test.hpp:128-131 does."""
    id: str
    input_info: list[ObjectInfo]
    output_info: ObjectInfo
    select_exp: list[str] = field(default_factory=list)
    filter_exp: list[str] = field(default_factory=list)
    metric_exp: list[str] = field(default_factory=list)
    reduce_key: list[KeyIndex] = field(default_factory=list)
    join_lkey: list[KeyIndex] = field(default_factory=list)
    join_rkey: list[KeyIndex] = field(default_factory=list)
    is_reduce: bool = False


def bind(info: PipelineInfo, ref_infos: list[ObjectInfo]) -> BoundPipeline:
    """core/pipeline.cu:11-80; ref_infos are the joined objects' ObjectInfo in
    pre_pipeline_id[1:] order (test/test.hpp:128-131)."""
    input_info: list[ObjectInfo] = []
    output_info = ObjectInfo()
    for op in info.workflow:
        if op.type == OpType.Source:
            input_info.append(op.output)
        elif op.type == OpType.Sink:
            output_info = op.output
    bp = BoundPipeline(info.id, input_info, output_info)
    exp_list: list[str] = []
    for op in info.workflow:
        if op.type == OpType.Map:
            bp.select_exp = str_split(op.args["select"], ",")
        elif op.type == OpType.Filter:
            bp.filter_exp.append(op.args["predication"])
        elif op.type == OpType.ReduceBy:
            bp.metric_exp = str_split(op.args["metric"], ",")
            if "dim" in op.args:
                exp_list = str_split(op.args["dim"], ",")
            for e in exp_list:
                bp.reduce_key.append(gen_key_index(e))
            bp.is_reduce = True
        elif op.type == OpType.JoinWith:
            bp.join_lkey.append(gen_key_index(op.args["lkey"]))
            bp.join_rkey.append(gen_key_index(op.args["rkey"]))
    bp.input_info.extend(ref_infos)
    return bp


def _col(schema: list[ObjectInfo], obj: int, col: int):
    return schema[obj].column_list[col]


def gen_expression(variable: dict, schema: list[ObjectInfo], exp: str, is_reduce: bool = False) -> str:
    """codegen/codegen.cpp:240-277 (CodeGen::GenExperssion)."""
    code = exp
    pos1 = 0
    while True:
        pos1 = code.find("$(", pos1)
        if pos1 == -1:
            return code
        pos2 = code.find(".", pos1)
        obj_off = code[pos1 + 2:pos2]
        pos3 = code.find(")", pos2)
        assert pos3 != -1
        col_off = code[pos2 + 1:pos3]
        inp = f"in_{obj_off}_{col_off}"
        variable[inp] = f"char* {inp}=(char*)in.GetColumn({obj_off},{col_off});\n"
        c = _col(schema, stoi(obj_off), stoi(col_off))
        typ = native_type(c.type)
        size = str(c.val_size)
        if stoi(obj_off) == 0:
            pos = f"{inp}+i*{size}"
        else:
            pos = f"{inp}+join_index[{obj_off}]*{size}"
        if c.type == ValType.String:
            value = f"Hash({pos},{size})" if is_reduce else f"(char*)({pos})"
        else:
            value = f"(*({typ}*)({pos}))"
        code = code[:pos1] + value + code[pos3 + 1:]
        pos1 += len(value)


def gen_filter_block(variable: dict, bp: BoundPipeline, filter_exp: list[str], is_gpu: bool) -> str:
    """codegen/codegen.cpp:100-119 (CodeGen::GenFilterBlock)."""
    code = "bool cond = " if filter_exp else "bool cond = true"
    for i, e in enumerate(filter_exp):
        code += gen_expression(variable, bp.input_info, e)
        if i != len(filter_exp) - 1:
            code += "&&"
    code += ";\n"
    if is_gpu:
        mask_col = len(bp.output_info.column_list) - 1
        mask = f"out_0_{mask_col}"
        variable[mask] = f"char* {mask}=(char*)out.GetColumn(0,{mask_col});\n"
        code += f"*((int*){mask}+i) = cond;\n"
    return code


def gen_join_block(variable: dict, bp: BoundPipeline, lkey: list[KeyIndex], rkey: list[KeyIndex],
                   is_gpu: bool) -> str:
    """codegen/codegen.cpp:121-149 (CodeGen::GenJoinBlock).  Note the reference
    stores join i's probe result in join_index[i+1] but reads dimension columns
    of object k through join_index[k]: joins must be listed in object order."""
    assert len(lkey) == len(rkey)
    code = ""
    for i in range(len(rkey)):
        l_obj, l_col = str(lkey[i].obj), str(lkey[i].col)
        r_obj, r_col = str(rkey[i].obj), str(rkey[i].col)
        hash_col = str(len(bp.input_info[rkey[i].obj].column_list) - 1)
        l_input = f"in_{l_obj}_{l_col}"
        r_input = f"in_{r_obj}_{r_col}"
        r_hash = f"in_{r_obj}_{hash_col}"
        c = _col(bp.input_info, rkey[i].obj, rkey[i].col)
        typ = native_type(c.type)
        variable[l_input] = f"char* {l_input}=(char*)in.GetColumn({l_obj},{l_col});\n"
        variable[r_input] = f"char* {r_input}=(char*)in.GetColumn({r_obj},{r_col});\n"
        variable[r_hash] = f"char* {r_hash}=(char*)in.GetColumn({r_obj},{hash_col});\n"
        size = str(c.val_size)
        index = f"join_index[{i + 1}]"
        probe = (f"Probe<{typ}>(({typ}*)({l_input}+{size}*i),{size},({typ}*)({r_input}),"
                 f"(int*){r_hash}, HashRate*in.max_tuple_ct_[{r_obj}])")
        join = f"{index}={probe};\n"
        join += f"cond = cond & ({index} >=0 ? true:false);\n"
        join = "if(cond) {\n" + join + "}\n"
        code += join
    return code


def gen_select_block(variable: dict, bp: BoundPipeline, exp_list: list[str], is_gpu: bool) -> str:
    """codegen/codegen.cpp:151-180 (CodeGen::GenSelectBlock)."""
    code = ""
    for i, e in enumerate(exp_list):
        oc = bp.output_info.column_list[i]
        proj_type = native_type(oc.type)
        proj_size = str(oc.val_size)
        proj_name = f"out_0_{i}"
        variable[proj_name] = f"char* {proj_name}=(char*)out.GetColumn(0,{i});\n"
        ex = gen_expression(variable, bp.input_info, e)
        move = f"+i*{proj_size}" if is_gpu else f"+j*{proj_size}"
        if oc.type != ValType.String:
            code += f"*({proj_type}*)({proj_name}{move})={ex};\n"
        else:
            code += f"StrCopy({proj_name}{move},{ex},{proj_size});\n"
    code = "if(cond){\n" + code + "}\n"
    if is_gpu:
        mask_col = len(bp.output_info.column_list) - 1
        mask = f"out_0_{mask_col}"
        variable[mask] = f"char* {mask}=(char*)out.GetColumn(0,{mask_col});\n"
        code += f"*(int*)({mask}+i*4)=cond;\n"
    else:
        code += "j+=cond;\n"
    return code


def gen_reduce_block(variable: dict, bp: BoundPipeline, metric_exp: list[str],
                     reduce_key: list[KeyIndex], is_gpu: bool) -> str:
    """codegen/codegen.cpp:182-229 (CodeGen::GenReduceBlock)."""
    code = ""
    for i, k in enumerate(reduce_key):
        exp = f"$({k.obj}.{k.col})"
        ex = gen_expression(variable, bp.input_info, exp, True)
        oc = bp.output_info.column_list[i]
        proj_type = native_type(oc.type)
        proj_size = str(oc.val_size)
        proj_name = f"out_0_{i}"
        variable[proj_name] = f"char* {proj_name}=(char*)out.GetColumn(0,{i});\n"
        move = "+i*" if is_gpu else "+j*"
        code += f"*({proj_type}*)({proj_name}{move}{proj_size})={ex};\n"
    nk = len(reduce_key)
    for i, e in enumerate(metric_exp):
        oc = bp.output_info.column_list[nk + i]
        proj_type = native_type(oc.type)
        proj_size = str(oc.val_size)
        proj_name = f"out_0_{nk + i}"
        variable[proj_name] = f"char* {proj_name}=(char*)out.GetColumn(0,{i + nk});\n"
        ex = gen_expression(variable, bp.input_info, e)
        if not is_gpu and nk == 0:
            variable[proj_name] += f"*({proj_type}*){proj_name}=0;\n"
            code += f"*({proj_type}*)({proj_name})+=cond*{ex};\n"
        else:
            if is_gpu:
                ex = ex + "*cond"
                move = "+i*"
            else:
                move = "+j*"
            if oc.type != ValType.String:
                code += f"*({proj_type}*)({proj_name}{move}{proj_size})={ex};\n"
            else:
                code += f"StrCopy({proj_name}{move}{proj_size},{ex},{proj_size})\n;"
    if not is_gpu:
        code = "if(cond){\n" + code + "\n}\n"
        code += "j+=cond;\n"
    return code


def gen_variable_define(variable: dict) -> str:
    """codegen/codegen.cpp:285-290: std::map iterates in key order."""
    return "".join(variable[k] for k in sorted(variable))


def gen_from_template(template: str, dic: dict) -> str:
    """codegen/codegen.cpp:80-96 (CodeGen::GenFromTemplate)."""
    code = template
    pos1 = 0
    while True:
        pos1 = code.find("$(", pos1)
        if pos1 == -1:
            return code
        pos2 = code.find(")", pos1)
        key = code[pos1 + 2:pos2]
        value = dic.get(key, "")
        code = code[:pos1] + value + code[pos1 + len(key) + 3:]
        pos1 += len(value)


# The host per-row loop of codegen/template.cpp:61-73 (CodeTemplate::HostQueryTransform).
HOST_QUERY_TRANSFORM = "\n".join([
    "",
    "int $(pipe_id)(int task_id, BulkVector in, BulkVector out, uint64 tuple_ct) { ",
    "$(define_variable)int j = 0;",
    "int join_index[8];",
    "for(int i = 0; i < tuple_ct; i++) {",
    "$(filter_block)$(join_block)$(select_block)$(reduce_block)}",
    "return j;",
    "}",
    "",
])

# codegen/compiler.cpp:111-120 (CodeContext::ExportHostCode) include lines.
REFERENCE_INCLUDES = ['#include "define.hpp" \n', '#include "cpu-runtime.hpp" \n',
                      '#include "cpu-udf.hpp" \n']
PORT_INCLUDES = ['#include "svm_port_runtime.h"\n']


def gen_host_function(bp: BoundPipeline) -> str:
    """core/operator.cpp:281-301 (Query::GenCode), host half."""
    variable: dict[str, str] = {}
    args = {"pipe_id": bp.id}
    args["filter_block"] = gen_filter_block(variable, bp, bp.filter_exp, False)
    args["join_block"] = gen_join_block(variable, bp, bp.join_lkey, bp.join_rkey, False)
    if not bp.is_reduce:
        args["select_block"] = gen_select_block(variable, bp, bp.select_exp, False)
    else:
        args["reduce_block"] = gen_reduce_block(variable, bp, bp.metric_exp, bp.reduce_key, False)
    args["define_variable"] = gen_variable_define(variable)
    return gen_from_template(HOST_QUERY_TRANSFORM, args)


def export_host_code(functions: list[str], includes=REFERENCE_INCLUDES) -> str:
    """codegen/compiler.cpp:111-120 (CodeContext::ExportHostCode)."""
    return "".join(includes) + 'extern "C" {\n' + "".join(functions) + "}"
