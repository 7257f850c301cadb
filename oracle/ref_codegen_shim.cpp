/*
 * ORACLE (test infrastructure only).  Compiles the reference's own code
 * generator (codegen/codegen.cpp and codegen/template.cpp, included from the
 * reference tree by oracle/build_ref.sh) without its protobuf/CUDA/thrust
 * dependencies, by standing in minimal ObjectInfo/ColumnInfo/Pipeline types
 * for the ones those files read.  It emits the host code the reference would
 * generate for one query pipeline, so oracle/codegen.py can be compared with it.
 *
 * Input (stdin), one record per line, fields separated by TAB:
 *   id <pipeline id>
 *   schema <obj> <type:size> ...      input_info_[obj] (0 = source, 1.. = joined)
 *   out <type:size> ...               the Sink schema (output_info_)
 *   filter <predication>              one per Filter operator, in order
 *   select <select arg>               the Map operator's "select" string
 *   reduce <dim arg> <metric arg>     the ReduceBy operator's "dim" and "metric"
 *   join <lkey> <rkey>                one per JoinWith operator, in order
 */
#include <cassert>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

using namespace std;

namespace ShadowVM {
enum ValType { Byte = 0, Int16 = 1, Int32 = 2, Int64 = 3, Float16 = 4, Float32 = 5, Float64 = 6, String = 7, Tensor = 8 };
class ColumnInfo {
 public:
  ValType t = Byte;
  long long s = 0;
  ValType type() const { return t; }
  long long val_size() const { return s; }
};
class ObjectInfo {
 public:
  vector<ColumnInfo> cols;
  int column_list_size() const { return (int)cols.size(); }
  const ColumnInfo& column_list(int i) const { return cols[i]; }
};
}  // namespace ShadowVM
using namespace ShadowVM;

#include "define.hpp"

/* Keep the heavy headers that codegen.hpp / template.hpp / codegen.cpp pull in
 * (protobuf messages, CUDA, thrust) out: their include guards are pre-set. */
#define COM_H_
#define JIT_COMPILER_HPP_
#define PIPELINE_HPP_
class Pipeline {
 public:
  vector<ObjectInfo> input_info_;
  ObjectInfo output_info_;
};

#include "codegen.cpp"
#include "template.cpp"

/* com/cpp/com.cu:79-93 (StrSplit), restated. */
static vector<string> str_split(const string& code, const string& sep) {
  vector<string> ret;
  size_t pos1 = 0, pos2 = code.find(sep);
  while (pos2 != string::npos) {
    ret.push_back(code.substr(pos1, pos2 - pos1));
    pos1 = pos2 + sep.size();
    pos2 = code.find(sep, pos1);
  }
  if (pos1 != code.length()) ret.push_back(code.substr(pos1));
  return ret;
}

static ObjectInfo parse_schema(istringstream& in) {
  ObjectInfo o;
  string tok;
  while (getline(in, tok, '\t')) {
    if (tok.empty()) continue;
    ColumnInfo c;
    size_t p = tok.find(':');
    c.t = (ValType)stoi(tok.substr(0, p));
    c.s = stoll(tok.substr(p + 1));
    o.cols.push_back(c);
  }
  return o;
}

int main() {
  Pipeline pipe;
  string id;
  vector<string> filter_exp, select_exp, metric_exp;
  vector<KeyIndex> reduce_key, lkey, rkey;
  bool is_reduce = false;
  string line;
  while (getline(cin, line)) {
    istringstream in(line);
    string tag;
    getline(in, tag, '\t');
    if (tag == "id") {
      getline(in, id);
    } else if (tag == "schema") {
      string k;
      getline(in, k, '\t');
      size_t obj = stoul(k);
      if (pipe.input_info_.size() <= obj) pipe.input_info_.resize(obj + 1);
      pipe.input_info_[obj] = parse_schema(in);
    } else if (tag == "out") {
      pipe.output_info_ = parse_schema(in);
    } else if (tag == "filter") {
      string e;
      getline(in, e);
      filter_exp.push_back(e);
    } else if (tag == "select") {
      string e;
      getline(in, e);
      select_exp = str_split(e, ",");
    } else if (tag == "reduce") {
      string dim, metric;
      getline(in, dim, '\t');
      getline(in, metric);
      metric_exp = str_split(metric, ",");
      for (auto& e : str_split(dim, ",")) reduce_key.push_back(CodeGen::GenKeyIndex(e));
      is_reduce = true;
    } else if (tag == "join") {
      string l, r;
      getline(in, l, '\t');
      getline(in, r);
      lkey.push_back(CodeGen::GenKeyIndex(l));
      rkey.push_back(CodeGen::GenKeyIndex(r));
    }
  }
  /* core/operator.cpp:281-301 (Query::GenCode), host half, restated. */
  map<string, string> args, variable;
  args["pipe_id"] = id;
  args["filter_block"] = CodeGen::GenFilterBlock(variable, pipe, filter_exp, false);
  args["join_block"] = CodeGen::GenJoinBlock(variable, pipe, lkey, rkey, false);
  if (!is_reduce)
    args["select_block"] = CodeGen::GenSelectBlock(variable, pipe, select_exp, false);
  else
    args["reduce_block"] = CodeGen::GenReduceBlock(variable, pipe, metric_exp, reduce_key, false);
  args["define_variable"] = CodeGen::GenVariableDefine(variable);
  string code = CodeGen::GenFromTemplate(CodeTemplate::HostQueryTransform, args);
  /* codegen/compiler.cpp:111-120 (ExportHostCode), restated. */
  cout << "#include \"define.hpp\" \n#include \"cpu-runtime.hpp\" \n#include \"cpu-udf.hpp\" \n"
       << "extern \"C\" {\n" << code << "}";
  return 0;
}
