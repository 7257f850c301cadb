// Parser for the expression strings carried in OperatorInfo.args
// (predication / select / metric / dim / lkey / rkey; com/svm.proto:103-109).
//
// The reference splices these strings, with every $(obj.col) rewritten into a
// typed column load (codegen/codegen.cpp:240-277), into C++ source and compiles
// it at run time.  This data plane has no run-time compiler, so it parses the
// same strings as C integer expressions over int32 columns into a tree, and
// the planner maps the tree onto the kernels' compile-time functors (range
// conjuncts, operand/binary metrics) or, for anything else inside the
// grammar, onto a short bytecode program the kernels interpret.
// StrCmp(column, "literal", n) parses into an N_STRCMP node that the planner
// resolves against the column's dictionary (strdict.h) before planning;
// other calls (UDFs), floating point and string literals elsewhere are
// reported as unsupported -- there is no fallback path.
#pragma once

#include <string>
#include <vector>

#include "svm_internal.h"

namespace svm {

struct ColRef {
  int obj;
  int col;
  bool operator==(const ColRef& o) const { return obj == o.obj && col == o.col; }
  bool operator<(const ColRef& o) const { return obj != o.obj ? obj < o.obj : col < o.col; }
};

enum NodeKind { N_COL, N_CONST, N_UNARY, N_BINARY, N_LAND, N_LOR, N_COND,
                N_STRCMP };  // a = column node, b = length node, value = literal index

struct Node {
  NodeKind kind;
  int op = 0;          // ExprOp for unary / binary
  int32_t value = 0;   // N_CONST
  ColRef ref{0, 0};    // N_COL
  int a = -1, b = -1, c = -1;
};

struct Expr {
  std::vector<Node> nodes;
  std::vector<std::string> strs;  // StrCmp literals
  int root = -1;
};

// Parses `text`; on failure returns false and sets *err ("unsupported: ..." for
// constructs outside the grammar, "syntax: ..." for malformed text).
bool parse_expr(const std::string& text, Expr* out, std::string* err);

// $(obj.col) parsed the way CodeGen::GenKeyIndex does (codegen/codegen.cpp:231-238).
bool parse_key_index(const std::string& text, ColRef* out, std::string* err);

// com/cpp/com.cu:79-93 (StrSplit): split on `sep`, no trailing empty piece.
std::vector<std::string> str_split(const std::string& s, const std::string& sep);

// All column references in the subtree.
void collect_refs(const Expr& e, int node, std::vector<ColRef>* refs);

// Top-level && conjuncts of the subtree.
void flatten_and(const Expr& e, int node, std::vector<int>* conj);

// Recognises `col OP const` / `const OP col` with OP in < <= > >= == and
// returns the equivalent inclusive range [lo, hi] (possibly empty: lo > hi).
bool as_range(const Expr& e, int node, ColRef* ref, int32_t* lo, int32_t* hi);

// Compiles the subtree into bytecode; `opnd_of` maps each column reference to
// an operand index.  Returns false (with *err) when it does not fit Prog.
bool compile_prog(const Expr& e, int node, const std::vector<ColRef>& opnd_of, Prog* p,
                  std::string* err);

// Constant folding helper: true and *v when the subtree has no column reference.
bool const_value(const Expr& e, int node, int32_t* v);

// Host-side evaluation of a program (used for constant subtrees and tests).
int32_t eval_prog_host(const Prog& p, const int32_t* opnd, bool* div0);

}  // namespace svm
