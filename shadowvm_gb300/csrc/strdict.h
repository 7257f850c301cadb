// String columns through dictionary encoding.
//
// The reference stores a String column as fixed-width char[val_size] values
// (com/svm.proto:62-72) and uses them three ways in generated code
// (codegen/codegen.cpp:240-277): as StrCmp(value, "literal", n) operands in
// predicates (com/cpp/cpu-runtime.hpp:37-45), as Hash(value, val_size) group
// keys in ReduceBy (cpu-runtime.hpp:68-74), and copied by Map with StrCopy
// (codegen.cpp:151-180).  Here a String column is a sorted dictionary of its
// distinct values plus one int32 code per row on the device, and the three
// uses become integer work the kernels already do:
//
//   * a comparison `StrCmp(col, lit, n) OP k` is evaluated once per
//     dictionary value and replaced by range tests on the code column
//     (sorted codes keep the accepted values in few ranges);
//   * a group key is the row's rank among the column's distinct Hash values
//     (a derived int32 column; ranks order like the hashes), turned back into
//     the Hash value when the result is written;
//   * Map copies the codes, sharing the dictionary (or a truncated one when
//     the output column is narrower).
#pragma once

#include <functional>
#include <string>
#include <vector>

#include "ctx.h"
#include "expr.h"

namespace svm {

// The dictionary of n values of `width` bytes (data: n x width), and the code
// of every value in *codes.
StrDictPtr build_dict(const char* data, unsigned long long n, int width, std::vector<int32_t>* codes);

// The dictionary of d's values cut to `width` bytes (width < d.width), and
// remap[k] = the code of value k once cut.
StrDictPtr truncate_dict(const StrDict& d, int width, std::vector<int32_t>* remap);

// StrCmp(value, lit, n) (cpu-runtime.hpp:37-45) for a value of `vwidth`
// bytes followed by NULs; chars are signed, as on the x86 reference.
int strcmp_ref(const char* v, int vwidth, const std::string& lit, int n);

// Hash(value, w) (cpu-runtime.hpp:68-74) of a value of `vwidth` bytes
// followed by NULs up to w bytes; signed chars.
uint32_t hash_ref(const char* v, int vwidth, int w);

// For a column of declared width w holding the codes k with present[k]:
// rank_of_code[k] = rank of Hash(value k, w) among the distinct hash values of
// the present codes (ascending; 0 for absent codes), hash_of_rank[r] = that
// value.  Ranking only what the column holds keeps the ranks dense.
void hash_ranks(const StrDict& d, int w, const std::vector<uint32_t>& present, std::vector<int32_t>* rank_of_code,
                std::vector<int32_t>* hash_of_rank);

// Rewrites every `StrCmp(col, lit, n) OP k` / `k OP StrCmp(...)` of *e (OP
// one of < <= > >= == !=, k and n constants) into tests of col's codes;
// strcol(ref) gives a String column's dictionary and width (nullptr: not a
// String column).  Fails (err "unsupported: ...") for a StrCmp anywhere
// else, for a String column used as a number, and when a comparison could
// read past the column's declared width (the reference then reads the next
// row's bytes).
bool rewrite_strings(Expr* e, const std::function<const StrCol*(const ColRef&)>& strcol, std::string* err);

// The subtree as expression text the parser reads back ($(o.c), int
// literals, fully parenthesised).
std::string print_expr(const Expr& e, int node);

}  // namespace svm
