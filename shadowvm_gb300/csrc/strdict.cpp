// String columns through dictionary encoding; see strdict.h.
#include "strdict.h"

#include <algorithm>
#include <climits>
#include <cstring>
#include <numeric>
#include <string_view>
#include <unordered_map>

namespace svm {

StrDictPtr build_dict(const char* data, unsigned long long n, int width, std::vector<int32_t>* codes) {
  auto d = std::make_shared<StrDict>();
  d->width = width;
  codes->assign(n, 0);
  if (width <= 0 || n == 0) return d;
  // Distinct values in order of first appearance, then sorted.
  std::unordered_map<std::string_view, uint32_t> first;
  first.reserve((size_t)std::min<unsigned long long>(n, 1ull << 24));
  std::vector<const char*> vals;
  std::vector<uint32_t> prov(n);
  for (unsigned long long i = 0; i < n; i++) {
    const char* v = data + i * (unsigned long long)width;
    auto ins = first.try_emplace(std::string_view(v, (size_t)width), (uint32_t)vals.size());
    if (ins.second) vals.push_back(v);
    prov[i] = ins.first->second;
  }
  std::vector<uint32_t> order(vals.size());
  std::iota(order.begin(), order.end(), 0u);
  std::sort(order.begin(), order.end(),
            [&](uint32_t a, uint32_t b) { return std::memcmp(vals[a], vals[b], (size_t)width) < 0; });
  std::vector<int32_t> code_of(vals.size());
  d->count = (uint32_t)vals.size();
  d->bytes.resize((size_t)d->count * width);
  for (uint32_t r = 0; r < d->count; r++) {
    code_of[order[r]] = (int32_t)r;
    std::memcpy(d->bytes.data() + (size_t)r * width, vals[order[r]], (size_t)width);
  }
  for (unsigned long long i = 0; i < n; i++) (*codes)[i] = code_of[prov[i]];
  return d;
}

StrDictPtr truncate_dict(const StrDict& d, int width, std::vector<int32_t>* remap) {
  auto t = std::make_shared<StrDict>();
  t->width = width;
  remap->assign(d.count, 0);
  // Cutting memcmp-sorted values keeps them sorted: equal prefixes are adjacent.
  for (uint32_t k = 0; k < d.count; k++) {
    const char* v = d.value(k);
    if (t->count == 0 || std::memcmp(t->bytes.data() + (size_t)(t->count - 1) * width, v, (size_t)width) != 0) {
      t->bytes.insert(t->bytes.end(), v, v + width);
      t->count++;
    }
    (*remap)[k] = (int32_t)(t->count - 1);
  }
  return t;
}

namespace {

// StrCmp with the index it stopped at: *reach = the largest value index read.
int strcmp_reach(const char* v, int vwidth, const std::string& lit, int n, int* reach) {
  *reach = -1;
  for (int i = 0; i < n; i++) {
    *reach = i;
    const int a = i < vwidth ? (int)(signed char)v[i] : 0;
    const int b = i < (int)lit.size() ? (int)(signed char)lit[i] : 0;
    if (a == 0 || b == 0) return 0;
    if (a != b) return a - b;
  }
  return 0;
}

bool is_cmp(int op) { return op == X_LT || op == X_LE || op == X_GT || op == X_GE || op == X_EQ || op == X_NE; }

bool cmp_holds(int op, int32_t a, int32_t b) {
  switch (op) {
    case X_LT: return a < b;
    case X_LE: return a <= b;
    case X_GT: return a > b;
    case X_GE: return a >= b;
    case X_EQ: return a == b;
    default: return a != b;
  }
}

int swap_cmp(int op) {  // k OP x  ==  x OP' k
  switch (op) {
    case X_LT: return X_GT;
    case X_LE: return X_GE;
    case X_GT: return X_LT;
    case X_GE: return X_LE;
    default: return op;
  }
}

bool reachable_walk(const Expr& e, int i, std::vector<char>* seen) {
  if (i < 0) return true;
  if ((*seen)[i]) return true;
  (*seen)[i] = 1;
  const Node& n = e.nodes[i];
  return reachable_walk(e, n.a, seen) && reachable_walk(e, n.b, seen) && reachable_walk(e, n.c, seen);
}

const char* op_text(int op) {
  switch (op) {
    case X_ADD: return "+";
    case X_SUB: return "-";
    case X_MUL: return "*";
    case X_DIV: return "/";
    case X_MOD: return "%";
    case X_SHL: return "<<";
    case X_SHR: return ">>";
    case X_LT: return "<";
    case X_LE: return "<=";
    case X_GT: return ">";
    case X_GE: return ">=";
    case X_EQ: return "==";
    case X_NE: return "!=";
    case X_BAND: return "&";
    case X_BXOR: return "^";
    case X_BOR: return "|";
    case X_NEG: return "-";
    case X_NOT: return "!";
    case X_BNOT: return "~";
  }
  return "?";
}

constexpr int kMaxCodeRanges = 16;

}  // namespace

int strcmp_ref(const char* v, int vwidth, const std::string& lit, int n) {
  int reach;
  return strcmp_reach(v, vwidth, lit, n, &reach);
}

uint32_t hash_ref(const char* v, int vwidth, int w) {
  uint32_t h = 0;
  for (int i = 0; i < w; i++) h = h * 31u + (uint32_t)(int)(i < vwidth ? (signed char)v[i] : (signed char)0);
  return h & 0x7FFFFFFFu;
}

void hash_ranks(const StrDict& d, int w, const std::vector<uint32_t>& present, std::vector<int32_t>* rank_of_code,
                std::vector<int32_t>* hash_of_rank) {
  std::vector<int32_t> h(d.count);
  hash_of_rank->clear();
  for (uint32_t k = 0; k < d.count; k++) {
    h[k] = (int32_t)hash_ref(d.value(k), d.width, w);
    if (k < present.size() && present[k]) hash_of_rank->push_back(h[k]);
  }
  std::sort(hash_of_rank->begin(), hash_of_rank->end());
  hash_of_rank->erase(std::unique(hash_of_rank->begin(), hash_of_rank->end()), hash_of_rank->end());
  rank_of_code->assign(d.count, 0);
  for (uint32_t k = 0; k < d.count; k++)
    if (k < present.size() && present[k])
      (*rank_of_code)[k] =
          (int32_t)(std::lower_bound(hash_of_rank->begin(), hash_of_rank->end(), h[k]) - hash_of_rank->begin());
}

bool rewrite_strings(Expr* e, const std::function<const StrCol*(const ColRef&)>& strcol, std::string* err) {
  if (e->root < 0) return true;
  std::vector<char> live(e->nodes.size(), 0);
  reachable_walk(*e, e->root, &live);
  // String columns appear only as StrCmp's first argument.
  std::vector<char> strcmp_arg(e->nodes.size(), 0);
  for (size_t i = 0; i < e->nodes.size(); i++)
    if (live[i] && e->nodes[i].kind == N_STRCMP) strcmp_arg[e->nodes[i].a] = 1;
  for (size_t i = 0; i < e->nodes.size(); i++) {
    if (!live[i] || e->nodes[i].kind != N_COL) continue;
    const bool s = strcol(e->nodes[i].ref) != nullptr;
    if (s && !strcmp_arg[i]) {
      *err = "unsupported: String column $(" + std::to_string(e->nodes[i].ref.obj) + "." +
             std::to_string(e->nodes[i].ref.col) + ") used outside StrCmp";
      return false;
    }
    if (!s && strcmp_arg[i]) {
      *err = "unsupported: StrCmp of a column that is not a String";
      return false;
    }
  }
  // Each `StrCmp(...) OP k` becomes range tests on the codes.
  const size_t n0 = e->nodes.size();
  for (size_t i = 0; i < n0; i++) {
    if (!live[i]) continue;
    const Node cmp = e->nodes[i];
    if (cmp.kind != N_BINARY || !is_cmp(cmp.op)) continue;
    int sc, kn, op = cmp.op;
    if (e->nodes[cmp.a].kind == N_STRCMP) {
      sc = cmp.a;
      kn = cmp.b;
    } else if (e->nodes[cmp.b].kind == N_STRCMP) {
      sc = cmp.b;
      kn = cmp.a;
      op = swap_cmp(op);
    } else {
      continue;
    }
    int32_t k, len;
    if (!const_value(*e, kn, &k)) {
      *err = "unsupported: StrCmp compared with something other than a constant";
      return false;
    }
    const Node sn = e->nodes[sc];
    if (!const_value(*e, sn.b, &len)) {
      *err = "unsupported: StrCmp's length must be a constant";
      return false;
    }
    const ColRef ref = e->nodes[sn.a].ref;
    const StrCol* col = strcol(ref);
    const std::string& lit = e->strs[sn.value];
    const StrDict& d = *col->dict;
    std::vector<std::pair<uint32_t, uint32_t>> ranges;
    for (uint32_t v = 0; v < d.count; v++) {
      int reach;
      const int r = strcmp_reach(d.value(v), d.width, lit, len, &reach);
      if (reach >= col->width) {
        *err = "unsupported: StrCmp(..., " + std::to_string(len) + ") reads past the " + std::to_string(col->width) +
               "-byte column (the reference reads the next row's bytes)";
        return false;
      }
      if (!cmp_holds(op, r, k)) continue;
      if (!ranges.empty() && ranges.back().second + 1 == v)
        ranges.back().second = v;
      else
        ranges.push_back({v, v});
    }
    if ((int)ranges.size() > kMaxCodeRanges) {
      *err = "unsupported: a string predicate accepting " + std::to_string(ranges.size()) + " separate code ranges";
      return false;
    }
    auto add = [&](Node n) {
      e->nodes.push_back(n);
      return (int)e->nodes.size() - 1;
    };
    auto konst = [&](int32_t v) {
      Node n{N_CONST};
      n.value = v;
      return add(n);
    };
    auto colnode = [&]() {
      Node n{N_COL};
      n.ref = ref;
      return add(n);
    };
    auto bin = [&](int o, int a, int b) {
      Node n{N_BINARY};
      n.op = o;
      n.a = a;
      n.b = b;
      return add(n);
    };
    int repl = -1;
    if (ranges.empty()) {
      repl = konst(0);
    } else if (ranges.size() == 1 && ranges[0].first == 0 && ranges[0].second + 1 == d.count) {
      repl = konst(1);
    } else {
      for (auto& rg : ranges) {
        int t;
        if (rg.first == rg.second) {
          t = bin(X_EQ, colnode(), konst((int32_t)rg.first));
        } else {
          Node a{N_LAND};
          a.a = bin(X_GE, colnode(), konst((int32_t)rg.first));
          a.b = bin(X_LE, colnode(), konst((int32_t)rg.second));
          t = add(a);
        }
        if (repl < 0) {
          repl = t;
        } else {
          Node o{N_LOR};
          o.a = repl;
          o.b = t;
          repl = add(o);
        }
      }
    }
    e->nodes[i] = e->nodes[repl];
  }
  // Anything left of StrCmp is outside the supported form.
  std::vector<char> after(e->nodes.size(), 0);
  reachable_walk(*e, e->root, &after);
  for (size_t i = 0; i < e->nodes.size(); i++)
    if (after[i] && e->nodes[i].kind == N_STRCMP) {
      *err = "unsupported: StrCmp used other than in a comparison with a constant";
      return false;
    }
  return true;
}

std::string print_expr(const Expr& e, int i) {
  const Node& n = e.nodes[i];
  switch (n.kind) {
    case N_CONST:
      if (n.value == INT_MIN) return "(-2147483647-1)";
      return n.value < 0 ? "(" + std::to_string(n.value) + ")" : std::to_string(n.value);
    case N_COL:
      return "$(" + std::to_string(n.ref.obj) + "." + std::to_string(n.ref.col) + ")";
    case N_UNARY:
      return std::string("(") + op_text(n.op) + print_expr(e, n.a) + ")";
    case N_BINARY:
      return "(" + print_expr(e, n.a) + " " + op_text(n.op) + " " + print_expr(e, n.b) + ")";
    case N_LAND:
      return "(" + print_expr(e, n.a) + " && " + print_expr(e, n.b) + ")";
    case N_LOR:
      return "(" + print_expr(e, n.a) + " || " + print_expr(e, n.b) + ")";
    case N_COND:
      return "(" + print_expr(e, n.a) + " ? " + print_expr(e, n.b) + " : " + print_expr(e, n.c) + ")";
    case N_STRCMP:
      break;
  }
  return "StrCmp";  // never printed: rewrite_strings removes every StrCmp first
}

}  // namespace svm
