// Expression parser; see expr.h.
#include "expr.h"

#include <climits>
#include <cstdlib>

namespace svm {

namespace {

enum TokKind { T_END, T_NUM, T_COL, T_OP, T_LP, T_RP, T_COMMA, T_STR, T_CALL };

struct Tok {
  TokKind kind;
  std::string op;
  int32_t num = 0;
  ColRef ref{0, 0};
};

bool strict_uint(const std::string& s, int* v) {
  size_t i = 0, j = s.size();
  while (i < j && isspace((unsigned char)s[i])) i++;
  while (j > i && isspace((unsigned char)s[j - 1])) j--;
  if (i == j) return false;
  long long x = 0;
  for (size_t k = i; k < j; k++) {
    if (!isdigit((unsigned char)s[k])) return false;
    x = x * 10 + (s[k] - '0');
    if (x > 1000000) return false;
  }
  *v = (int)x;
  return true;
}

class Lexer {
 public:
  explicit Lexer(const std::string& s) : s_(s) {}

  bool next(Tok* t, std::string* err) {
    while (i_ < s_.size() && isspace((unsigned char)s_[i_])) i_++;
    if (i_ >= s_.size()) {
      t->kind = T_END;
      return true;
    }
    char c = s_[i_];
    if (c == '$') {
      // $(obj.col), split as CodeGen::GenExperssion does (codegen/codegen.cpp:244-250).
      if (i_ + 1 >= s_.size() || s_[i_ + 1] != '(') return fail(err, "syntax: '$' not followed by '('");
      size_t dot = s_.find('.', i_);
      size_t rp = dot == std::string::npos ? dot : s_.find(')', dot);
      if (rp == std::string::npos) return fail(err, "syntax: unterminated $(obj.col)");
      int obj, col;
      if (!strict_uint(s_.substr(i_ + 2, dot - i_ - 2), &obj) ||
          !strict_uint(s_.substr(dot + 1, rp - dot - 1), &col))
        return fail(err, "syntax: bad column reference " + s_.substr(i_, rp - i_ + 1));
      t->kind = T_COL;
      t->ref = {obj, col};
      i_ = rp + 1;
      return true;
    }
    if (isdigit((unsigned char)c)) {
      size_t j = i_;
      unsigned long long v = 0;
      int base = 10;
      if (c == '0' && j + 1 < s_.size() && (s_[j + 1] == 'x' || s_[j + 1] == 'X')) {
        base = 16;
        j += 2;
      } else if (c == '0') {
        base = 8;
      }
      size_t start = j;
      while (j < s_.size() && isxdigit((unsigned char)s_[j])) {
        int d = isdigit((unsigned char)s_[j]) ? s_[j] - '0' : (tolower(s_[j]) - 'a' + 10);
        if (d >= base) break;
        v = v * base + d;
        if (v > (unsigned long long)INT_MAX) return fail(err, "unsupported: integer literal wider than int");
        j++;
      }
      if (base == 16 && j == start) return fail(err, "syntax: bad hex literal");
      if (j < s_.size() && (isalnum((unsigned char)s_[j]) || s_[j] == '.' || s_[j] == '_'))
        return fail(err, "unsupported: literal " + s_.substr(i_, j - i_ + 1) + "... (only plain int literals)");
      t->kind = T_NUM;
      t->num = (int32_t)v;
      i_ = j;
      return true;
    }
    if (isalpha((unsigned char)c) || c == '_') {
      size_t j = i_;
      while (j < s_.size() && (isalnum((unsigned char)s_[j]) || s_[j] == '_')) j++;
      std::string id = s_.substr(i_, j - i_);
      if (id == "true" || id == "false") {
        t->kind = T_NUM;
        t->num = id == "true";
        i_ = j;
        return true;
      }
      size_t k = j;
      while (k < s_.size() && isspace((unsigned char)s_[k])) k++;
      if (k < s_.size() && s_[k] == '(') {
        // StrCmp (com/cpp/cpu-runtime.hpp:37-45) is resolved against the
        // column's dictionary by the planner; other calls (UDFs) are not.
        if (id != "StrCmp") return fail(err, "unsupported: function call " + id + "(...) (UDF expressions)");
        t->kind = T_CALL;
        t->op = id;
        i_ = j;
        return true;
      }
      return fail(err, "unsupported: identifier '" + id + "'");
    }
    if (c == ',') {
      t->kind = T_COMMA;
      i_++;
      return true;
    }
    // A string literal, its quotes optionally backslash-escaped as the Java
    // DSL writes them (StrCmp($(1.2),\"abc\",3)); C escapes \\ \" \0.
    if (c == '"' || (c == '\\' && i_ + 1 < s_.size() && s_[i_ + 1] == '"')) {
      const bool escaped = c == '\\';
      size_t j = i_ + (escaped ? 2 : 1);
      std::string v;
      for (;;) {
        if (j >= s_.size()) return fail(err, "syntax: unterminated string literal");
        if (escaped && s_[j] == '\\' && j + 1 < s_.size() && s_[j + 1] == '"') {
          j += 2;
          break;
        }
        if (!escaped && s_[j] == '"') {
          j++;
          break;
        }
        if (s_[j] == '\\' && j + 1 < s_.size()) {
          const char e = s_[j + 1];
          if (e == '0') v.push_back('\0');
          else if (e == 'n') v.push_back('\n');
          else if (e == 't') v.push_back('\t');
          else v.push_back(e);
          j += 2;
          continue;
        }
        v.push_back(s_[j++]);
      }
      t->kind = T_STR;
      t->op = v;
      i_ = j;
      return true;
    }
    if (c == '\'') return fail(err, "unsupported: char literal");
    static const char* two[] = {"<<", ">>", "<=", ">=", "==", "!=", "&&", "||"};
    for (const char* op : two) {
      if (s_.compare(i_, 2, op) == 0) {
        t->kind = T_OP;
        t->op = op;
        i_ += 2;
        return true;
      }
    }
    if (c == '(' || c == ')') {
      t->kind = c == '(' ? T_LP : T_RP;
      i_++;
      return true;
    }
    if (std::string("+-*/%<>!~&^|?:").find(c) != std::string::npos) {
      t->kind = T_OP;
      t->op = std::string(1, c);
      i_++;
      return true;
    }
    return fail(err, std::string("syntax: unexpected character '") + c + "'");
  }

 private:
  static bool fail(std::string* err, const std::string& m) {
    *err = m;
    return false;
  }
  const std::string& s_;
  size_t i_ = 0;
};

class Parser {
 public:
  Parser(const std::string& s, Expr* e, std::string* err) : lex_(s), e_(e), err_(err) {}

  bool run() {
    if (!advance()) return false;
    int r;
    if (!cond(&r)) return false;
    if (tok_.kind != T_END) return fail("syntax: trailing input");
    e_->root = r;
    return true;
  }

 private:
  bool advance() { return lex_.next(&tok_, err_); }
  bool fail(const std::string& m) {
    if (err_->empty()) *err_ = m;
    return false;
  }
  bool is_op(const char* o) const { return tok_.kind == T_OP && tok_.op == o; }
  int add(Node n) {
    e_->nodes.push_back(n);
    return (int)e_->nodes.size() - 1;
  }
  int bin(int op, int a, int b) {
    Node n{N_BINARY};
    n.op = op;
    n.a = a;
    n.b = b;
    return add(n);
  }

  bool cond(int* out) {
    int c;
    if (!lor(&c)) return false;
    if (!is_op("?")) {
      *out = c;
      return true;
    }
    if (!advance()) return false;
    int t, f;
    if (!cond(&t)) return false;
    if (!is_op(":")) return fail("syntax: expected ':'");
    if (!advance() || !cond(&f)) return false;
    Node n{N_COND};
    n.a = c;
    n.b = t;
    n.c = f;
    *out = add(n);
    return true;
  }
  bool lor(int* out) {
    if (!land(out)) return false;
    while (is_op("||")) {
      int r;
      if (!advance() || !land(&r)) return false;
      Node n{N_LOR};
      n.a = *out;
      n.b = r;
      *out = add(n);
    }
    return true;
  }
  bool land(int* out) {
    if (!binlevel(0, out)) return false;
    while (is_op("&&")) {
      int r;
      if (!advance() || !binlevel(0, &r)) return false;
      Node n{N_LAND};
      n.a = *out;
      n.b = r;
      *out = add(n);
    }
    return true;
  }
  // Binary levels from | down to * (C precedence).
  bool binlevel(int lvl, int* out) {
    static const std::vector<std::vector<std::pair<const char*, int>>> levels = {
        {{"|", X_BOR}},
        {{"^", X_BXOR}},
        {{"&", X_BAND}},
        {{"==", X_EQ}, {"!=", X_NE}},
        {{"<", X_LT}, {"<=", X_LE}, {">", X_GT}, {">=", X_GE}},
        {{"<<", X_SHL}, {">>", X_SHR}},
        {{"+", X_ADD}, {"-", X_SUB}},
        {{"*", X_MUL}, {"/", X_DIV}, {"%", X_MOD}},
    };
    if (lvl == (int)levels.size()) return unary(out);
    if (!binlevel(lvl + 1, out)) return false;
    for (;;) {
      int op = -1;
      if (tok_.kind == T_OP)
        for (auto& p : levels[lvl])
          if (tok_.op == p.first) op = p.second;
      if (op < 0) return true;
      int r;
      if (!advance() || !binlevel(lvl + 1, &r)) return false;
      *out = bin(op, *out, r);
    }
  }
  bool unary(int* out) {
    if (tok_.kind == T_OP && (tok_.op == "-" || tok_.op == "+" || tok_.op == "!" || tok_.op == "~")) {
      std::string o = tok_.op;
      if (!advance()) return false;
      int a;
      if (!unary(&a)) return false;
      if (o == "+") {
        *out = a;
        return true;
      }
      Node n{N_UNARY};
      n.op = o == "-" ? X_NEG : o == "!" ? X_NOT : X_BNOT;
      n.a = a;
      *out = add(n);
      return true;
    }
    return primary(out);
  }
  bool primary(int* out) {
    if (tok_.kind == T_NUM) {
      Node n{N_CONST};
      n.value = tok_.num;
      *out = add(n);
      return advance();
    }
    if (tok_.kind == T_COL) {
      Node n{N_COL};
      n.ref = tok_.ref;
      *out = add(n);
      return advance();
    }
    if (tok_.kind == T_LP) {
      if (!advance() || !cond(out)) return false;
      if (tok_.kind != T_RP) return fail("syntax: expected ')'");
      return advance();
    }
    if (tok_.kind == T_CALL) {  // StrCmp(column, "literal", n)
      if (!advance() || tok_.kind != T_LP) return fail("syntax: expected '(' after StrCmp");
      int col, n;
      if (!advance() || !cond(&col)) return false;
      if (tok_.kind != T_COMMA) return fail("syntax: expected ',' in StrCmp");
      if (!advance() || tok_.kind != T_STR) return fail("unsupported: StrCmp's second argument must be a string literal");
      std::string lit = tok_.op;
      if (!advance() || tok_.kind != T_COMMA) return fail("syntax: expected ',' in StrCmp");
      if (!advance() || !cond(&n)) return false;
      if (tok_.kind != T_RP) return fail("syntax: expected ')' after StrCmp's arguments");
      if (e_->nodes[col].kind != N_COL) return fail("unsupported: StrCmp's first argument must be a column");
      Node nd{N_STRCMP};
      nd.a = col;
      nd.b = n;
      nd.value = (int32_t)e_->strs.size();
      e_->strs.push_back(lit);
      *out = add(nd);
      return advance();
    }
    if (tok_.kind == T_STR) return fail("unsupported: a string literal outside StrCmp");
    if (tok_.kind == T_END) return fail("syntax: unexpected end of expression");
    return fail("syntax: unexpected token '" + tok_.op + "'");
  }

  Lexer lex_;
  Tok tok_;
  Expr* e_;
  std::string* err_;
};

int32_t apply_bin(int op, int32_t a, int32_t b, bool* div0) {
  uint32_t ua = (uint32_t)a, ub = (uint32_t)b;
  switch (op) {
    case X_ADD: return (int32_t)(ua + ub);
    case X_SUB: return (int32_t)(ua - ub);
    case X_MUL: return (int32_t)(ua * ub);
    case X_DIV:
      if (b == 0) { *div0 = true; return 0; }
      if (a == INT_MIN && b == -1) return INT_MIN;
      return a / b;
    case X_MOD:
      if (b == 0) { *div0 = true; return 0; }
      if (b == -1) return 0;
      return a % b;
    case X_SHL: return (int32_t)(ua << (ub & 31));
    case X_SHR: return a >> (ub & 31);
    case X_LT: return a < b;
    case X_LE: return a <= b;
    case X_GT: return a > b;
    case X_GE: return a >= b;
    case X_EQ: return a == b;
    case X_NE: return a != b;
    case X_BAND: return a & b;
    case X_BXOR: return a ^ b;
    case X_BOR: return a | b;
  }
  return 0;
}

struct Emitter {
  Prog* p;
  const std::vector<ColRef>* opnds;
  std::string* err;
  int depth = 0, max_depth = 0;
  int nconst = 0;

  bool emit(int op, int arg) {
    if (p->n >= kMaxProg) {
      *err = "unsupported: expression too long for the kernel bytecode";
      return false;
    }
    p->op[p->n] = (uint8_t)op;
    p->arg[p->n] = (uint8_t)arg;
    p->n++;
    return true;
  }
  void push(int k) {
    depth += k;
    if (depth > max_depth) max_depth = depth;
  }
  bool node(const Expr& e, int i) {
    const Node& n = e.nodes[i];
    int32_t v;
    if (n.kind != N_CONST && n.kind != N_COL && const_value(e, i, &v)) {
      return konst(v);
    }
    switch (n.kind) {
      case N_CONST: return konst(n.value);
      case N_COL: {
        for (size_t k = 0; k < opnds->size(); k++)
          if ((*opnds)[k] == n.ref) {
            push(1);
            return emit(X_OPND, (int)k);
          }
        *err = "internal: operand not bound";
        return false;
      }
      case N_UNARY:
        return node(e, n.a) && emit(n.op, 0);
      case N_BINARY:
        if (!node(e, n.a) || !node(e, n.b)) return false;
        push(-1);
        return emit(n.op, 0);
      case N_LAND:
      case N_LOR: {
        if (!node(e, n.a)) return false;
        int jpos = p->n;
        if (!emit(n.kind == N_LAND ? X_JZ_KEEP : X_JNZ_ONE, 0)) return false;
        push(-1);
        if (!node(e, n.b) || !emit(X_NORM, 0)) return false;
        p->arg[jpos] = (uint8_t)p->n;
        return true;
      }
      case N_STRCMP:
        *err = "unsupported: StrCmp left after string resolution";
        return false;
      case N_COND: {
        if (!node(e, n.a)) return false;
        int jz = p->n;
        if (!emit(X_JZ_POP, 0)) return false;
        push(-1);
        if (!node(e, n.b)) return false;
        int jmp = p->n;
        if (!emit(X_JMP, 0)) return false;
        push(-1);
        p->arg[jz] = (uint8_t)p->n;
        if (!node(e, n.c)) return false;
        p->arg[jmp] = (uint8_t)p->n;
        return true;
      }
    }
    return false;
  }
  bool konst(int32_t v) {
    for (int k = 0; k < nconst; k++)
      if (p->konst[k] == v) {
        push(1);
        return emit(X_CONST, k);
      }
    if (nconst >= 16) {
      *err = "unsupported: too many constants in one expression";
      return false;
    }
    p->konst[nconst] = v;
    push(1);
    return emit(X_CONST, nconst++);
  }
};

}  // namespace

bool parse_expr(const std::string& text, Expr* out, std::string* err) {
  out->nodes.clear();
  out->root = -1;
  err->clear();
  Parser p(text, out, err);
  return p.run();
}

std::vector<std::string> str_split(const std::string& s, const std::string& sep) {
  std::vector<std::string> ret;
  size_t pos1 = 0, pos2 = s.find(sep);
  while (pos2 != std::string::npos) {
    ret.push_back(s.substr(pos1, pos2 - pos1));
    pos1 = pos2 + sep.size();
    pos2 = s.find(sep, pos1);
  }
  if (pos1 != s.size()) ret.push_back(s.substr(pos1));
  return ret;
}

bool parse_key_index(const std::string& text, ColRef* out, std::string* err) {
  size_t p1 = text.find("$(");
  size_t p2 = p1 == std::string::npos ? p1 : text.find('.', p1);
  size_t p3 = p2 == std::string::npos ? p2 : text.find(')', p2);
  if (p3 == std::string::npos) {
    *err = "syntax: expected $(obj.col) in '" + text + "'";
    return false;
  }
  // std::stoi semantics: leading blanks, then digits; trailing text ignored.
  auto stoi_like = [](const std::string& s, int* v) {
    size_t i = 0;
    while (i < s.size() && isspace((unsigned char)s[i])) i++;
    size_t j = i;
    long long x = 0;
    while (j < s.size() && isdigit((unsigned char)s[j]) && x < 1000000) x = x * 10 + (s[j++] - '0');
    *v = (int)x;
    return j > i;
  };
  int obj, col;
  if (!stoi_like(text.substr(p1 + 2, p2 - p1 - 2), &obj) || !stoi_like(text.substr(p2 + 1), &col)) {
    *err = "syntax: bad key reference '" + text + "'";
    return false;
  }
  *out = {obj, col};
  return true;
}

void collect_refs(const Expr& e, int i, std::vector<ColRef>* refs) {
  if (i < 0) return;
  const Node& n = e.nodes[i];
  if (n.kind == N_COL) {
    for (auto& r : *refs)
      if (r == n.ref) return;
    refs->push_back(n.ref);
    return;
  }
  collect_refs(e, n.a, refs);
  collect_refs(e, n.b, refs);
  collect_refs(e, n.c, refs);
}

void flatten_and(const Expr& e, int i, std::vector<int>* conj) {
  const Node& n = e.nodes[i];
  if (n.kind == N_LAND) {
    flatten_and(e, n.a, conj);
    flatten_and(e, n.b, conj);
  } else {
    conj->push_back(i);
  }
}

bool const_value(const Expr& e, int i, int32_t* v) {
  const Node& n = e.nodes[i];
  int32_t a, b;
  bool div0 = false;
  switch (n.kind) {
    case N_CONST: *v = n.value; return true;
    case N_COL: return false;
    case N_UNARY:
      if (!const_value(e, n.a, &a)) return false;
      *v = n.op == X_NEG ? (int32_t)(0u - (uint32_t)a) : n.op == X_NOT ? !a : ~a;
      return true;
    case N_BINARY:
      if (!const_value(e, n.a, &a) || !const_value(e, n.b, &b)) return false;
      *v = apply_bin(n.op, a, b, &div0);
      return !div0;  // keep a constant division by zero for the kernel to report
    case N_LAND:
      if (!const_value(e, n.a, &a)) return false;
      if (!a) { *v = 0; return true; }
      if (!const_value(e, n.b, &b)) return false;
      *v = b != 0;
      return true;
    case N_LOR:
      if (!const_value(e, n.a, &a)) return false;
      if (a) { *v = 1; return true; }
      if (!const_value(e, n.b, &b)) return false;
      *v = b != 0;
      return true;
    case N_COND:
      if (!const_value(e, n.a, &a)) return false;
      return const_value(e, a ? n.b : n.c, v);
  }
  return false;
}

bool as_range(const Expr& e, int i, ColRef* ref, int32_t* lo, int32_t* hi) {
  const Node& n = e.nodes[i];
  if (n.kind != N_BINARY) return false;
  int op = n.op;
  if (op != X_LT && op != X_LE && op != X_GT && op != X_GE && op != X_EQ) return false;
  int32_t k;
  int col_side;
  if (e.nodes[n.a].kind == N_COL && const_value(e, n.b, &k)) {
    col_side = 0;
  } else if (e.nodes[n.b].kind == N_COL && const_value(e, n.a, &k)) {
    col_side = 1;
    op = op == X_LT ? X_GT : op == X_LE ? X_GE : op == X_GT ? X_LT : op == X_GE ? X_LE : op;
  } else {
    return false;
  }
  *ref = e.nodes[col_side == 0 ? n.a : n.b].ref;
  long long l = INT_MIN, h = INT_MAX, kk = k;
  if (op == X_LT) h = kk - 1;
  if (op == X_LE) h = kk;
  if (op == X_GT) l = kk + 1;
  if (op == X_GE) l = kk;
  if (op == X_EQ) l = h = kk;
  if (l > h || l > INT_MAX || h < INT_MIN) {
    *lo = 1;
    *hi = 0;  // empty
  } else {
    *lo = (int32_t)l;
    *hi = (int32_t)h;
  }
  return true;
}

bool compile_prog(const Expr& e, int node, const std::vector<ColRef>& opnd_of, Prog* p,
                  std::string* err) {
  *p = Prog{};
  Emitter em{p, &opnd_of, err};
  if (!em.node(e, node)) return false;
  if (em.max_depth > 16) {
    *err = "unsupported: expression nests too deeply for the kernel bytecode";
    return false;
  }
  return true;
}

int32_t eval_prog_host(const Prog& p, const int32_t* opnd, bool* div0) {
  int32_t st[16];
  int sp = 0;
  for (int pc = 0; pc < p.n;) {
    int op = p.op[pc], arg = p.arg[pc];
    pc++;
    switch (op) {
      case X_OPND: st[sp++] = opnd[arg]; break;
      case X_CONST: st[sp++] = p.konst[arg]; break;
      case X_NEG: st[sp - 1] = (int32_t)(0u - (uint32_t)st[sp - 1]); break;
      case X_NOT: st[sp - 1] = !st[sp - 1]; break;
      case X_BNOT: st[sp - 1] = ~st[sp - 1]; break;
      case X_NORM: st[sp - 1] = st[sp - 1] != 0; break;
      case X_JZ_KEEP: if (st[sp - 1] == 0) pc = arg; else sp--; break;
      case X_JNZ_ONE: if (st[sp - 1] != 0) { st[sp - 1] = 1; pc = arg; } else sp--; break;
      case X_JZ_POP: if (st[--sp] == 0) pc = arg; break;
      case X_JMP: pc = arg; break;
      default: {
        int32_t b = st[--sp];
        st[sp - 1] = apply_bin(op, st[sp - 1], b, div0);
      }
    }
  }
  return sp ? st[sp - 1] : 0;
}

}  // namespace svm
