"""ORACLE (test infrastructure only): an independent NumPy evaluation of a
pipeline's SQL meaning, used where the reference's capped hash table drops
nothing (then it equals the reference) and as the "exact" join semantics.

Expressions are parsed here with their own small recursive-descent parser and
evaluated with C int32 semantics (wrapping + - *, truncating / and %,
comparisons and && || giving 0/1), the semantics the reference's generated C
code has (codegen/codegen.cpp:240-277).  A join matches a key's FIRST row in
the joined object, as the reference's Probe returns the first inserted match
(com/cpp/cpu-runtime.hpp:125-138).

String columns are NumPy fixed-width byte arrays ('S<w>', w = the column's
val_size).  StrCmp(col, "lit", n) follows cpu-runtime.hpp:37-45 (compare at
most n bytes, stop at a NUL on either side, signed chars); a String ReduceBy
key is Hash(value, w) (cpu-runtime.hpp:68-74, signed chars); Map copies a
String into its output width, cut or NUL-padded (the reference's StrCopy
reads the following rows' bytes when the output is wider).
"""
from __future__ import annotations

import re

import numpy as np

from shadowvm_gb300.pipeline import str_split
from shadowvm_gb300.proto import OpType, PipelineInfo

_TOK = re.compile(r"\s*(\$\(\s*\d+\s*\.\s*\d+\s*\)|0[xX][0-9a-fA-F]+|\d+|<<|>>|<=|>=|==|!=|&&|\|\||[-+*/%<>!~&^|()?:])")
_LEVELS = [["|"], ["^"], ["&"], ["==", "!="], ["<", "<=", ">", ">="], ["<<", ">>"], ["+", "-"], ["*", "/", "%"]]


class Lit(str):
    """A string literal token."""


def tokenize(s: str) -> list[str]:
    out, i = [], 0
    s = s.rstrip()
    while i < len(s):
        while i < len(s) and s[i].isspace():
            i += 1
        if i >= len(s):
            break
        if s[i] == '"' or s.startswith('\\"', i):  # "lit" or \"lit\" (the Java DSL's form)
            esc = s[i] == "\\"
            j = i + (2 if esc else 1)
            v = []
            while True:
                if j >= len(s):
                    raise ValueError("unterminated string literal")
                if esc and s.startswith('\\"', j):
                    j += 2
                    break
                if not esc and s[j] == '"':
                    j += 1
                    break
                if s[j] == "\\" and j + 1 < len(s):
                    v.append({"0": "\0", "n": "\n", "t": "\t"}.get(s[j + 1], s[j + 1]))
                    j += 2
                    continue
                v.append(s[j])
                j += 1
            out.append(Lit("".join(v)))
            i = j
            continue
        if s.startswith("StrCmp", i):
            out.append("StrCmp")
            i += 6
            continue
        if s[i] == ",":
            out.append(",")
            i += 1
            continue
        m = _TOK.match(s, i)
        if not m:
            raise ValueError(f"cannot tokenize {s[i:]!r}")
        out.append(m.group(1))
        i = m.end()
    return out


def parse(s: str):
    toks = tokenize(s)
    pos = [0]

    def peek():
        return toks[pos[0]] if pos[0] < len(toks) else None

    def take():
        t = toks[pos[0]]
        pos[0] += 1
        return t

    def cond():
        c = lor()
        if peek() == "?":
            take()
            a = cond()
            assert take() == ":"
            b = cond()
            return ("?", c, a, b)
        return c

    def lor():
        a = land()
        while peek() == "||":
            take()
            a = ("||", a, land())
        return a

    def land():
        a = level(0)
        while peek() == "&&":
            take()
            a = ("&&", a, level(0))
        return a

    def level(k):
        if k == len(_LEVELS):
            return unary()
        a = level(k + 1)
        while peek() in _LEVELS[k]:
            op = take()
            a = (op, a, level(k + 1))
        return a

    def unary():
        if peek() in ("-", "+", "!", "~"):
            op = take()
            a = unary()
            return a if op == "+" else ("u" + op, a)
        return primary()

    def primary():
        t = take()
        if t == "StrCmp" and not isinstance(t, Lit):
            assert take() == "("
            col = cond()
            assert take() == ","
            lit = take()
            assert isinstance(lit, Lit), "StrCmp's second argument must be a string literal"
            assert take() == ","
            n = cond()
            assert take() == ")"
            return ("strcmp", col, str(lit), n)
        if t == "(":
            a = cond()
            assert take() == ")"
            return a
        if t.startswith("$("):
            o, c = t[2:-1].split(".")
            return ("col", int(o), int(c))
        if t.lower().startswith("0x"):
            return ("const", int(t, 16))
        if len(t) > 1 and t.startswith("0"):
            return ("const", int(t, 8))
        return ("const", int(t))

    tree = cond()
    if pos[0] != len(toks):
        raise ValueError(f"trailing tokens in {s!r}")
    return tree


def _i32(x):
    return np.asarray(x, dtype=np.int64).astype(np.int32)


def _sbytes(v: bytes, i: int) -> int:
    return (v[i] ^ 0x80) - 0x80 if i < len(v) else 0  # signed char, NUL past the value


def strcmp_value(v: bytes, width: int, lit: str, n: int) -> int:
    """StrCmp(value, lit, n) of a value of `width` bytes (cpu-runtime.hpp:37-45)."""
    lb = lit.encode("utf-8")  # the bytes the pipeline's text carries
    for i in range(n):
        if i >= width:
            raise ValueError("unsupported: StrCmp reads past the column's width (the next row's bytes)")
        a, b = _sbytes(v, i), _sbytes(lb, i)
        if a == 0 or b == 0:
            return 0
        if a != b:
            return a - b
    return 0


def hash_value(v: bytes, width: int) -> int:
    """Hash(value, width) (cpu-runtime.hpp:68-74), signed chars."""
    h = 0
    for i in range(width):
        h = (h * 31 + _sbytes(v, i)) & 0xFFFFFFFF
    return h & 0x7FFFFFFF


def _per_value(arr: np.ndarray, fn) -> np.ndarray:
    """fn over the distinct values of a String array, mapped back to rows."""
    uniq, inv = np.unique(arr, return_inverse=True)
    vals = np.array([fn(bytes(u)) for u in uniq], np.int64)
    return vals[inv.reshape(-1)] if len(arr) else np.zeros(0, np.int64)


def _num(a: np.ndarray) -> np.ndarray:
    if a.dtype.kind == "S":
        raise ValueError("unsupported: a String column used as a number")
    return a


def evaluate(tree, env, n: int) -> np.ndarray:
    """env[(obj, col)] -> int32 array (or 'S<w>' bytes for a String column) of length n."""
    op = tree[0]
    if op == "const":
        return np.full(n, tree[1], np.int64).astype(np.int32)
    if op == "col":
        return _num(env[(tree[1], tree[2])])
    if op == "strcmp":
        col = env[(tree[1][1], tree[1][2])]
        if tree[1][0] != "col" or col.dtype.kind != "S":
            raise ValueError("unsupported: StrCmp of a column that is not a String")
        nn = int(evaluate(tree[3], env, 1)[0])
        w = col.dtype.itemsize
        return _per_value(col, lambda v: strcmp_value(v, w, tree[2], nn)).astype(np.int32)
    if op == "?":
        c = evaluate(tree[1], env, n)
        return np.where(c != 0, evaluate(tree[2], env, n), evaluate(tree[3], env, n)).astype(np.int32)
    if op == "u-":
        return _i32(-evaluate(tree[1], env, n).astype(np.int64))
    if op == "u!":
        return (evaluate(tree[1], env, n) == 0).astype(np.int32)
    if op == "u~":
        return ~evaluate(tree[1], env, n)
    a = evaluate(tree[1], env, n).astype(np.int64)
    b = evaluate(tree[2], env, n).astype(np.int64)
    if op == "&&":
        return ((a != 0) & (b != 0)).astype(np.int32)
    if op == "||":
        return ((a != 0) | (b != 0)).astype(np.int32)
    if op in ("+", "-", "*"):
        r = a + b if op == "+" else a - b if op == "-" else a * b
        return _i32(r & 0xFFFFFFFF)
    if op in ("/", "%"):
        if np.any(b == 0):
            raise ZeroDivisionError("division by zero in expression")
        q = np.abs(a) // np.abs(b) * np.sign(a) * np.sign(b)
        return _i32(q if op == "/" else a - q * b)
    if op == "<<":
        return _i32((a << (b & 31)) & 0xFFFFFFFF)
    if op == ">>":
        return _i32(a >> (b & 31))
    cmp = {"<": np.less, "<=": np.less_equal, ">": np.greater, ">=": np.greater_equal,
           "==": np.equal, "!=": np.not_equal}
    if op in cmp:
        return cmp[op](a, b).astype(np.int32)
    bit = {"&": np.bitwise_and, "|": np.bitwise_or, "^": np.bitwise_xor}
    return _i32(bit[op](a, b))


def _bind(p: PipelineInfo):
    filt, sel, met, dims, joins, reduce = [], None, None, None, [], False
    for op in p.workflow:
        if op.type == OpType.Filter:
            filt.append(op.args["predication"])
        elif op.type == OpType.Map:
            sel = str_split(op.args["select"], ",")
        elif op.type == OpType.ReduceBy:
            met = str_split(op.args["metric"], ",")
            dims = str_split(op.args.get("dim", ""), ",")
            reduce = True
        elif op.type == OpType.JoinWith:
            joins.append((op.args["lkey"], op.args["rkey"]))
    return filt, sel, met, dims, joins, reduce


def _keyref(s: str) -> tuple[int, int]:
    m = re.search(r"\$\(\s*(\d+)\s*\.\s*(\d+)", s)
    return int(m.group(1)), int(m.group(2))


def _col(v) -> np.ndarray:
    a = np.asarray(v)
    return a if a.dtype.kind == "S" else a.astype(np.int32)


def run_select(p: PipelineInfo, cols: list[np.ndarray]) -> list[np.ndarray]:
    filt, sel, *_ = _bind(p)
    n = len(cols[0]) if cols else 0
    env = {(0, c): _col(v) for c, v in enumerate(cols)}
    mask = np.ones(n, bool)
    if filt:
        mask = evaluate(parse("&&".join(filt)), env, n) != 0
    out_schema = [op.output for op in p.workflow if op.type == OpType.Map][0].column_list
    res = []
    for i, e in enumerate(sel):
        t = parse(e)
        if t[0] == "col" and env[(t[1], t[2])].dtype.kind == "S":  # a String copy into its output width
            res.append(env[(t[1], t[2])][mask].astype(f"S{int(out_schema[i].val_size)}"))
        else:
            res.append(evaluate(t, env, n)[mask])
    return res


def run_join_select(p: PipelineInfo, fact: list[np.ndarray], dims: list[list[np.ndarray]]) -> list[np.ndarray]:
    """A Map pipeline with joins (the reference's join block, then its select
    block, codegen/codegen.cpp:121-180): rows passing the filter whose every
    join key has a match (the first dimension row with that key), projected
    in row order."""
    filt, sel, _, _, joins, _ = _bind(p)
    n = len(fact[0]) if fact else 0
    env = {(0, c): _col(v) for c, v in enumerate(fact)}
    mask = np.ones(n, bool)
    if filt and n:
        mask = evaluate(parse("&&".join(filt)), env, n) != 0
    for lk, rk in joins:
        lo, lc = _keyref(lk)
        ro, rc = _keyref(rk)
        idx = first_match(np.asarray(dims[ro - 1][rc], np.int32), _num(env[(lo, lc)]))
        mask &= idx >= 0
        safe = np.where(idx >= 0, idx, 0)
        for c, col in enumerate(dims[ro - 1]):
            col = _col(col)
            env[(ro, c)] = col[safe] if len(col) else np.zeros(n, col.dtype)
    sub = {k: v[mask] for k, v in env.items()}
    m = int(mask.sum())
    return [evaluate(parse(e), sub, m).astype(np.int32) for e in sel]


def first_match(dim_keys: np.ndarray, probe: np.ndarray) -> np.ndarray:
    """Index of the first row of dim_keys equal to each probe value, else -1."""
    if len(dim_keys) == 0:
        return np.full(len(probe), -1, np.int64)
    uniq, first = np.unique(dim_keys, return_index=True)
    pos = np.searchsorted(uniq, probe)
    pos_c = np.minimum(pos, len(uniq) - 1)
    hit = uniq[pos_c] == probe
    return np.where(hit, first[pos_c], -1).astype(np.int64)


def run_reduce(p: PipelineInfo, fact: list[np.ndarray], dims: list[list[np.ndarray]],
               metric_wide: list[bool] | None = None):
    """Returns (keys int32 [g, k], sums int64 [g, m]) sorted by key; an empty
    fact table gives no rows (the reference runs no bulk task)."""
    filt, _, met, keyexp, joins, _ = _bind(p)
    n = len(fact[0]) if fact else 0
    nk = len(keyexp)
    if n == 0:
        return np.zeros((0, nk), np.int32), np.zeros((0, len(met)), np.int64)
    env = {(0, c): _col(v) for c, v in enumerate(fact)}
    mask = np.ones(n, bool)
    if filt:
        mask = evaluate(parse("&&".join(filt)), env, n) != 0
    for lk, rk in joins:
        lo, lc = _keyref(lk)
        ro, rc = _keyref(rk)
        idx = first_match(np.asarray(dims[ro - 1][rc], np.int32), _num(env[(lo, lc)]))
        mask &= idx >= 0
        safe = np.where(idx >= 0, idx, 0)
        for c, col in enumerate(dims[ro - 1]):
            col = _col(col)
            env[(ro, c)] = col[safe] if len(col) else np.zeros(n, col.dtype)
    sub = {k: v[mask] for k, v in env.items()}
    m = int(mask.sum())
    vals = [evaluate(parse(e), sub, m).astype(np.int64) for e in met]
    if metric_wide is None:
        metric_wide = [True] * len(met)
    if nk == 0:
        sums = [int(v.sum(dtype=np.int64)) for v in vals]
        sums = [s if w else int(np.int64(s).astype(np.int32)) for s, w in zip(sums, metric_wide)]
        return np.zeros((1, 0), np.int32), np.array([sums], np.int64)
    def key(e):  # a String key is its Hash over the column's width
        a = sub[_keyref(e)]
        if a.dtype.kind == "S":
            w = a.dtype.itemsize
            return _per_value(a, lambda v: hash_value(v, w)).astype(np.int32)
        return a
    keys = np.stack([key(e) for e in keyexp], axis=1) if m else np.zeros((0, nk), np.int32)
    if m == 0:
        return np.zeros((0, nk), np.int32), np.zeros((0, len(met)), np.int64)
    uniq, inv = np.unique(keys, axis=0, return_inverse=True)
    inv = inv.reshape(-1)
    order = np.argsort(inv, kind="stable")
    starts = np.searchsorted(inv[order], np.arange(len(uniq)))
    sums = np.zeros((len(uniq), len(met)), np.int64)
    for j, v in enumerate(vals):
        s = np.add.reduceat(v[order], starts)
        sums[:, j] = s if metric_wide[j] else s.astype(np.int32)
    return uniq.astype(np.int32), sums
