"""ORACLE (test infrastructure only): an independent NumPy evaluation of a
pipeline's SQL meaning, used where the reference's capped hash table drops
nothing (then it equals the reference) and as the "exact" join semantics.

Expressions are parsed here with their own small recursive-descent parser and
evaluated with C int32 semantics (wrapping + - *, truncating / and %,
comparisons and && || giving 0/1), the semantics the reference's generated C
code has (codegen/codegen.cpp:240-277).  A join matches a key's FIRST row in
the joined object, as the reference's Probe returns the first inserted match
(com/cpp/cpu-runtime.hpp:125-138).
"""
from __future__ import annotations

import re

import numpy as np

from shadowvm_gb300.pipeline import str_split
from shadowvm_gb300.proto import OpType, PipelineInfo

_TOK = re.compile(r"\s*(\$\(\s*\d+\s*\.\s*\d+\s*\)|0[xX][0-9a-fA-F]+|\d+|<<|>>|<=|>=|==|!=|&&|\|\||[-+*/%<>!~&^|()?:])")
_LEVELS = [["|"], ["^"], ["&"], ["==", "!="], ["<", "<=", ">", ">="], ["<<", ">>"], ["+", "-"], ["*", "/", "%"]]


def tokenize(s: str) -> list[str]:
    out, i = [], 0
    s = s.rstrip()
    while i < len(s):
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


def evaluate(tree, env, n: int) -> np.ndarray:
    """env[(obj, col)] -> int32 array of length n."""
    op = tree[0]
    if op == "const":
        return np.full(n, tree[1], np.int64).astype(np.int32)
    if op == "col":
        return env[(tree[1], tree[2])]
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


def run_select(p: PipelineInfo, cols: list[np.ndarray]) -> list[np.ndarray]:
    filt, sel, *_ = _bind(p)
    n = len(cols[0]) if cols else 0
    env = {(0, c): np.asarray(v, np.int32) for c, v in enumerate(cols)}
    mask = np.ones(n, bool)
    if filt:
        mask = evaluate(parse("&&".join(filt)), env, n) != 0
    return [evaluate(parse(e), env, n)[mask] for e in sel]


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
    env = {(0, c): np.asarray(v, np.int32) for c, v in enumerate(fact)}
    mask = np.ones(n, bool)
    if filt:
        mask = evaluate(parse("&&".join(filt)), env, n) != 0
    for lk, rk in joins:
        lo, lc = _keyref(lk)
        ro, rc = _keyref(rk)
        idx = first_match(np.asarray(dims[ro - 1][rc], np.int32), env[(lo, lc)])
        mask &= idx >= 0
        safe = np.where(idx >= 0, idx, 0)
        for c, col in enumerate(dims[ro - 1]):
            col = np.asarray(col, np.int32)
            env[(ro, c)] = col[safe] if len(col) else np.zeros(n, np.int32)
    sub = {k: v[mask] for k, v in env.items()}
    m = int(mask.sum())
    vals = [evaluate(parse(e), sub, m).astype(np.int64) for e in met]
    if metric_wide is None:
        metric_wide = [True] * len(met)
    if nk == 0:
        sums = [int(v.sum(dtype=np.int64)) for v in vals]
        sums = [s if w else int(np.int64(s).astype(np.int32)) for s, w in zip(sums, metric_wide)]
        return np.zeros((1, 0), np.int32), np.array([sums], np.int64)
    keys = np.stack([sub[_keyref(e)] for e in keyexp], axis=1) if m else np.zeros((0, nk), np.int32)
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
