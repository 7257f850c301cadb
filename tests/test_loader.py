"""The text Loader (core/operator.cpp:24-48): the oracle's restatement
pinned to the C library's own atoi/atol, its line/field rules, and (GPU)
the device loader bit-exact against it."""
import ctypes
import random

import numpy as np
import pytest

import oracle
from shadowvm_gb300.proto import ValType
from shadowvm_gb300.workloads import ssb_like_text

I32, I64 = int(ValType.Int32), int(ValType.Int64)

ITEMS = ["42", " 42", "\t\v\f\r 7", "-7", "+3", "", "abc", "12abc", "  -0012", "0x1A", "- 5", "+-5",
         "2147483647", "2147483648", "-2147483648", "-2147483649", "4294967296", "99999999999999999999",
         "-99999999999999999999", "9223372036854775807", "9223372036854775808", "-9223372036854775808",
         "-9223372036854775809", "000000000000000000000000123", "1 2", "7\x00 8", "3.9", "٣"]


def test_conversion_matches_libc_atoi_atol():
    libc = ctypes.CDLL(None)
    libc.atoi.restype, libc.atoi.argtypes = ctypes.c_int, [ctypes.c_char_p]
    libc.atol.restype, libc.atol.argtypes = ctypes.c_long, [ctypes.c_char_p]
    rng = random.Random(5)
    items = [s.encode("utf-8") for s in ITEMS] + \
        [(" " * rng.randint(0, 2) + rng.choice(["", "-", "+"]) + str(rng.randint(0, 10 ** rng.randint(1, 22)))).encode()
         for _ in range(300)]
    items = [it for it in items if b"|" not in it and b"\n" not in it]
    text = b"".join(it + b"|" + it + b"|\n" for it in items)
    n, (a, b) = oracle.load_text(text, [I32, I64])
    assert n == len(items)
    for k, it in enumerate(items):
        c = it.split(b"\x00")[0]  # C strings end at the first NUL
        assert a[k] == libc.atoi(c), it
        assert b[k] == libc.atol(c), it


def test_line_and_field_rules():
    text = (b"1|2|3|\n"          # three fields
            b"4|5|6\n"           # the 6 has no column delimiter after it: dropped
            b"7|\n"              # missing fields stay 0
            b"8|9|10|11|12|\n"   # fields past the schema are ignored
            b"\n"                # an empty line is a row of zeros
            b"13|14|15|")        # no row delimiter: not a row
    n, cols = oracle.load_text(text, [I32, I32, I64])
    assert n == 5
    assert [c.tolist() for c in cols] == [[1, 4, 7, 8, 0], [2, 5, 0, 9, 0], [3, 0, 0, 10, 0]]
    n, cols = oracle.load_text(b"a,b;1,2;", [I32, I32], ",", ";")
    assert n == 2 and [c.tolist() for c in cols] == [[0, 1], [0, 0]]  # "b" and "2" end at the row delimiter
    with pytest.raises(ValueError):
        oracle.load_text(b"1" * 4096 + b"|\n", [I32])
    assert oracle.load_text(b"1" * 4095 + b"|\n", [I64])[1][0][0] == 9223372036854775807


def test_fixed_width_generator_round_trips():
    text, cols = ssb_like_text(500, 4, 3)
    n, got = oracle.load_text(text, [I64] * 4)
    assert n == 500
    for g, c in zip(got, cols):
        np.testing.assert_array_equal(g, c)


# ---------------------------------------------------------------- GPU
def adversarial_text(seed: int, rows: int) -> bytes:
    rng = random.Random(seed)
    parts = []
    for _ in range(rows):
        k = rng.randint(0, 7)
        fields = []
        for _ in range(k):
            r = rng.random()
            if r < 0.05:
                fields.append(" " * rng.randint(0, 300) + str(rng.randint(-10 ** 6, 10 ** 6)))  # long items
            elif r < 0.1:
                fields.append(rng.choice(ITEMS))
            else:
                fields.append(str(rng.randint(-2 ** 40, 2 ** 40)))
        line = "|".join(fields) + ("|" if rng.random() < 0.8 else "")
        parts.append(line)
    return ("\n".join(parts) + "\n").encode("utf-8")


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [1, 2])
def test_gpu_loader_equals_oracle(engine_factory, seed):
    eng = engine_factory()
    types = [I32, I64, I32, I32, I64]
    text = adversarial_text(seed, 20_000)
    n = eng.load_text("t", text, types)
    en, ecols = oracle.load_text(text, types)
    assert n == en
    for k in range(len(types)):
        np.testing.assert_array_equal(eng.read("t", k), ecols[k], err_msg=f"column {k}")


@pytest.mark.gpu
def test_gpu_loader_device_text_at_every_alignment(engine_factory):
    """Device text starting at each of the 16 byte offsets, surrounded by
    delimiters: a loader that read outside [text, text + bytes) would count
    them."""
    import torch
    eng = engine_factory()
    types = [I64, I32, I64]
    text = adversarial_text(3, 3000)
    en, ecols = oracle.load_text(text, types)
    src = torch.frombuffer(bytearray(text), dtype=torch.uint8).cuda()
    fill = torch.frombuffer(bytearray(b"|\n" * (len(text) // 2 + 40)), dtype=torch.uint8).cuda()
    for off in range(16):
        buf = fill.clone()
        buf[off:off + len(text)] = src
        n = eng.load_text("a", None, types, device_ptr=buf.data_ptr() + off, nbytes=len(text))
        assert n == en, off
        for k in range(len(types)):
            np.testing.assert_array_equal(eng.read("a", k), ecols[k], err_msg=f"offset {off} column {k}")


@pytest.mark.gpu
@pytest.mark.parametrize("cd,rd", [(" ", "\n"), (",", ";"), ("\t", "\n"), ("5", "\n"), ("-", "|")])
def test_gpu_loader_other_delimiters(engine_factory, cd, rd):
    """Delimiters that can be part of a number or of whitespace (space, tab,
    a digit, a sign): the field walks must stop at the field's end."""
    eng = engine_factory()
    rng = random.Random(ord(cd) * 31 + ord(rd))
    lines = []
    for _ in range(3000):
        fields = [" " * rng.randint(0, 3) + rng.choice(["", "-", "+"]) + str(rng.randint(0, 10 ** rng.randint(1, 12)))
                  for _ in range(rng.randint(0, 6))]
        lines.append(cd.join(fields) + (cd if rng.random() < 0.7 else ""))
    text = (rd.join(lines) + rd).encode()
    types = [I32, I64, I32, I64]
    n = eng.load_text("d", text, types, col_delim=cd, row_delim=rd)
    en, ecols = oracle.load_text(text, types, cd, rd)
    assert n == en
    for k in range(len(types)):
        np.testing.assert_array_equal(eng.read("d", k), ecols[k], err_msg=f"column {k}")


@pytest.mark.gpu
def test_gpu_loader_edges(engine_factory):
    eng = engine_factory()
    for text in [b"", b"\n", b"1|2|", b"1|2|\n", b"|||\n||\n", b"5|" * 100 + b"\n",
                 b"x" * 5000 + b"\n3|\n", (b"7|\n" * 1000)[:-1]]:
        n = eng.load_text("e", text, [I32, I64])
        en, ecols = oracle.load_text(text, [I32, I64])
        assert n == en, text[:40]
        if n:
            np.testing.assert_array_equal(eng.read("e", 0), ecols[0])
            np.testing.assert_array_equal(eng.read("e", 1), ecols[1])
    from shadowvm_gb300 import SvmError
    with pytest.raises(SvmError):
        eng.load_text("e", b"1" * 4096 + b"|\n", [I32])


@pytest.mark.gpu
def test_gpu_loader_large_fixed_width_and_query(engine_factory):
    """100 MB of SSB-like text; then the loaded columns answer a query as
    the same columns put directly do."""
    from shadowvm_gb300 import workloads as W
    eng = engine_factory(tuple_per_bulk=1_000_000)
    text, cols = ssb_like_text(1_000_000, 9, 11)
    n = eng.load_text("big", text, [I64] * 9)
    assert n == 1_000_000
    for k in range(9):
        np.testing.assert_array_equal(eng.read("big", k), cols[k])
    # config-0 fact columns as text, loaded and queried
    w = W.make(0, fact_rows=300_000, tuple_per_bulk=100_000)
    fact = w.fact_host(0, w.fact_rows)
    lines = "\n".join("|".join(str(int(c[i])) for c in fact) + "|" for i in range(w.fact_rows)) + "\n"
    eng2 = engine_factory(tuple_per_bulk=w.tuple_per_bulk)
    for name, dcols in w.dims.items():
        eng2.put(name, dcols)
    assert eng2.load_text("lineorder", lines.encode(), [I32] * len(fact)) == w.fact_rows
    k_text, s_text = W.run_engine(eng2, w)
    ek, es = oracle.exact_workload(w)
    eng3 = engine_factory(tuple_per_bulk=w.tuple_per_bulk, join_mode="exact")
    for name, dcols in w.dims.items():
        eng3.put(name, dcols)
    eng3.load_text("lineorder", lines.encode(), [I32] * len(fact))
    k3, s3 = W.run_engine(eng3, w)
    np.testing.assert_array_equal(k3, ek)
    np.testing.assert_array_equal(s3, es)
