"""Seeded, counter-based synthetic star-schema data.

Every value is a pure function of (seed, column id, row index), so a row range
can be generated anywhere -- here in NumPy, on the GPU by the library's
``svm_gen_uniform`` kernel, or inside the oracle -- and the results are
bit-identical.  The mixer is splitmix64's output function (Steele, Lea and
Flood, "Fast splittable pseudorandom number generators", OOPSLA 2014); a value
in ``[lo, hi]`` is ``lo + ((u >> 32) * (hi - lo + 1)) >> 32``.

The table shapes follow the star-schema workloads the reference was built for
(lineorder / date / part / customer / supplier, cf. test/test-load.cu:69-119 and
example/svm_load_SSB.cu:10-75); the SSB dbgen files themselves are not used --
these are synthetic columns with the same shapes and value ranges.
"""
from __future__ import annotations

import datetime as _dt

import numpy as np

GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)
_STREAM = np.uint64(0xD1B54A32D192ED03)

DEFAULT_SEED = 20190306

# Column ids: every generated column draws from its own stream.
COL = {
    "orderdate": 1, "quantity": 2, "discount": 3, "extprice": 4,
    "partkey": 5, "custkey": 6, "suppkey": 7, "revenue": 8, "supplycost": 9,
    "p_category": 21, "p_brand_lo": 22,
    "c_city": 31, "s_city": 41,
}

# Fact column value ranges (inclusive).  FK columns draw a dimension ROW index.
RANGES = {
    "quantity": (1, 50), "discount": (0, 10), "extprice": (90_000, 10_500_000),
    "revenue": (100, 1_000_000), "supplycost": (50, 600_000),
}

N_DATE = 2557


def mix64(z: np.ndarray) -> np.ndarray:
    """splitmix64 output function applied to ``z + golden`` (wrapping uint64)."""
    with np.errstate(over="ignore"):
        z = z + GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def stream_key(seed: int, col_id: int) -> np.uint64:
    with np.errstate(over="ignore"):
        x = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) ^ (np.uint64(col_id) * _STREAM)
    return mix64(np.array([x], dtype=np.uint64))[0]


def uniform(seed: int, col_id: int, lo: int, hi: int, row0: int, n: int) -> np.ndarray:
    """int32 values uniform in [lo, hi] for rows row0 .. row0+n-1."""
    key = stream_key(seed, col_id)
    rows = np.arange(row0, row0 + n, dtype=np.uint64)
    with np.errstate(over="ignore"):
        u = mix64(rows + key)
    span = np.uint64(hi - lo + 1)
    off = ((u >> np.uint64(32)) * span) >> np.uint64(32)
    return (off.astype(np.int64) + lo).astype(np.int32)


def draw(seed: int, stream: int, lo: int, hi: int) -> int:
    """One seeded scalar in [lo, hi] (query constants)."""
    return int(uniform(seed, 1000 + stream, lo, hi, 0, 1)[0])


# ---------------------------------------------------------------- dimensions
def date_table() -> dict[str, np.ndarray]:
    """Every day 1992-01-01 .. 1998-12-31: datekey yyyymmdd, year, month."""
    d0 = _dt.date(1992, 1, 1)
    days = [d0 + _dt.timedelta(days=i) for i in range(N_DATE)]
    assert days[-1] == _dt.date(1998, 12, 31)
    return {
        "datekey": np.array([d.year * 10000 + d.month * 100 + d.day for d in days], np.int32),
        "year": np.array([d.year for d in days], np.int32),
        "month": np.array([d.month for d in days], np.int32),
    }


def part_table(n: int, seed: int = DEFAULT_SEED) -> dict[str, np.ndarray]:
    """partkey = row; category U[0,24]; brand = category*40 + U[0,39] (so brand
    is uniform over 0..999 and nests inside category)."""
    cat = uniform(seed, COL["p_category"], 0, 24, 0, n)
    lo = uniform(seed, COL["p_brand_lo"], 0, 39, 0, n)
    return {"partkey": np.arange(n, dtype=np.int32), "category": cat,
            "brand": (cat * 40 + lo).astype(np.int32)}


def geo_table(n: int, city_col: int, seed: int = DEFAULT_SEED) -> dict[str, np.ndarray]:
    """key = row; city U[0,249]; nation = city/10; region = nation/5."""
    city = uniform(seed, city_col, 0, 249, 0, n)
    nation = (city // 10).astype(np.int32)
    return {"key": np.arange(n, dtype=np.int32), "city": city, "nation": nation,
            "region": (nation // 5).astype(np.int32)}


def customer_table(n: int = 3_000_000, seed: int = DEFAULT_SEED):
    return geo_table(n, COL["c_city"], seed)


def supplier_table(n: int = 200_000, seed: int = DEFAULT_SEED):
    return geo_table(n, COL["s_city"], seed)


# ---------------------------------------------------------------- fact
def fact_column(name: str, row0: int, n: int, *, seed: int = DEFAULT_SEED,
                n_part: int = 400_000, n_cust: int = 3_000_000, n_supp: int = 200_000,
                datekeys: np.ndarray | None = None) -> np.ndarray:
    cid = COL[name]
    if name == "orderdate":
        idx = uniform(seed, cid, 0, N_DATE - 1, row0, n)
        dk = date_table()["datekey"] if datekeys is None else datekeys
        return dk[idx]
    if name == "partkey":
        return uniform(seed, cid, 0, n_part - 1, row0, n)
    if name == "custkey":
        return uniform(seed, cid, 0, n_cust - 1, row0, n)
    if name == "suppkey":
        return uniform(seed, cid, 0, n_supp - 1, row0, n)
    lo, hi = RANGES[name]
    return uniform(seed, cid, lo, hi, row0, n)
