"""svm_scan_aggregate_noalloc: the allocation-free variant of the fused scan.

It exists for callers that cannot allocate device memory on their query path
(a runtime that owns all device memory through its own pool, a thread that
must not take cudaMalloc's implicit device-wide synchronisation).  Its scratch
is a static device array shared by every call, so this checks, through the C
ABI, that two calls in a row each give exactly the rows svm_run_pipeline gives
for the equivalent Filter/ReduceBy pipeline (integer sums: bit-exact), that a
grouped call equals an independent NumPy group-by, that a query too large for
the array is refused, and that its error paths (a key outside its declared
range, too few output rows, an unaligned column) report their own status and
leave the shared scratch usable.  The test's own buffers are
allocated by the test, never by the entry point.

This file is collected last so that a failure here comes after every other test.
"""
import ctypes

import numpy as np
import pytest

from shadowvm_gb300 import capi
from shadowvm_gb300.pipeline import fact_pipeline
from shadowvm_gb300.workloads import int_schema

pytestmark = pytest.mark.gpu


def _arr(ctype, values):
    return (ctype * max(len(values), 1))(*values)


def noalloc(eng, ptrs, nrows, ranges, keys, metrics, max_rows):
    """Calls the entry point; returns (keys [g, k] int32, sums [g, m] int64)."""
    import torch
    dev = torch.device("cuda")
    key_t = [torch.full((max_rows,), -7, dtype=torch.int32, device=dev) for _ in keys]
    sum_t = [torch.full((max_rows,), -7, dtype=torch.int64, device=dev) for _ in metrics]
    torch.cuda.synchronize()
    q = capi.svm_noalloc_scan()
    q.ncols = len(ptrs)
    q.cols = _arr(ctypes.c_void_p, ptrs)
    q.nrows = nrows
    q.nranges = len(ranges)
    q.range_col = _arr(ctypes.c_int, [r[0] for r in ranges])
    q.range_lo = _arr(ctypes.c_int, [r[1] for r in ranges])
    q.range_hi = _arr(ctypes.c_int, [r[2] for r in ranges])
    q.nkeys = len(keys)
    q.key_col = _arr(ctypes.c_int, [k[0] for k in keys])
    q.key_min = _arr(ctypes.c_int, [k[1] for k in keys])
    q.key_max = _arr(ctypes.c_int, [k[2] for k in keys])
    q.nmetrics = len(metrics)
    q.metric_op = _arr(ctypes.c_int, [m[0] for m in metrics])
    q.metric_a = _arr(ctypes.c_int, [m[1] for m in metrics])
    q.metric_b = _arr(ctypes.c_int, [m[2] for m in metrics])
    kp = _arr(ctypes.c_void_p, [t.data_ptr() for t in key_t])
    sp = _arr(ctypes.c_void_p, [t.data_ptr() for t in sum_t])
    out = ctypes.c_ulonglong(12345)
    st = eng.lib.svm_scan_aggregate_noalloc(eng.h, ctypes.byref(q), kp, sp, max_rows, ctypes.byref(out))
    if st != capi.OK:
        raise capi.SvmError(st, (eng.lib.svm_last_error(eng.h) or b"").decode())
    g = out.value
    k = np.stack([t[:g].cpu().numpy() for t in key_t], axis=1) if keys else np.zeros((g, 0), np.int32)
    s = np.stack([t[:g].cpu().numpy() for t in sum_t], axis=1)
    return k, s


@pytest.fixture(scope="module")
def table(engine_factory):
    eng = engine_factory(tuple_per_bulk=100_000)
    rng = np.random.default_rng(11)
    n = 1_000_003
    cols = [rng.integers(0, 50, n, dtype=np.int32), rng.integers(-1000, 1000, n, dtype=np.int32),
            rng.integers(0, 7, n, dtype=np.int32), rng.integers(1, 1_000_000, n, dtype=np.int32)]
    eng.put("nf", cols)
    ptrs = [eng.device_ptr("nf", c) for c in range(4)]
    return eng, ptrs, n


def test_noalloc_grouped_matches_run_pipeline_twice(table):
    eng, ptrs, n = table
    eng.run(fact_pipeline("nq", "nf", int_schema(4), [], [], "$(0.2),$(0.0)",
                          "$(0.3),$(0.3)*$(0.1),$(0.1)-$(0.0)",
                          predication="$(0.0)>=10 && $(0.0)<=40 && $(0.1)>=-500"))
    want_k, want_s = eng.result("nq", 2)
    ranges = [(0, 10, 40), (1, -500, 2**31 - 1)]
    keys = [(2, 0, 6), (0, 0, 49)]
    metrics = [(capi.METRIC_COL, 3, 3), (capi.METRIC_MUL, 3, 1), (capi.METRIC_SUB, 1, 0)]
    for _ in range(2):  # the second call must not see the first call's slots
        k, s = noalloc(eng, ptrs, n, ranges, keys, metrics, max_rows=7 * 50)
        np.testing.assert_array_equal(k, want_k)
        np.testing.assert_array_equal(s, want_s)


def test_noalloc_scalar_matches_run_pipeline_twice(table):
    eng, ptrs, n = table
    eng.run(fact_pipeline("ns", "nf", int_schema(4), [], [], "", "$(0.3)+$(0.1)",
                          predication="$(0.2)==3"))
    _, want_s = eng.result("ns", 0)
    for _ in range(2):
        k, s = noalloc(eng, ptrs, n, [(2, 3, 3)], [], [(capi.METRIC_ADD, 3, 1)], max_rows=1)
        assert k.shape == (1, 0)
        np.testing.assert_array_equal(s, want_s)


def test_noalloc_rejects_groups_beyond_the_static_scratch(table):
    eng, ptrs, n = table
    with pytest.raises(capi.SvmError) as e:
        noalloc(eng, ptrs, n, [], [(3, 0, 999_999)], [(capi.METRIC_COL, 1, 1)], max_rows=1)
    assert e.value.status == capi.E_INVALID_ARG
    assert "scratch" in e.value.message


def test_noalloc_grouped_matches_numpy(table):
    """The same grouped query against an independent NumPy group-by of the
    host columns (the C semantics: int32 products wrap, sums are int64)."""
    eng, ptrs, n = table
    cols = [eng.read("nf", c).astype(np.int64) for c in range(4)]
    keep = (cols[0] >= 5) & (cols[0] <= 45) & (cols[3] <= 700_000)
    k0, k1 = cols[2][keep], cols[0][keep]
    prod = ((cols[3][keep] * cols[1][keep]) & 0xFFFFFFFF).astype(np.uint32).astype(np.int32).astype(np.int64)
    uniq, inv = np.unique(np.stack([k0, k1], axis=1), axis=0, return_inverse=True)
    inv = inv.reshape(-1)
    want = np.zeros((len(uniq), 2), np.int64)
    np.add.at(want[:, 0], inv, prod)
    np.add.at(want[:, 1], inv, cols[1][keep])
    k, s = noalloc(eng, ptrs, n, [(0, 5, 45), (3, -2**31, 700_000)], [(2, 0, 6), (0, 0, 49)],
                   [(capi.METRIC_MUL, 3, 1), (capi.METRIC_COL, 1, 1)], max_rows=7 * 50)
    np.testing.assert_array_equal(k, uniq.astype(np.int32))
    np.testing.assert_array_equal(s, want)


def test_noalloc_error_paths(table):
    eng, ptrs, n = table
    # a key value outside [key_min, key_max] (column 2 holds 0..6): a device error
    with pytest.raises(capi.SvmError) as e:
        noalloc(eng, ptrs, n, [], [(2, 0, 5)], [(capi.METRIC_COL, 1, 1)], max_rows=64)
    assert e.value.status == capi.E_DEVICE and "key" in e.value.message
    # more groups than max_rows
    with pytest.raises(capi.SvmError) as e:
        noalloc(eng, ptrs, n, [], [(2, 0, 6)], [(capi.METRIC_COL, 1, 1)], max_rows=6)
    assert e.value.status == capi.E_INVALID_ARG and "max_rows" in e.value.message
    # a query without keys writes one row: max_rows 0 is refused before any launch
    with pytest.raises(capi.SvmError) as e:
        noalloc(eng, ptrs, n, [], [], [(capi.METRIC_COL, 1, 1)], max_rows=0)
    assert e.value.status == capi.E_INVALID_ARG
    # a column pointer that is not 16-byte aligned
    bad = list(ptrs)
    bad[1] = ptrs[1] + 4
    with pytest.raises(capi.SvmError) as e:
        noalloc(eng, bad, n - 1, [], [(2, 0, 6)], [(capi.METRIC_COL, 1, 1)], max_rows=64)
    assert e.value.status == capi.E_INVALID_ARG and "aligned" in e.value.message
    # the shared scratch keeps no error from the failed calls
    k, s = noalloc(eng, ptrs, n, [], [(2, 0, 6)], [(capi.METRIC_COL, 1, 1)], max_rows=64)
    c1, c2 = eng.read("nf", 1).astype(np.int64), eng.read("nf", 2)
    np.testing.assert_array_equal(k[:, 0], np.arange(7, dtype=np.int32))
    np.testing.assert_array_equal(s[:, 0], np.array([c1[c2 == v].sum() for v in range(7)], np.int64))
