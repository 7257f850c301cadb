"""svm_scan_aggregate_noalloc: the allocation-free variant of the fused scan.

It exists for callers that cannot allocate device memory on their query path
(a runtime that owns all device memory through its own pool, a thread that
must not take cudaMalloc's implicit device-wide synchronisation).  Its scratch
is a static device array shared by every call, so this checks, through the C
ABI, that two calls in a row each give exactly the rows svm_run_pipeline gives
for the equivalent Filter/ReduceBy pipeline (integer sums: bit-exact), and
that a query too large for the array is refused.  The test's own buffers are
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
