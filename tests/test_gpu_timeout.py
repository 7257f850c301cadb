"""A bounded device wait that runs out: the fused scan's copy warp is told to
issue no copies (svm_test_device_wait), so every consumer warp's wait for its
first tile gives up after the shortened poll limit.  The kernel must exit on
its own, the call must report SVM_E_TIMEOUT, and the context must then run
the same query to the same result.  Nothing here faults or hangs the GPU: the
waits are bounded by construction and the copy warp has nothing in flight."""
import time

import numpy as np
import pytest

from shadowvm_gb300 import SvmError, capi
from shadowvm_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("config", [0, 2])
def test_starved_wait_reports_timeout_and_context_recovers(engine_factory, config):
    w = W.make(config, fact_rows=300_000, tuple_per_bulk=100_000, n_part=20_000, n_cust=30_000, n_supp=2_000)
    eng = engine_factory(tuple_per_bulk=w.tuple_per_bulk, autotune=False)
    W.load_engine(eng, w)
    keys, sums = W.run_engine(eng, w)
    assert len(sums) > 0

    eng.test_device_wait(1 << 12, stall_copies=True)
    t0 = time.perf_counter()
    with pytest.raises(SvmError) as err:
        eng.run(w.query)
    assert err.value.status == capi.E_TIMEOUT, err.value
    assert time.perf_counter() - t0 < 30.0

    eng.test_device_wait(0, stall_copies=False)
    eng.run(w.query)
    k2, s2 = eng.result(w.query.id, w.key_num)
    np.testing.assert_array_equal(k2, keys)
    np.testing.assert_array_equal(s2, sums)
