"""The served loop's host logic (continuous batching, HBM-footprint admission,
error isolation, Poisson driver) and the RPC handler, on a fake engine: no
GPU, no grpc needed."""
import threading
import time

import numpy as np
import pytest

from shadowvm_gb300 import capi, proto, serving
from shadowvm_gb300.capi import SvmError
from shadowvm_gb300.pipeline import fact_pipeline
from shadowvm_gb300.service import DataPlane
from shadowvm_gb300.workloads import int_schema


class FakeEngine:
    """Records folds; a pipeline's "result" is derived from its id."""

    def __init__(self, resident=0, footprints=None, fail_ids=(), delay=0.002):
        self.resident = resident
        self.footprints = footprints or {}
        self.fail_ids = set(fail_ids)
        self.delay = delay
        self.objects = {"lineorder", "date"}
        self.batches, self.singles = [], []
        self.lock = threading.Lock()
        self.max_concurrency = 0
        self._active = 0

    def _ids(self, prepared):
        return [prepared.arr[i].id.decode() for i in range(prepared.n)]

    def _exec(self, ids):
        with self.lock:
            self._active += 1
            self.max_concurrency = max(self.max_concurrency, self._active)
        time.sleep(self.delay)
        with self.lock:
            self._active -= 1
        for i in ids:
            if i in self.fail_ids:
                raise SvmError(capi.E_UNSUPPORTED, f"cannot run {i}")
        self.objects.update(ids)

    def run(self, prepared):
        ids = self._ids(prepared)
        self.singles.append(ids[0])
        self._exec(ids)

    def run_batch(self, prepared):
        ids = self._ids(prepared)
        self.batches.append(ids)
        self._exec(ids)

    def footprint(self, prepared):
        return self.footprints.get(self._ids(prepared)[0], 1000)

    def bytes_in_use(self):
        return self.resident

    def info(self, oid):
        if oid not in self.objects:
            raise SvmError(capi.E_NOT_FOUND, oid)
        return 2, 10

    def result(self, oid, key_num):
        if oid not in self.objects:
            raise SvmError(capi.E_NOT_FOUND, oid)
        v = sum(map(ord, oid))
        return np.array([[v % 7]], np.int32), np.array([[v]], np.int64)

    def drop(self, oid):
        self.objects.discard(oid)


def query(i):
    return fact_pipeline(f"q{i}", "lineorder", int_schema(2), ["date"], [("$(0.0)", "$(1.0)")], "$(1.1)",
                         "$(0.1)")


def test_concurrent_arrivals_fold_and_each_gets_its_own_result():
    eng = FakeEngine(delay=0.01)
    with serving.BatchLoop(eng, fetch=True) as loop:
        futs = {}

        def client(k):
            for j in range(20):
                i = k * 100 + j
                futs[i] = loop.submit(query(i), 1)
                time.sleep(0.001)

        ts = [threading.Thread(target=client, args=(k,)) for k in range(4)]
        for t in ts:
            t.start()
        for t in ts:
            t.join()
        for i, f in futs.items():
            keys, sums = f.result(timeout=10)
            assert sums[0, 0] == sum(map(ord, f"q{i}"))
    assert len(futs) == 80
    assert any(len(b) > 3 for b in eng.batches), eng.batches      # arrivals folded into launches
    assert sum(len(b) for b in eng.batches) + len(eng.singles) == 80
    assert eng.max_concurrency == 1                               # one fold on the device at a time


def test_admission_by_footprint():
    fp = {f"q{i}": 40 for i in range(10)}
    fp["q99"] = 500
    fp["q50"] = 40
    eng = FakeEngine(resident=100, footprints=fp, delay=0.02)
    with serving.BatchLoop(eng, budget_bytes=300, min_fold=1) as loop:
        first = loop.submit(query(50), 1)    # occupies the worker while the rest arrive
        time.sleep(0.005)
        futs = [loop.submit(query(i), 1) for i in range(10)]
        big = loop.submit(query(99), 1)
        first.result(timeout=10)
        for f in futs:
            f.result(timeout=10)
        with pytest.raises(SvmError) as e:
            big.result(timeout=10)
        assert e.value.status == capi.E_OOM_BUDGET
    # resident 100 + 5 x 40 = 300: no fold holds more than 5 of the 40-byte requests
    sizes = [len(b) for b in eng.batches] + [1] * len(eng.singles)
    assert max(sizes) <= 5
    assert sum(len(b) for b in eng.batches if all(x != "q50" for x in b)) + \
        sum(1 for s in eng.singles if s != "q50") == 10


def test_failing_request_is_isolated():
    eng = FakeEngine(fail_ids={"q3"}, delay=0.02)
    with serving.BatchLoop(eng) as loop:
        block = loop.submit(query(100), 1)
        time.sleep(0.005)
        futs = [loop.submit(query(i), 1) for i in range(8)]
        block.result(timeout=10)
        for i, f in enumerate(futs):
            if i == 3:
                with pytest.raises(SvmError):
                    f.result(timeout=10)
            else:
                assert f.result(timeout=10) == f"q{i}"


def test_serial_mode_runs_one_per_launch():
    eng = FakeEngine(delay=0.001)
    with serving.BatchLoop(eng, serial=True) as loop:
        futs = [loop.submit(query(i), 1) for i in range(12)]
        for f in futs:
            f.result(timeout=10)
    assert not eng.batches and len(eng.singles) == 12
    assert eng.singles == [f"q{i}" for i in range(12)]             # FIFO


def test_poisson_driver_reports_latency():
    eng = FakeEngine(delay=0.003)
    with serving.BatchLoop(eng, fetch=True, drop_results=True) as loop:
        r = serving.poisson_run(loop, lambda i: (query(i), 1), rate=400, seconds=0.5, seed=7)
    assert r["requests"] > 100 and r["errors"] == 0
    assert 0 < r["latency_ms"]["p50"] <= r["latency_ms"]["p99"] <= r["latency_ms"]["p999"]
    assert r["mean_fold"] >= 1 and r["achieved_qps"] > 0
    assert "q0" not in eng.objects                                 # results dropped after the fetch


def test_rpc_handler_semantics():
    eng = FakeEngine(fail_ids={"bad"})
    with serving.BatchLoop(eng) as loop:
        dp = DataPlane(loop)
        status, ret = dp.handle(query(1))
        assert status == "OK" and ret.success and ret.info == "ShadowVM exec: q1"
        missing = fact_pipeline("q2", "nope", int_schema(2), ["date"], [("$(0.0)", "$(1.0)")], "$(1.1)", "$(0.1)")
        status, ret = dp.handle(missing)
        assert status == "CANCELLED" and not ret.success
        bad = fact_pipeline("bad", "lineorder", int_schema(2), [], [], "", "$(0.1)")
        status, ret = dp.handle(bad)
        assert status == "OK" and not ret.success and "ShadowVM error" in ret.info


def test_wire_codec_round_trip():
    p = query(7)
    p.workflow[0].args["type"] = "object"
    back = proto.decode_pipeline(proto.encode_pipeline(p))
    assert back.id == p.id and back.pre_pipeline_id == p.pre_pipeline_id
    assert [o.type for o in back.workflow] == [o.type for o in p.workflow]
    assert [o.args for o in back.workflow] == [o.args for o in p.workflow]
    r = proto.decode_ret(proto.encode_ret(proto.Ret(True, "ShadowVM exec: q7")))
    assert r.success and r.info == "ShadowVM exec: q7"


def test_grpc_end_to_end():
    grpc = pytest.importorskip("grpc")
    from shadowvm_gb300.service import Client, make_server
    eng = FakeEngine()
    with serving.BatchLoop(eng) as loop:
        server, port = make_server(DataPlane(loop), "127.0.0.1:0", workers=4)
        server.start()
        try:
            client = Client(f"127.0.0.1:{port}")
            ret = client.run_pipeline_cmd(query(5), timeout=10)
            assert ret.success and ret.info == "ShadowVM exec: q5"
            missing = fact_pipeline("q6", "nope", int_schema(2), ["date"], [("$(0.0)", "$(1.0)")], "$(1.1)",
                                    "$(0.1)")
            with pytest.raises(grpc.RpcError) as e:
                client.run_pipeline_cmd(missing, timeout=10)
            assert e.value.code() == grpc.StatusCode.CANCELLED
            client.close()
        finally:
            server.stop(0)


class FakeFold:
    def __init__(self, eng, ids, host_results):
        self.eng, self.ids, self.host = eng, ids, host_results
        self.done = threading.Event()
        self.error = None

    def wait(self):
        self.done.wait(10)
        if self.error:
            raise self.error
        return [1] * len(self.ids)

    def release(self, types=None):
        with self.eng.lock:
            self.eng.outstanding -= 1
        if types is None:
            return None
        out = []
        for i in self.ids:
            v = sum(map(ord, i))
            out.append([np.array([v % 7], np.int32), np.array([v], np.int64)])
        return out


class FakeAsyncEngine(FakeEngine):
    """A device that runs begun folds one after another, `delay` each."""

    def __init__(self, **kw):
        super().__init__(**kw)
        import queue
        self.q = queue.Queue()
        self.outstanding = 0
        self.max_outstanding = 0
        self.log = []  # (event, fold index, time)
        threading.Thread(target=self._device, daemon=True).start()

    def _device(self):
        while True:
            k, f = self.q.get()
            time.sleep(self.delay)
            if any(i in self.fail_ids for i in f.ids):
                f.error = SvmError(capi.E_DEVICE, "fold failed")
            else:
                self.objects.update(f.ids)
            self.log.append(("done", k, time.perf_counter()))
            f.done.set()

    def batch_begin(self, prepared, host_results=False):
        ids = self._ids(prepared)
        with self.lock:
            self.outstanding += 1
            self.max_outstanding = max(self.max_outstanding, self.outstanding)
            k = len(self.batches)
            self.batches.append(ids)
        self.log.append(("begin", k, time.perf_counter()))
        f = FakeFold(self, ids, host_results)
        self.q.put((k, f))
        return f


def test_folds_in_flight_overlap_and_keep_results():
    """The next fold is begun while the previous one runs on the device; at
    most `inflight` folds are begun and not complete; every request gets its
    own result."""
    eng = FakeAsyncEngine(delay=0.02)
    with serving.BatchLoop(eng, fetch=True, inflight=2) as loop:
        futs = {}
        for i in range(300):
            futs[i] = loop.submit(query(i), 1)
            time.sleep(0.0003)
        for i, f in futs.items():
            keys, sums = f.result(timeout=20)
            assert sums[0, 0] == sum(map(ord, f"q{i}"))
    assert eng.max_outstanding <= 2
    begins = {k: t for e, k, t in eng.log if e == "begin"}
    dones = {k: t for e, k, t in eng.log if e == "done"}
    overlapped = sum(1 for k in dones if k + 1 in begins and begins[k + 1] < dones[k])
    assert overlapped >= 1, eng.log
    assert sum(len(b) for b in eng.batches) + len(eng.singles) == 300


def test_failed_fold_in_flight_isolates_its_requests():
    eng = FakeAsyncEngine(delay=0.01, fail_ids={"q7"})
    with serving.BatchLoop(eng, fetch=True, inflight=2, min_fold=1) as loop:
        futs = [loop.submit(query(i), 1) for i in range(12)]
        for i, f in enumerate(futs):
            if i == 7:
                with pytest.raises(SvmError):
                    f.result(timeout=10)
            else:
                assert f.result(timeout=10)[1][0, 0] == sum(map(ord, f"q{i}"))
    assert "q7" in eng.singles  # rerun alone after its fold failed
