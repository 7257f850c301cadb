"""The served form: continuous batching of RunPipelineCMD requests over one
engine (service/service.cu:25-63 runs one synchronous RPC at a time, with no
batching and no admission control).

A `BatchLoop` owns two worker threads.  Requests from any thread are queued
with their arrival time.  The launcher takes everything that has arrived,
admits requests in arrival order while the context's resident bytes plus the
admitted requests' footprints (svm_pipeline_footprint: group slots, finalize
scratch, the largest result) stay within the HBM budget, and begins a fold:
svm_batch_begin plans the fold and enqueues its batched launch without
waiting for it.  The completer waits for each fold in order
(svm_batch_wait), copies its results out of the fold's staging and completes
the requests.  So while one fold runs on the GPU, the requests that arrived
meanwhile are already being admitted and planned into the next fold, which
the device starts as soon as the running one ends: work that arrives during
a fold overlaps it, and at most `inflight` folds are begun and not yet
complete.  A request over budget waits until memory frees up; one that can
never fit fails with the budget error.  If a fold fails, its requests run one
by one so that each gets its own result or error.  Small folds and serial
mode run one launch per request.

`poisson_run` drives a loop with a seeded Poisson arrival stream and reports
queries/s and latency percentiles (latency = completion time minus scheduled
arrival time, results copied back to the host).
"""
from __future__ import annotations

import collections
import concurrent.futures as cf
import queue
import threading
import time

import numpy as np

from . import capi
from .capi import SvmError

DEFAULT_BUDGET = 150 * 10**9


class Request:
    __slots__ = ("pipe", "prepared", "future", "t_arrival", "t_done", "key_num", "footprint", "fold")

    def __init__(self, pipe, prepared, key_num, t_arrival):
        self.pipe = pipe
        self.prepared = prepared
        self.future = cf.Future()
        self.t_arrival = t_arrival
        self.t_done = None
        self.key_num = key_num
        self.footprint = None
        self.fold = 0


class BatchLoop:
    """Continuous batching over `engine` (an Engine, or any object with its
    run / run_batch / footprint / bytes_in_use / result / drop methods).

    fetch=True: each request's future resolves to its (keys, sums) arrays,
    copied to the host; drop_results=True then frees the result object on the
    device (a benchmark of a long stream would otherwise keep every result)."""

    def __init__(self, engine, budget_bytes: int = DEFAULT_BUDGET, max_fold: int = 1024, min_fold: int = 3,
                 serial: bool = False, fetch: bool = False, drop_results: bool = False, inflight: int = 2):
        self.engine = engine
        self.budget = budget_bytes
        self.max_fold = max_fold
        self.min_fold = min_fold
        self.serial = serial
        self.fetch = fetch
        self.drop_results = drop_results
        self.inflight = max(1, inflight)
        self.folds = []                 # size of every fold run (statistics)
        # seconds spent per phase (statistics): launcher admit / slot wait /
        # begin, completer wait / release / finish
        self.phase_s = collections.Counter()
        self._pending = collections.deque()
        self._cv = threading.Condition()
        self._stop = False
        self._known = set()
        self._async = hasattr(engine, "batch_begin") and self.inflight > 1
        # folds begun and handed to the completer, in order; a slot is taken
        # before a fold is begun and given back once it is complete, so at
        # most `inflight` folds are begun and not complete
        self._begun = queue.Queue()
        self._slots = threading.Semaphore(self.inflight)
        self._thread = threading.Thread(target=self._run, name="svm-batch-loop", daemon=True)
        self._thread.start()
        self._completer = None
        if self._async:
            self._completer = threading.Thread(target=self._complete, name="svm-batch-complete", daemon=True)
            self._completer.start()

    # ---------------------------------------------------------------- API
    def register(self, *ids: str):
        """Objects the service may name as pre_pipeline_id without asking the engine."""
        self._known.update(ids)

    def known(self, oid: str) -> bool:
        if oid in self._known:
            return True
        try:
            self.engine.info(oid)
        except SvmError:
            return False
        self._known.add(oid)
        return True

    def submit(self, pipe, key_num: int | None = None, t_arrival: float | None = None) -> cf.Future:
        from .engine import Prepared, reduce_shape
        if key_num is None:
            key_num = reduce_shape(pipe)[0]
        req = Request(pipe, Prepared([pipe]), key_num, time.perf_counter() if t_arrival is None else t_arrival)
        req.future.request = req
        with self._cv:
            if self._stop:
                raise RuntimeError("BatchLoop is closed")
            self._pending.append(req)
            self._cv.notify()
        return req.future

    def close(self):
        with self._cv:
            self._stop = True
            self._cv.notify()
        self._thread.join()
        if self._completer is not None:
            self._begun.put(None)
            self._completer.join()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---------------------------------------------------------------- worker
    def _take(self):
        """Everything that has arrived, in arrival order (waits for the first)."""
        with self._cv:
            while not self._pending and not self._stop:
                self._cv.wait()
            if not self._pending:
                return None
            reqs = list(self._pending)
            self._pending.clear()
        return reqs

    def _admit(self, reqs):
        admitted, deferred = [], []
        try:
            base = self.engine.bytes_in_use()
        except Exception:
            base = 0
        used = base
        for r in reqs:
            if len(admitted) >= self.max_fold or deferred:
                deferred.append(r)
                continue
            if r.footprint is None:
                try:
                    r.footprint = self.engine.footprint(r.prepared)
                except Exception as e:  # unknown input, unsupported expression ...
                    self._finish(r, error=e)
                    continue
            if base + r.footprint > self.budget and not admitted:
                self._finish(r, error=SvmError(capi.E_OOM_BUDGET, f"request {r.pipe.id} needs {r.footprint} B "
                                                                  f"beyond {base} B resident; budget "
                                                                  f"{self.budget} B"))
                continue
            if used + r.footprint > self.budget:
                deferred.append(r)  # waits for memory to free up (keeps arrival order)
                continue
            used += r.footprint
            admitted.append(r)
        if deferred:
            with self._cv:
                self._pending.extendleft(reversed(deferred))
        return admitted

    def _finish(self, r: Request, error=None):
        self._finish_fold([r], [error])

    def _finish_fold(self, reqs, errors):
        """Completes requests; with fetch, the successful ones' results are read
        in one device pass."""
        results = {}
        ok = [r for r, e in zip(reqs, errors) if e is None]
        if self.fetch and ok:
            try:
                if hasattr(self.engine, "read_objects"):
                    cols = self.engine.read_objects([r.pipe.id for r in ok], [sink_types(r.pipe) for r in ok])
                    for r, c in zip(ok, cols):
                        results[r.pipe.id] = split_result(c, r.key_num)
                else:
                    for r in ok:
                        results[r.pipe.id] = self.engine.result(r.pipe.id, r.key_num)
                if self.drop_results:
                    for r in ok:
                        self.engine.drop(r.pipe.id)
            except Exception as e:
                errors = [e if x is None else x for x in errors]
        t = time.perf_counter()
        for r, e in zip(reqs, errors):
            r.t_done = t
            if e is not None:
                r.future.set_exception(e)
                continue
            r.future.set_result(results[r.pipe.id] if self.fetch else r.pipe.id)
            if not self.drop_results:
                self._known.add(r.pipe.id)

    def _run_one(self, r: Request):
        try:
            self.engine.run(r.prepared)
        except Exception as e:
            self._finish(r, error=e)
            return
        self._finish(r)

    def _run(self):
        from .engine import Prepared
        while True:
            reqs = self._take()
            if reqs is None:
                return
            t0 = time.perf_counter()
            fold = self._admit(reqs)
            self.phase_s["admit"] += time.perf_counter() - t0
            if not fold:
                continue
            self.folds.append(len(fold))
            for r in fold:
                r.fold = len(self.folds)
            if self.serial or (not self._async and len(fold) < self.min_fold):
                for r in fold:
                    self._run_one(r)
                continue
            batch = Prepared.__new__(Prepared)
            batch.keep = [r.prepared for r in fold]
            batch.n = len(fold)
            batch.arr = (capi.svm_pipeline * len(fold))(*[r.prepared.arr[0] for r in fold])
            if self._async:
                t2 = time.perf_counter()
                self._slots.acquire()  # waits while `inflight` folds are begun and not complete
                t3 = time.perf_counter()
                self.phase_s["slot_wait"] += t3 - t2
                try:
                    handle = self.engine.batch_begin(batch, host_results=self.fetch)
                except Exception:
                    self._slots.release()
                    for r in fold:  # isolate: every request gets its own result or error
                        self._run_one(r)
                    continue
                self.phase_s["begin"] += time.perf_counter() - t3
                self._begun.put((fold, handle))
                continue
            try:
                self.engine.run_batch(batch)
            except Exception:
                for r in fold:  # isolate: every request gets its own result or error
                    self._run_one(r)
                continue
            self._finish_fold(fold, [None] * len(fold))

    def _complete(self):
        """Completes begun folds in order: wait, results to the host, futures."""
        while True:
            item = self._begun.get()
            if item is None:
                return
            fold, handle = item
            try:
                t0 = time.perf_counter()
                handle.wait()
                t1 = time.perf_counter()
                results = handle.release([sink_types(r.pipe) for r in fold] if self.fetch else None)
                self.phase_s["wait"] += t1 - t0
                self.phase_s["release"] += time.perf_counter() - t1
            except Exception:
                try:
                    handle.release()
                except Exception:
                    pass
                self._slots.release()
                for r in fold:  # isolate: every request gets its own result or error
                    self._run_one(r)
                continue
            self._slots.release()
            if self.fetch:
                done = {r.pipe.id: split_result(c, r.key_num) for r, c in zip(fold, results)}
                if self.drop_results:
                    for r in fold:
                        try:
                            self.engine.drop(r.pipe.id)
                        except Exception:
                            pass
            t = time.perf_counter()
            for r in fold:
                r.t_done = t
                r.future.set_result(done[r.pipe.id] if self.fetch else r.pipe.id)
                if not self.drop_results:
                    self._known.add(r.pipe.id)
            self.phase_s["finish"] += time.perf_counter() - t


def sink_types(pipe) -> list[int]:
    """Column types of a pipeline's output (its Sink / last operator schema)."""
    return [int(c.type) for c in pipe.workflow[-1].output.column_list]


def split_result(cols, key_num: int):
    g = len(cols[0]) if cols else 0
    keys = np.stack(cols[:key_num], axis=1).astype(np.int32) if key_num else np.zeros((g, 0), np.int32)
    sums = np.stack([c.astype(np.int64) for c in cols[key_num:]], axis=1) if len(cols) > key_num else \
        np.zeros((g, 0), np.int64)
    return keys, sums


def poisson_run(loop: BatchLoop, make_pipe, rate: float, seconds: float, seed: int = 0, tick: float = 0.0005,
                check=None):
    """Submits a seeded Poisson stream of `rate` requests/s for `seconds`
    (make_pipe(i) -> (PipelineInfo, key_num) builds request i) and waits for
    all of them.  Returns throughput and latency statistics; with `check`
    (check(i, result) -> bool, on the fetched results) also how many
    results it accepted and rejected."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=int(rate * seconds * 1.2) + 16)
    arrivals = np.cumsum(gaps)
    arrivals = arrivals[arrivals < seconds]
    futures = []
    loop.phase_s.clear()
    submit_s = 0.0
    t0 = time.perf_counter()
    i = 0
    n = len(arrivals)
    while i < n:
        now = time.perf_counter() - t0
        while i < n and arrivals[i] <= now:
            ts = time.perf_counter()
            pipe, key_num = make_pipe(i)
            futures.append(loop.submit(pipe, key_num, t_arrival=t0 + arrivals[i]))
            submit_s += time.perf_counter() - ts
            i += 1
        if i < n:
            time.sleep(max(0.0, min(tick, arrivals[i] - (time.perf_counter() - t0))))
    errors = 0
    checked = mismatched = 0
    for i, f in enumerate(futures):
        try:
            res = f.result()
        except Exception:
            errors += 1
            continue
        if check is not None:
            checked += 1
            mismatched += 0 if check(i, res) else 1
    reqs = [f.request for f in futures]
    lat = np.array([(r.t_done - r.t_arrival) * 1e3 for r in reqs]) if reqs else np.zeros(1)
    t_end = max(r.t_done for r in reqs) if reqs else t0
    span = t_end - t0
    per_fold = collections.Counter(r.fold for r in reqs)
    return {"offered_qps": rate, "seconds": seconds, "requests": len(reqs), "errors": errors,
            "achieved_qps": len(reqs) / span if span > 0 else 0.0,
            "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                           "p999": float(np.percentile(lat, 99.9)), "max": float(lat.max())},
            "folds": len(per_fold), "mean_fold": float(np.mean(list(per_fold.values()))) if per_fold else 0.0,
            "host_s": dict(loop.phase_s, submit=submit_s),
            "checked": checked, "mismatched": mismatched}
