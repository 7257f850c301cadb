#!/usr/bin/env python
"""Benchmark: the fused star query on one GB300 (or N, one rank per GPU).

Default workload (N=1): the 600 M-row four-dimension star schema, query
"date + customer + supplier join, GROUP BY (c_nation, s_nation, year)
SUM(revenue - supplycost)", fact columns resident in HBM.  A step is one
RunPipelineCMD of that fact pipeline (scan + probes + aggregate + result
materialisation); the dimension pipelines and their tables are built during
warm-up and stay cached, as in the served form.

  python bench.py [--gpus N --steps K --warmup W] [--impl reference] [--config 0|1|2|5]

Under torchrun each rank owns its own slice of one global fact table (rows
rank*R .. rank*R+R-1), so per-GPU work is fixed ("weak" scaling); ranks only
meet at the timing barriers.  The reference arm (--impl reference) times the
reference's generated CPU path (the oracle port: codegen.py text compiled with
g++ -O2, run bulk by bulk on every host core) on a bounded sample of the same
workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "fact rows/s"
UNIT = "rows/s"


def rank_info():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def measured_hbm_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def committed_traffic(config: int):
    """DRAM traffic of the workload's kernel from the committed ncu summaries: per
    fact row for the star kernel, per shared-scan byte for the batch kernel."""
    p = os.path.join(ROOT, "profiles", "star_kernel_traffic.json")
    try:
        d = json.load(open(p))
        # config 5 runs config 2's kernel over the same fact columns (String
        # dimensions only change the probe tables' payloads)
        return d[f"config{2 if config == 5 else config}"]
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi samples during the timed region (clocks and throttle reasons)."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names[1:], f[5:9]):
                if v.lower() in ("active", "1"):
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def gpu_numa_node(device: int):
    """The host NUMA node the GPU's PCI function reports (sysfs), or None."""
    try:
        import torch
        pr = torch.cuda.get_device_properties(device)
        bus = f"{pr.pci_domain_id:04x}:{pr.pci_bus_id:02x}:{pr.pci_device_id:02x}.0"
        with open(f"/sys/bus/pci/devices/{bus}/numa_node") as f:
            node = int(f.read().strip())
        return node if node >= 0 else None
    except Exception:
        return None


def node_cpus(node: int):
    """CPUs of a NUMA node (sysfs cpulist), or None."""
    try:
        text = open(f"/sys/devices/system/node/node{node}/cpulist").read().strip()
    except OSError:
        return None
    cpus = set()
    for part in text.split(","):
        if not part:
            continue
        a, _, b = part.partition("-")
        cpus.update(range(int(a), int(b or a) + 1))
    return cpus or None


def pages_node(addr: int, nbytes: int, samples: int = 16):
    """NUMA nodes of a few pages of a host buffer (move_pages with no target
    nodes only reports where each page is); {} where the call is missing."""
    import ctypes
    import platform
    nr = {"aarch64": 239, "x86_64": 279}.get(platform.machine())
    if nr is None or nbytes <= 0:
        return {}
    try:
        libc = ctypes.CDLL(None, use_errno=True)
        page = os.sysconf("SC_PAGE_SIZE")
        addrs = [addr + (nbytes - page) * i // max(1, samples - 1) // page * page for i in range(samples)]
        pages = (ctypes.c_void_p * samples)(*addrs)
        status = (ctypes.c_int * samples)()
        if libc.syscall(nr, 0, samples, pages, None, status, 0) != 0:
            return {}
        out = {}
        for v in status:
            out[v] = out.get(v, 0) + 1
        return out
    except Exception:
        return {}


def cpu_reference_run(cfg: int, sample_rows: int, steps: int, threads: int):
    """The reference's generated CPU path (oracle port) on `sample_rows` fact rows.
    Returns (rows/s per step list, hash build ms, description)."""
    import oracle
    from shadowvm_gb300 import workloads as W
    w = W.make(cfg, fact_rows=sample_rows)
    used = {0: [0, 1, 2, 3], 1: [0, 4, 5], 2: [0, 5, 6, 7, 8], 5: [0, 5, 6, 7, 8]}[cfg]
    fact = []
    from shadowvm_gb300 import datagen as dg
    # generate only the columns the query reads; the others stay zero
    for c, name in enumerate(w.fact_cols):
        if c in used:
            fact.append(dg.fact_column(name, 0, sample_rows, seed=w.seed, n_part=w.n_part, n_cust=w.n_cust,
                                       n_supp=w.n_supp, datekeys=w.dims["date"][0]))
        else:
            fact.append(np.zeros(sample_rows, np.int32))
    rates, opens, result = [], [], None
    for _ in range(steps):
        result, stats = oracle.run_workload(w, "port", threads=threads, fact=fact)
        rates.append(sample_rows / (stats.compute_ms / 1e3))
        opens.append(stats.open_ms)
    desc = (f"{sample_rows} fact rows (rows 0..{sample_rows - 1}) of config {cfg}, tuple_per_bulk "
            f"{w.tuple_per_bulk}, generated host loop compiled by g++ -O2 (key bytes hashed as signed char), "
            f"{threads} worker threads; pipeline compute time (transform + reduce), hash build excluded "
            f"({statistics.median(opens):.0f} ms)")
    return rates, statistics.median(opens), desc, result


def default_cpu_sample(cfg: int, threads: int) -> int:
    """One reference bulk per host thread (the reference runs one task per bulk,
    core/pipeline.cu:161-212), at most 32 bulks."""
    tpb = 3_000_000 if cfg in (2, 5) else 2_000_000
    return tpb * max(4, min(threads, 32))


def reference_arm(args):
    rank, world, _ = rank_info()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    sample = args.cpu_sample_rows or default_cpu_sample(args.config, threads)
    _ = cpu_reference_run(args.config, min(sample, 3_000_000), 1, threads)  # compile + warm caches
    for _ in range(max(0, args.warmup - 1)):
        cpu_reference_run(args.config, sample, 1, threads)
    t0 = time.time()
    rates, _, desc, _ = cpu_reference_run(args.config, sample, args.steps, threads)
    wall = time.time() - t0
    v = statistics.median(rates)
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": sample / v * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
           "data": "synthetic (seeded counter-based generator, star-schema shapes)",
           "config": workload_config(args.config, sample),
           "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": desc},
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "wall_s": wall}
    print(json.dumps(out))


def workload_config(cfg: int, rows: int):
    names = {0: "date join, SUM(extprice*discount)", 1: "date+part join, GROUP BY (year, brand) SUM(revenue)",
             2: "4-dimension star schema: date+customer+supplier join, GROUP BY (c_nation, s_nation, year) "
                "SUM(revenue-supplycost)",
             5: "config 2 with String geography columns: StrCmp region filters, GROUP BY the c_nation / "
                "s_nation strings (Hash keys) and year"}
    return {"workload": f"config {cfg}: {names[cfg]}", "fact_rows": rows,
            "fact_columns_read": {0: 4, 1: 3, 2: 5, 5: 5}[cfg], "int32_columns": True,
            "l2": "inputs larger than L2 (no flush needed)" if rows * 4 > 129e6 else "flush not applied"}


def batched_measure(eng, bw, steps: int, warmup: int):
    """The config-3 query mix two ways on one engine: one svm_run_pipeline per
    query (one launch each) and one svm_run_batch for all of them.  Both are
    timed on the host around the API calls (each call returns once its
    results are materialised on the device); per-query latency assumes every
    query of the mix arrives at t=0.  Results are compared bit for bit."""
    from shadowvm_gb300 import capi
    from shadowvm_gb300.engine import Prepared
    # Both forms take pipelines already marshalled into C structs (a server
    # decodes each request once).
    singles = [Prepared([q.pipe]) for q in bw.queries]
    pipes = Prepared([q.pipe for q in bw.queries])
    nq = len(singles)
    for p in singles:
        eng.run(p)
    serial_res = {q.pipe.id: eng.result(q.pipe.id, q.key_num) for q in bw.queries}
    eng.profile(True)
    eng.profile_reset()
    serial_walls, lat = [], []
    for _ in range(max(1, min(steps, 3))):
        t0 = time.perf_counter()
        for p in singles:
            eng.run(p)
            lat.append((time.perf_counter() - t0) * 1e3)
        serial_walls.append(time.perf_counter() - t0)
    n_star, star_ms = eng.profile_read(capi.K_STAR)
    for _ in range(warmup):
        eng.run_batch(pipes)
    exact = all(np.array_equal(a, b) for q in bw.queries
                for a, b in zip(eng.result(q.pipe.id, q.key_num), serial_res[q.pipe.id]))
    eng.profile_reset()
    batch_walls = []
    for _ in range(steps):
        t0 = time.perf_counter()
        eng.run_batch(pipes)
        batch_walls.append(time.perf_counter() - t0)
    n_b, b_ms = eng.profile_read(capi.K_BATCH)
    eng.profile(False)
    batch_launch = eng.last_launch()
    serial_s, batch_s = statistics.median(serial_walls), statistics.median(batch_walls)
    lat = np.array(lat)
    bl = np.array(batch_walls) * 1e3
    return {"metric": "queries/s", "unit": "queries/s", "queries_per_batch": nq,
            "value": nq / batch_s, "one_query_per_launch": nq / serial_s, "speedup": serial_s / batch_s,
            "batched_ms": batch_s * 1e3, "serial_ms": serial_s * 1e3,
            "latency_ms": {"batched": {"p50": float(np.percentile(bl, 50)), "p99": float(np.percentile(bl, 99))},
                           "one_query_per_launch": {"p50": float(np.percentile(lat, 50)),
                                                    "p99": float(np.percentile(lat, 99))}},
            "device_ms": {"batch_kernel": b_ms / max(n_b, 1), "serial_star_kernels": star_ms / max(1, n_star) * nq},
            "query_rows_total": int(sum(q.nrows for q in bw.queries)),
            "shapes": {str(k): sum(q.shape == k for q in bw.queries) for k in range(3)},
            "bit_exact_vs_one_query_per_launch": bool(exact), "launch": batch_launch}


def ours_arm(args):
    import torch
    from shadowvm_gb300 import Engine, capi
    from shadowvm_gb300 import workloads as W

    rank, world, local = rank_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    if args.config == 3:
        return batched_arm(args)
    w = W.make(args.config, fact_rows=args.rows)
    rows = w.fact_rows
    eng = Engine(device=local, tuple_per_bulk=w.tuple_per_bulk, join_mode=args.join_mode)
    if args.pin:
        pins = [int(v) for v in args.pin.split(",")]
        r, mb, st, sg = pins[:4]
        eng.pin_launch(r, st, sg, blocks_per_sm=mb)
        if len(pins) > 4:
            eng.pin_list_after(pins[4])
    W.load_engine(eng, w, row0=rank * rows)
    t_build0 = time.time()
    for p in w.dim_pipelines:
        eng.run(p)
    eng.run(w.query)  # builds and caches the dimension tables
    build_s = time.time() - t_build0
    stream = torch.cuda.ExternalStream(eng.stream)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    for _ in range(args.warmup):
        eng.run(w.query)
    clocks = ClockSampler(local)
    clocks.start()
    eng.profile(True)
    eng.profile_reset()
    barrier()
    l0 = eng.kernel_launches()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        eng.run(w.query)
    e1.record(stream)
    barrier()
    launches = eng.kernel_launches() - l0
    ms = e0.elapsed_time(e1)
    n_star, star_ms = eng.profile_read(capi.K_STAR)
    eng.profile(False)
    clk = clocks.stop()
    launch_cfg = eng.last_launch()
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    ms_step = ms / args.steps
    value = rows * world / (ms_step / 1e3)

    # roofline of the star kernel (algorithmic bytes / event-timed launch duration)
    bpr = w.fact_bytes_per_row()
    star_avg_s = (star_ms / max(n_star, 1)) / 1e3
    achieved = rows * bpr / star_avg_s / 1e9
    peak, peak_src = measured_hbm_peak()
    tr = committed_traffic(args.config)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": (tr["dram_bytes_per_row"] * rows) if tr else None,
                "algorithmic_bytes_per_launch": rows * bpr, "kernel_ms": star_avg_s * 1e3,
                "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)" if peak_src == "measured"
                else "fallback 6800 GB/s", "traffic_source": tr.get("source") if tr else None}

    # e2e: the same query through the C ABI with the fact columns coming from
    # pinned host memory every step and the result read back to the host.
    e2e = None
    if not args.no_e2e:
        used = {0: [0, 1, 2, 3], 1: [0, 4, 5], 2: [0, 5, 6, 7, 8], 5: [0, 5, 6, 7, 8]}[args.config]
        # The page-locked columns are placed on the host NUMA node local to
        # the GPU: the allocating thread runs on that node's CPUs while the
        # pages are allocated, pinned and first written (host-side placement
        # only; no GPU setting changes).
        node = gpu_numa_node(local)
        cpus = node_cpus(node) if node is not None else None
        saved = os.sched_getaffinity(0)
        if cpus:
            os.sched_setaffinity(0, cpus & set(range(os.cpu_count() or 1)) or saved)
        pinned = {}
        for c in used:
            t = torch.empty(rows, dtype=torch.int32, pin_memory=True)
            a = t.numpy()
            a[:] = eng.read("lineorder", c)
            pinned[c] = (t, a)
        os.sched_setaffinity(0, saved)
        placed = pages_node(pinned[used[0]][1].ctypes.data, pinned[used[0]][1].nbytes)
        import copy
        qp = copy.deepcopy(w.query)
        qp.pre_pipeline_id[0] = "lineorder_e2e"
        cols = [pinned[c][1] if c in pinned else None for c in range(len(w.fact_cols))]

        def max_over_ranks(v):
            if world > 1:
                import torch.distributed as dist
                t = torch.tensor([v], device="cuda")
                dist.all_reduce(t, op=dist.ReduceOp.MAX)
                v = float(t.item())
            return v

        # (1) every column uploaded each step (svm_object_put), then the query
        eng.put("lineorder_e2e", cols)
        eng.run(qp)
        barrier()
        times = []
        for _ in range(max(1, min(args.steps, 10))):
            t0 = time.perf_counter()
            eng.put("lineorder_e2e", cols)
            eng.run(qp)
            keys, sums = eng.result(qp.id, w.key_num)
            times.append(time.perf_counter() - t0)
        copy_s = max_over_ranks(statistics.median(times))
        copy_h2d = sum(4 * rows for _ in used)
        eng.drop("lineorder_e2e")
        # (2) the headline: the columns left in page-locked host memory and read
        # in place (svm_object_put_host, as the reference keeps its fact bulks in
        # mapped pinned memory): the scan copies the columns its filters read
        # and gathers the others from host memory at the surviving rows
        qh = copy.deepcopy(w.query)
        qh.pre_pipeline_id[0] = "lineorder_e2h"
        eng.put_host("lineorder_e2h", cols)
        eng.run(qh)
        barrier()
        times = []
        for _ in range(max(1, min(args.steps, 10))):
            t0 = time.perf_counter()
            eng.put_host("lineorder_e2h", cols)
            eng.run(qh)
            keys, sums = eng.result(qh.id, w.key_num)
            times.append(time.perf_counter() - t0)
        hl = eng.last_launch()
        e2e_s = max_over_ranks(statistics.median(times))
        staged, late = int(hl.get("staged_columns", len(used))), int(hl.get("late_columns", 0))
        h2d = 4 * rows * staged
        d2h = keys.nbytes + sums.nbytes
        e2e = {"value": rows * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_s * 1e3,
               "h2d_gb_per_s": h2d / e2e_s / 1e9,
               "h2d_note": f"{staged} columns the filters read copied per step ({h2d} B); {late} metric "
                           "column(s) read from host memory only at the surviving rows (4 B per row, fetched "
                           "in 32 B sectors; not counted)",
               "host_numa": {"gpu_node": node, "pinned_pages_on_node": {str(k): v for k, v in placed.items()}},
               "api": "svm_object_put_host (page-locked host columns, read in place) + svm_run_pipeline + "
                      "svm_object_read",
               "copy_all": {"value": rows * world / copy_s, "unit": UNIT, "ms_per_step": copy_s * 1e3,
                            "h2d_bytes_per_step": copy_h2d, "h2d_gb_per_s": copy_h2d / copy_s / 1e9,
                            "api": "svm_object_put (every column uploaded) + svm_run_pipeline + "
                                   "svm_object_read"}}
        eng.drop(qh.id)
        eng.drop("lineorder_e2h")

    cpu, parity = None, None
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        sample = min(rows, args.cpu_sample_rows or default_cpu_sample(args.config, threads))
        rates, _, desc, (pk, ps) = cpu_reference_run(args.config, sample, 3, threads)
        cpu = {"value": statistics.median(rates), "unit": UNIT, "cores": threads, "kind": "port",
               "sample": desc}
        # Parity at full dimension sizes: the same query on the GPU over a view
        # of the same fact rows the port just ran, compared bit for bit.
        import copy
        qp = copy.deepcopy(w.query)
        qp.id = w.query.id + "_parity"
        qp.pre_pipeline_id[0] = "lineorder_parity"
        eng.view("lineorder_parity", "lineorder", 0, sample)
        eng.run(qp)
        gk, gs = eng.result(qp.id, w.key_num)
        parity = {"rows": sample, "groups": int(len(gs)), "equal": bool(np.array_equal(gk, pk) and
                                                                         np.array_equal(gs, ps)),
                  "against": "oracle port (the reference's generated CPU path) on the same fact rows, "
                             "full-size dimensions, REF_COMPAT; int64 sums and key rows compared bit for bit"}
        eng.drop(qp.id)
        eng.drop("lineorder_parity")

    batched = None
    if args.config == 2 and not args.no_batched:
        # The config-3 query mix over the same resident fact table.
        bw = W.make_batch(256, fact_rows=rows, tuple_per_bulk=w.tuple_per_bulk)
        eng.put("part", bw.fact.dims["part"])
        for i, q in enumerate(bw.queries):
            eng.view(f"lo_q{i}", "lineorder", q.row0, q.nrows)
        for p in bw.dim_pipelines:
            eng.run(p)
        batched = batched_measure(eng, bw, max(3, min(args.steps, 10)), 3)

    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "int32",
               "data": "synthetic (seeded counter-based generator on the device, star-schema shapes)",
               "config": dict(workload_config(args.config, rows * world), join_mode=args.join_mode,
                              rows_per_gpu=rows, parallelism=f"row shards x{world}"),
               "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
               "launch": launch_cfg,
               "clocks": clk, "dimension_build_s": build_s,
               "hbm_frac_of_measured": roofline["frac"], "parity": parity, "batched": batched}
        print(json.dumps(out))
    eng.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def batched_arm(args):
    """--config 3: the 256-query mix over views of the resident 600 M-row
    table, batched (one launch) against one launch per query."""
    import torch
    from shadowvm_gb300 import Engine
    from shadowvm_gb300 import workloads as W
    rank, world, local = rank_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    bw = W.make_batch(256, fact_rows=args.rows)
    rows = bw.fact.fact_rows
    eng = Engine(device=local, tuple_per_bulk=bw.fact.tuple_per_bulk, join_mode=args.join_mode)
    if args.pin_batch:
        cw, st = (int(v) for v in args.pin_batch.split(","))
        eng.pin_batch_launch(cw, st)
    W.load_engine(eng, bw.fact, row0=rank * rows)
    for i, q in enumerate(bw.queries):
        eng.view(f"lo_q{i}", "lineorder", q.row0, q.nrows)
    for p in bw.dim_pipelines:
        eng.run(p)
    clocks = ClockSampler(local)
    clocks.start()
    l0 = eng.kernel_launches()
    m = batched_measure(eng, bw, args.steps, args.warmup)
    launches = eng.kernel_launches() - l0
    clk = clocks.stop()
    v = m["value"]
    # roofline of the batch kernel: the shared scan reads the union of the
    # queries' fact columns over the union of their row ranges once
    used = {0: {0, 1, 2, 3}, 1: {0, 4, 5}, 2: {0, 5, 6, 7, 8}}
    ucols = set().union(*[used[q.shape] for q in bw.queries])
    spans = sorted((q.row0, q.row0 + q.nrows) for q in bw.queries)
    urows, cur_lo, cur_hi = 0, None, None
    for lo, hi in spans:
        if cur_hi is None or lo > cur_hi:
            urows += 0 if cur_hi is None else cur_hi - cur_lo
            cur_lo, cur_hi = lo, hi
        else:
            cur_hi = max(cur_hi, hi)
    urows += 0 if cur_hi is None else cur_hi - cur_lo
    scan_bytes = 4 * len(ucols) * urows
    k_s = m["device_ms"]["batch_kernel"] / 1e3
    peak, peak_src = measured_hbm_peak()
    tr = committed_traffic(3)
    roofline = {"bound": "hbm", "achieved": scan_bytes / k_s / 1e9, "peak": peak, "unit": "GB/s",
                "frac": scan_bytes / k_s / 1e9 / peak,
                "traffic": tr["dram_bytes_per_scan_byte"] * scan_bytes if tr else None,
                "traffic_source": tr.get("source") if tr else None, "kernel": "mbatch_kernel",
                "kernel_ms": k_s * 1e3, "algorithmic_bytes_per_launch": scan_bytes,
                "unshared_bytes": int(sum(4 * len(used[q.shape]) * q.nrows for q in bw.queries)),
                "peak_source": peak_src,
                "note": "shared-scan bytes (union columns x union rows x 4 B); the kernel is bound by per-query "
                        "instruction work on the staged tiles, not by DRAM"}
    # e2e: the batch and every query's result copied to the host (one bulk read)
    from shadowvm_gb300.engine import Prepared
    pipes = Prepared([q.pipe for q in bw.queries])
    ids = [q.pipe.id for q in bw.queries]
    rtypes = [[2] * q.key_num + [3] for q in bw.queries]
    e2e_t, d2h = [], 0
    for _ in range(max(3, min(args.steps, 10))):
        t0 = time.perf_counter()
        eng.run_batch(pipes)
        res = eng.read_objects(ids, rtypes)
        e2e_t.append(time.perf_counter() - t0)
        d2h = sum(a.nbytes for r in res for a in r)
    e2e_s = statistics.median(e2e_t)
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([m["batched_ms"]], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        v = 256 * world / (float(t.item()) / 1e3)
    if rank == 0:
        out = {"metric": "queries/s", "value": v, "unit": "queries/s", "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": m["batched_ms"], "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "int32",
               "data": "synthetic (seeded counter-based generator on the device, star-schema shapes)",
               "config": {"workload": "config 3: 256 seeded queries shaped like configs 0-2 over views of the "
                                      "resident 600 M-row star-schema fact table (log-uniform ranges 1M..600M, "
                                      "selectivity 1e-4..0.5), one svm_run_batch per step",
                          "fact_rows": rows, "join_mode": args.join_mode,
                          "l2": "inputs larger than L2 (no flush needed)"},
               "batched": m, "gpu_launches": launches, "clocks": clk, "roofline": roofline,
               "e2e": {"value": 256 / e2e_s, "unit": "queries/s", "h2d_bytes_per_step": 0,
                       "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_s * 1e3,
                       "note": "svm_run_batch + svm_objects_read of all 256 results, host-timed; the fact "
                               "table is resident (queries are requests over it)"}}
        print(json.dumps(out))
    eng.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def served_arm(args):
    """--config 4: a seeded Poisson stream of requests drawn from the config-3
    mix (each request a fresh pipeline id) into the served loop, batched and
    serial (one query per launch, FIFO), at each offered rate.  Latency is
    completion (result copied to the host) minus scheduled arrival."""
    import dataclasses

    import torch
    from shadowvm_gb300 import Engine, capi, serving
    from shadowvm_gb300 import workloads as W
    rank, world, local = rank_info()
    if rank != 0:
        return
    torch.cuda.set_device(local)
    bw = W.make_batch(256, fact_rows=args.rows)
    eng = Engine(device=local, tuple_per_bulk=bw.fact.tuple_per_bulk, join_mode=args.join_mode)
    W.load_engine(eng, bw.fact)
    for i, q in enumerate(bw.queries):
        eng.view(f"lo_q{i}", "lineorder", q.row0, q.nrows)
    for p in bw.dim_pipelines:
        eng.run(p)
    for _ in range(args.warmup):  # dimension tables, merged tables, device pool
        eng.run_batch([q.pipe for q in bw.queries])
    alone = {}
    for q in bw.queries:
        eng.run(q.pipe)
        alone[q.pipe.id] = eng.result(q.pipe.id, q.key_num)
    pick = np.random.default_rng(4321).integers(0, len(bw.queries), size=10_000_000)

    def check(i, res):  # every served result against its query run alone
        want = alone[bw.queries[pick[i]].pipe.id]
        return bool(np.array_equal(res[0], want[0]) and np.array_equal(res[1], want[1]))

    def make_pipe(i):
        q = bw.queries[pick[i]]
        return dataclasses.replace(q.pipe, id=f"s{i}"), q.key_num

    rates = [float(r) for r in args.rates.split(",")]
    clocks = ClockSampler(local)
    clocks.start()
    points = {"batched": [], "serial": []}
    for rate in rates:
        for mode in ("batched", "serial"):
            eng.profile(True)
            eng.profile_reset()
            with serving.BatchLoop(eng, budget_bytes=150 * 10**9, serial=(mode == "serial"), fetch=True,
                                   drop_results=True, max_fold=args.max_fold, inflight=args.inflight) as loop:
                r = serving.poisson_run(loop, make_pipe, rate, args.serve_seconds, seed=int(rate), check=check)
            r["device_s"] = {name: eng.profile_read(k)[1] / 1e3 for name, k in
                             (("batch", capi.K_BATCH), ("star", capi.K_STAR), ("finalize", capi.K_FINALIZE))}
            eng.profile(False)
            points[mode].append(r)
    clk = clocks.stop()

    def sustained(pts):
        ok = [p for p in pts if p["achieved_qps"] >= 0.95 * p["offered_qps"]]
        return max(ok, key=lambda p: p["achieved_qps"]) if ok else None

    top_b, top_s = points["batched"][-1], points["serial"][-1]
    sb, ss = sustained(points["batched"]), sustained(points["serial"])
    out = {"metric": "queries/s", "value": top_b["achieved_qps"], "unit": "queries/s", "n_gpus": 1,
           "steps": len(rates), "warmup": args.warmup, "ms_per_step": args.serve_seconds * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
           "data": "synthetic (seeded counter-based generator on the device, star-schema shapes)",
           "config": {"workload": "config 4: seeded Poisson arrivals of queries drawn from the config-3 mix "
                                  "over the resident 600 M-row table, continuous batching with HBM-footprint "
                                  "admission (150 GB budget)",
                      "fact_rows": bw.fact.fact_rows, "rates_qps": rates, "seconds_per_point": args.serve_seconds,
                      "join_mode": args.join_mode},
           "served": {"batched": points["batched"], "serial": points["serial"],
                      "top_rate": {"batched_qps": top_b["achieved_qps"], "serial_qps": top_s["achieved_qps"],
                                   "speedup": top_b["achieved_qps"] / max(top_s["achieved_qps"], 1e-9),
                                   "batched_p99_ms": top_b["latency_ms"]["p99"],
                                   "serial_p99_ms": top_s["latency_ms"]["p99"]},
                      "max_sustained_qps": {"batched": sb["achieved_qps"] if sb else None,
                                            "serial": ss["achieved_qps"] if ss else None},
                      "results_checked": sum(p["checked"] for m in points.values() for p in m),
                      "results_equal_to_alone": all(p["mismatched"] == 0 for m in points.values() for p in m)},
           "clocks": clk,
           "e2e": {"value": top_b["achieved_qps"], "unit": "queries/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": None, "note": "every request's result is copied to the host"}}
    print(json.dumps(out))
    eng.close()


def loader_arm(args):
    """--loader: the text Loader (svm_object_load_text) on SSB-like lines of
    9 space-padded int32 fields ("   1234567|" x 9 + "\n", 100 B per row),
    text resident on the device (value) and uploaded from pinned host memory
    every step (e2e); CPU baseline: the Loader restatement (oracle/loader.c,
    the reference's byte loop, one core) on a sample."""
    import torch
    import oracle
    from shadowvm_gb300 import Engine, capi
    from shadowvm_gb300.workloads import ssb_like_text
    rows = args.rows or 10_000_000
    text, _ = ssb_like_text(rows, 9, 7)
    nbytes = len(text)
    eng = Engine()
    dev = torch.frombuffer(bytearray(text), dtype=torch.uint8).cuda()
    host = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    host.numpy()[:] = np.frombuffer(text, np.uint8)
    types = [2] * 9
    for _ in range(args.warmup):
        eng.load_text("t", None, types, device_ptr=dev.data_ptr(), nbytes=nbytes)
    eng.profile(True)
    eng.profile_reset()
    launches0 = eng.kernel_launches()
    times = []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        eng.load_text("t", None, types, device_ptr=dev.data_ptr(), nbytes=nbytes)
        times.append(time.perf_counter() - t0)
    launches = eng.kernel_launches() - launches0
    n_parse, parse_ms = eng.profile_read(capi.K_LOAD)
    n_index, index_ms = eng.profile_read(capi.K_OTHER)
    eng.profile(False)
    dev_s = statistics.median(times)
    parse_s = parse_ms / max(n_parse, 1) / 1e3
    e2e = []
    for _ in range(max(3, args.steps // 2)):
        t0 = time.perf_counter()
        eng.load_text("t", host.numpy(), types)
        e2e.append(time.perf_counter() - t0)
    e2e_s = statistics.median(e2e)
    sample = text[: min(nbytes, 100 * 2_000_000)]
    t0 = time.perf_counter()
    oracle.load_text(sample, types)
    cpu_s = time.perf_counter() - t0
    peak, src = measured_hbm_peak()
    algo = nbytes + rows * 9 * 4  # the parse kernel reads the text and writes the columns
    # ncu, 200 MB case (profiles/load_parse_kernel_text.md): 203.0 MB read + 49.0 MB written per launch,
    # scaled by the text bytes
    traffic = (202.97e6 + 49.0e6) * nbytes / 200e6
    out = {"metric": "text bytes/s", "value": nbytes / dev_s, "unit": "B/s", "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": dev_s * 1e3, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "u8",
           "data": "synthetic SSB-like text: 9 space-padded int32 fields per line, '|' after each, '\\n' per line",
           "config": {"workload": f"text Loader, {rows} rows x 9 fields, {nbytes} bytes",
                      "l2": "inputs larger than L2 (no flush needed)"},
           "roofline": {"bound": "hbm", "achieved": algo / parse_s / 1e9, "peak": peak, "unit": "GB/s",
                        "frac": algo / parse_s / 1e9 / peak, "traffic": traffic, "kernel": "load_parse_kernel",
                        "kernel_ms": parse_s * 1e3, "index_ms": index_ms / max(n_index, 1),
                        "algorithmic_bytes_per_launch": algo, "peak_source": src,
                        "note": "parse kernel CUDA-event time; value is host-timed around the whole call "
                                "(index pass, row-count read, column allocation, parse, error read)"},
           "gpu_launches": launches,
           "e2e": {"value": nbytes / e2e_s, "unit": "B/s", "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": 8,
                   "ms_per_step": e2e_s * 1e3},
           "cpu_baseline": {"value": len(sample) / cpu_s, "unit": "B/s", "cores": 1, "kind": "port",
                            "sample": f"first {len(sample)} bytes through oracle/loader.c (the Loader byte loop)"}}
    print(json.dumps(out))
    eng.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", type=int, default=2, choices=[0, 1, 2, 3, 4, 5])
    ap.add_argument("--rows", type=int, default=None, help="fact rows per GPU (default: the config's)")
    ap.add_argument("--cpu-sample-rows", type=int, default=None)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the config-3 batched measurement")
    ap.add_argument("--rates", default="100,1000,2500,5000", help="config 4: offered queries/s")
    ap.add_argument("--serve-seconds", type=float, default=5.0, help="config 4: seconds of arrivals per point")
    ap.add_argument("--max-fold", type=int, default=1024, help="config 4: most requests in one fold")
    ap.add_argument("--inflight", type=int, default=2, help="config 4: folds begun and not complete, at most")
    ap.add_argument("--loader", action="store_true", help="measure the text Loader instead")
    ap.add_argument("--pin-batch", default=None,
                    help="consumer_warps,ring_stages: pin the merged batch kernel's launch configuration "
                         "(svm_pin_batch_launch), e.g. for a profile of the tuned variant")
    ap.add_argument("--pin", default=None,
                    help="rows_per_lane,blocks_per_sm,ring_stages,tables_staged[,list_after]: pin the scan's "
                         "launch configuration (svm_pin_launch, svm_pin_list_after), e.g. for a profile of "
                         "one variant")
    ap.add_argument("--join-mode", default="ref_compat", choices=["ref_compat", "exact"])
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.loader:
        loader_arm(args)
    elif args.impl == "reference":
        reference_arm(args)
    elif args.config == 4:
        served_arm(args)
    else:
        ours_arm(args)


if __name__ == "__main__":
    main()
