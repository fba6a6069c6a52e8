"""Benchmark: AST nodes/s of the GB300 code generator, batched vs plain, bit-exact.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--mode batched|single]
                    [--programs P] [--config c1] [--impl gb300|reference]

Default (--mode batched): the batched workload, 4,096 seeded synthetic programs of
1k..500k nodes (lognormal, ~285M nodes, 4..512 functions each).  A step compiles all of
them through the batched pipeline (ptl_batch_compile: one launch per stage step for the
whole batch).  Prints one JSON line (rank 0):

  value       nodes/s with the trees resident in HBM: device time of the compile from the
              CUDA events the library records on its stream (after the input copy, before
              the output copy)
  e2e         the same call timed on the host: gathering the host trees into pinned
              memory, host->device, the pipeline, device->host of every program's words and
              function table
  plain       the plain pipeline (one program at a time, ptl_generator_*) on a sample of
              the same programs; batched_over_plain = value / plain value
  roofline    the dominant stage: algorithmic bytes / its event-timed duration, against
              the measured HBM copy bandwidth
  cpu_baseline  the oracle's CPU restatement on a bounded sample, on all host cores
  flatten     AST flattening (ptl_flatten) on 16 programs given in random node order,
              host arrays in and out, against the oracle's restatement on one core
  scalar      the scalar generator's semantics (the reference's -s, rv_generator_st) on
              the plain pipeline over a sample of the programs, checked against and timed
              beside the oracle's restatement of that generator on all host cores

--mode single times one large program (config c1, ~4M nodes) per step instead; --mode
scalar runs only the scalar generator's measurement.
--impl reference times the oracle restatement on the host cores on a sample of the same
workload (the reference itself is AVX2-only and cannot run on the aarch64 GPU hosts).
Multi-GPU: every rank compiles its own batch (programs are independent, no collective on
the data path); value aggregates nodes over ranks, timed to the slowest rank.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "AST nodes/s codegen, batched vs plain GPU (bit-exact); serving p50/p99 latency"
UNIT = "nodes/s"

# Algorithmic bytes per unit (node n, word w) of each stage: the minimum single-pass
# traffic of the reference's arrays.
STAGE_BYTES = {
    "preprocess": lambda n, w, w2, w3: 20 * n,
    "isn_cnt": lambda n, w, w2, w3: 14 * n,
    "isn_gen": lambda n, w, w2, w3: 22 * n + 16 * n + 20 * w,
    "optimize": lambda n, w, w2, w3: 16 * w + 8 * w,
    "regalloc": lambda n, w, w2, w3: 24 * w + 20 * w2,
    "fix_jumps": lambda n, w, w2, w3: 20 * w2 + 4 * w3,
}


# DRAM bytes each stage's kernels moved per node in one ncu capture of a batched compile
# of the workload's first 256 programs (profiles/stage_traffic_256_programs.md); a
# batch's traffic is estimated as this times its nodes.
STAGE_DRAM_BYTES_PER_NODE = {"preprocess": 67.2, "isn_cnt": 53.7, "isn_gen": 371.0, "optimize": 55.6,
                             "regalloc": 177.2, "fix_jumps": 26.3}


def stage_rooflines(stage_ms, tot, peak):
    """Per stage: algorithmic bytes over its event-timed time, as a fraction of the HBM
    peak; the scan, generation and compaction stages (isn_cnt, isn_gen, optimize) as a
    group; regalloc also as instruction steps per second (its step loop is a dependent
    chain per function, not a bandwidth-bound pass)."""
    from ptilopsis_gb300 import STAGES
    out, grp_b, grp_ms = {}, 0.0, 0.0
    for s, ms in zip(STAGES, stage_ms):
        if s not in STAGE_BYTES or ms <= 0:
            continue
        b = STAGE_BYTES[s](tot["n"], tot["W"], tot["W2"], tot["W3"])
        gbs = b / (ms / 1000.0) / 1e9
        traffic = STAGE_DRAM_BYTES_PER_NODE[s] * tot["n"]
        out[s] = {"ms": round(float(ms), 3), "algorithmic_bytes": int(b), "achieved_gbs": round(gbs, 1),
                  "frac": round(gbs / peak, 4), "traffic_bytes_est": int(traffic),
                  "traffic_over_algorithmic": round(traffic / b, 2)}
        if s in ("isn_cnt", "isn_gen", "optimize"):
            grp_b += b
            grp_ms += ms
    group = {"stages": ["isn_cnt", "isn_gen", "optimize"], "algorithmic_bytes": int(grp_b),
             "ms": round(grp_ms, 3), "frac": round(grp_b / (grp_ms / 1000.0) / 1e9 / peak, 4) if grp_ms else None}
    ra_ms = float(stage_ms[STAGES.index("regalloc")])
    ra = {"instruction_steps": int(tot["W"]), "steps_per_s": tot["W"] / (ra_ms / 1000.0) if ra_ms else None}
    return {"stages": out, "scan_gen_compaction": group, "regalloc_steps": ra}


def env_rank():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for name, val in zip(names, parts[5:9]):
                    if val.lower() == "active":
                        reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def l2_flush(buf):
    buf.fill_(1)  # 256 MB > the 129 MB L2


def cpu_baseline(tree, sample: str):
    from oracle import portbind
    from oracle.refbind import Ast
    ast = Ast(tree.type, tree.rtype, tree.parent, tree.depth, tree.child_idx, tree.data, tree.max_depth)
    t0 = time.perf_counter()
    res = portbind.compile_ast(ast)
    dt = time.perf_counter() - t0
    return {"value": tree.n / dt, "unit": UNIT, "cores": 1, "kind": "port", "sample": sample,
            "seconds": round(dt, 3), "words": int(len(res.words))}, res


def to_ast(tree):
    from oracle.refbind import Ast
    return Ast(tree.type, tree.rtype, tree.parent, tree.depth, tree.child_idx, tree.data, tree.max_depth)


def port_parallel(trees, threads):
    """Oracle restatement over trees on `threads` host threads (the library call releases
    the GIL); returns (nodes/s, seconds, outputs)."""
    from concurrent.futures import ThreadPoolExecutor
    from oracle import portbind
    asts = [to_ast(t) for t in trees]
    t0 = time.perf_counter()
    with ThreadPoolExecutor(threads) as ex:
        outs = list(ex.map(portbind.compile_ast, asts))
    dt = time.perf_counter() - t0
    return sum(t.n for t in trees) / dt, dt, outs


def reduce_max(x: float, dist=None, device=None) -> float:
    """The largest of the ranks' values (a step is as slow as its slowest rank); with no
    process group, x itself.  device: where the reduction tensor lives (a CUDA device for
    NCCL, None for gloo)."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def planned_nodes(k: int) -> float:
    """Program k's planned size (functions x mean function size), known before it is
    generated."""
    from ptilopsis_gb300.synth import config_params
    p = config_params("c3", program=k)
    return p.n_functions * p.median_fn_nodes * float(np.exp(p.sigma ** 2 / 2))


def rank_programs(programs: int, rank: int, world: int) -> list:
    """The program indices one rank compiles: the N x `programs` programs of the whole
    job, split over the N ranks by planned size (shard_programs), so that every rank has
    about `programs` programs and the same number of nodes (weak scaling: the work per
    GPU is fixed as N grows; programs are independent, so no rank exchanges data)."""
    from ptilopsis_gb300.batch import shard_programs
    if world == 1:
        return list(range(programs))
    sizes = [planned_nodes(k) for k in range(programs * world)]
    return shard_programs(sizes, world)[rank]


def make_workload(args, rank, world=1):
    from concurrent.futures import ThreadPoolExecutor
    from ptilopsis_gb300.synth import config_params, generate
    idx = rank_programs(args.programs, rank, world)
    with ThreadPoolExecutor(min(32, os.cpu_count() or 8)) as ex:
        return list(ex.map(lambda k: generate(config_params("c3", program=k)), idx))


def batched_config(trees, words):
    """The workload description both arms print (the GPU arm's tiles and parallelism are
    separate keys)."""
    nodes = sum(t.n for t in trees)
    return {"workload": f"c3: {len(trees)} synthetic programs per GPU (1k..500k nodes, lognormal), {nodes} nodes, "
                        f"{words} output words",
            "programs": len(trees), "nodes": nodes, "words": int(words)}


def compare_all(trees, words_of, table_of, outs):
    """Every program's words and function table against the oracle's outputs."""
    equal, first_bad = 0, None
    for k, o in enumerate(outs):
        tab = table_of(k)
        ok = np.array_equal(words_of(k), o.words) and all(
            np.array_equal(tab[a], o.bufs[b]) for a, b in (("starts", "fn_start"), ("ends", "fn_end"),
                                                            ("sizes", "fn_size"), ("ids", "fn_id")))
        equal += ok
        if not ok and first_bad is None:
            first_bad = k
    return {"programs": len(outs), "equal": int(equal), "first_mismatch": first_bad,
            "compared": "words and function table of every program"}


def run_reference(args):
    rank, world, _ = env_rank()
    if rank != 0:
        return
    from ptilopsis_gb300 import build as b
    from oracle import portbind
    b.build_synth()
    portbind.build()
    threads = os.cpu_count() or 1
    if args.mode == "single":
        from ptilopsis_gb300.synth import config_tree
        tree = config_tree(args.config, args.scale)
        trees = [tree]
        sample = f"one full compile of config {args.config} ({tree.n} nodes) per step, one thread"
        threads = 1
        workload = f"{args.config}: one synthetic program, {tree.n} nodes"
        config = {"workload": workload, "nodes_per_step": tree.n}
    else:
        trees = make_workload(args, 0)
        sample = (f"all {len(trees)} programs of the batched workload ({sum(t.n for t in trees)} nodes) per step, "
                  f"{threads} threads, one program per thread at a time")
        config = None
    words = 0
    for k in range(args.warmup):
        _, _, outs = port_parallel(trees, threads)
        if k == 0:
            words = sum(len(o.words) for o in outs)
        del outs
    times = []
    for _ in range(args.steps):
        _, dt, outs = port_parallel(trees, threads)
        times.append(dt)
        words = sum(len(o.words) for o in outs)
        del outs
    if config is None:
        config = batched_config(trees, words)
    ms = 1000.0 * sum(times) / len(times)
    value = sum(t.n for t in trees) / (ms / 1000.0)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded grammar)", "impl": "reference",
            "config": config,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_serving(device, args):
    """Open-loop Poisson arrivals of compile requests at each rate for a fixed window of
    arrivals (args.serve_seconds), drawn from a pool of distinct requests (80% 1k..10k
    nodes, 20% lognormal in 100k..2M; request k is pool[k % pool size]), each lent to the
    server (no copy at submit).  Latency = completion - scheduled arrival, on the server's
    clock.  Per rate: the completion rate inside the window and over the whole run, the
    queue depth sampled every 50 ms, and whether the offered load is above what the
    server completes (then the queue grows for the whole window and the latencies grow
    with it: they are reported, but they measure the window's length).  Requests still
    queued args.serve_drain seconds after the window are left unserved and counted."""
    import threading
    from concurrent.futures import ThreadPoolExecutor
    from ptilopsis_gb300 import RvGenerator
    from ptilopsis_gb300.batch import CompileServer, clock_ns
    from ptilopsis_gb300.synth import config_params, generate
    n_pool = args.serve_requests
    with ThreadPoolExecutor(min(32, os.cpu_count() or 8)) as ex:
        pool = list(ex.map(lambda k: generate(config_params("c4", program=k)), range(n_pool)))
    pool_nodes = np.array([t.n for t in pool], dtype=np.float64)
    rng = np.random.default_rng(0x50544C04)
    budget = 120 << 30
    out = {"slots": args.serve_slots, "memory_budget_gb": 120, "distinct_requests": n_pool,
           "request_nodes_mean": float(pool_nodes.mean()), "window_s": args.serve_seconds,
           "drain_limit_s": args.serve_drain, "rates": []}
    for rate in args.serve_rates:
        with CompileServer(device=device, slots=args.serve_slots, memory_budget=budget) as srv:
            for t in [srv.submit(r, copy=False) for r in pool[:8]]:  # warm-up: arenas and code paths
                srv.result(t)
                srv.release(t)
            sched = np.cumsum(rng.exponential(1.0 / rate, int(rate * args.serve_seconds * 1.5) + 16))
            sched = sched[sched < args.serve_seconds]
            m = len(sched)
            tickets = np.zeros(m, dtype=np.int64)
            submitted = threading.Event()
            n_sub = [0]
            done_ns = np.zeros(m, dtype=np.int64)
            depth = []
            stop = threading.Event()

            def sampler():
                while not stop.is_set():
                    st, mem = srv.stats(), srv.memory()
                    depth.append((clock_ns(), st["queued"], st["bytes_in_flight"], mem["held"]))
                    stop.wait(0.05)

            def reaper():
                k = 0
                while k < m:
                    if k >= n_sub[0]:
                        if submitted.is_set() and k >= n_sub[0]:
                            break
                        time.sleep(0.0005)
                        continue
                    tk = int(tickets[k])
                    if srv.poll(tk):
                        done_ns[k] = srv.times(tk)[2]
                        srv.release(tk)
                        k += 1
                    elif stop.is_set():
                        break
                    else:
                        time.sleep(0.0002)

            ts = threading.Thread(target=sampler, daemon=True)
            tr = threading.Thread(target=reaper, daemon=True)
            t0 = clock_ns() + 5_000_000
            ts.start()
            tr.start()
            for k in range(m):
                due = t0 + int(sched[k] * 1e9)
                while clock_ns() < due:
                    pass
                tickets[k] = srv.submit(pool[k % n_pool], copy=False)  # the pool outlives the server
                n_sub[0] = k + 1
            submit_end = clock_ns()
            submitted.set()
            tr.join(timeout=args.serve_drain)
            stop.set()
            tr.join()
            ts.join()
            end_ns = clock_ns()
        arrive = t0 + (sched * 1e9).astype(np.int64)
        fin = done_ns > 0
        lat = (done_ns[fin] - arrive[fin]) / 1e6
        win_end = t0 + int(args.serve_seconds * 1e9)
        in_win = fin & (done_ns <= win_end)
        nodes_k = pool_nodes[np.arange(m) % n_pool]
        offered = float(nodes_k.sum() / args.serve_seconds)
        done_rate_win = float(nodes_k[in_win].sum() / args.serve_seconds)
        q = np.array([d[1] for d in depth]) if depth else np.zeros(1)
        out["rates"].append({
            "rate_per_s": rate, "requests": int(m),
            "achieved_submit_rate_per_s": m / ((submit_end - t0) / 1e9),
            "completed_in_window": int(in_win.sum()), "completed": int(fin.sum()),
            "unserved_at_drain_limit": int(m - fin.sum()),
            "completion_rate_per_s": float(in_win.sum() / args.serve_seconds),
            "offered_nodes_per_s": offered, "completed_nodes_per_s_in_window": done_rate_win,
            "sustained_nodes_per_s": float(nodes_k[fin].sum() / max((end_ns - t0) / 1e9, 1e-9)),
            "above_capacity": bool(done_rate_win < 0.95 * offered),
            "p50_ms": float(np.percentile(lat, 50)) if len(lat) else None,
            "p99_ms": float(np.percentile(lat, 99)) if len(lat) else None,
            "max_ms": float(lat.max()) if len(lat) else None,
            "queue_depth": {"max": int(q.max()), "at_window_end": int(q[min(len(q) - 1, int(args.serve_seconds / 0.05))]),
                            "samples_every_ms": 50,
                            "series": [int(x) for x in q[::max(1, len(q) // 40)]]},
            "device_bytes_held_max": int(max((d[3] for d in depth), default=0)),
            "memory_budget_bytes": budget})
    # results in the mix equal compiling alone and the oracle: the first 64 requests
    # submitted together, so that they are batched with one another
    k_mix = min(64, n_pool)
    with CompileServer(device=device, slots=args.serve_slots, memory_budget=budget) as srv:
        tickets = [srv.submit(r) for r in pool[:k_mix]]
        mixed = [srv.result(t) for t in tickets]
        for t in tickets:
            srv.release(t)
    with RvGenerator(pool[0], device=device) as g:
        same = True
        for k in range(k_mix):
            g.upload(pool[k])
            g.process()
            same &= bool(np.array_equal(g.get_instructions(), mixed[k].words))
    out["bit_exact_vs_plain"] = same
    _, _, outs = port_parallel(pool[:k_mix], os.cpu_count() or 1)
    chk = compare_all(pool[:k_mix], lambda k: mixed[k].words, lambda k: mixed[k].table, outs)
    out["bit_exact_vs_oracle"] = chk["equal"] == chk["programs"]
    out["oracle_check"] = chk
    return out


def run_scalar(trees, device, sample_n):
    """The scalar generator (RvGenerator(scalar=True)) one program at a time on a sample
    of the workload: device time (stage events) and wall time, the words compared with
    the oracle's scalar restatement, which runs the same sample on all host cores."""
    from concurrent.futures import ThreadPoolExecutor
    from oracle import portbind
    from ptilopsis_gb300 import STAGES, RvGenerator
    sample = trees[:sample_n]
    sn = sum(t.n for t in sample)
    gen = RvGenerator(sample[0], device=device, scalar=True)
    gen.process()
    dev, words, stage = 0.0, [], np.zeros(len(STAGES))
    t0 = time.perf_counter()
    for t in sample:
        gen.upload(t)
        gen.process(profile=True)
        words.append(gen.get_instructions())
        ns = np.array(gen.stage_ns(), dtype=np.float64)
        stage += ns
        dev += ns.sum() / 1e9
    wall = time.perf_counter() - t0
    gen.close()
    threads = os.cpu_count() or 1
    asts = [to_ast(t) for t in sample]
    t0 = time.perf_counter()
    with ThreadPoolExecutor(threads) as ex:
        outs = list(ex.map(lambda a: portbind.compile_ast(a, scalar=True), asts))
    cdt = time.perf_counter() - t0
    equal = sum(bool(np.array_equal(w, o.words)) for w, o in zip(words, outs))
    out = {"value": sn / dev, "e2e_value": sn / wall, "unit": UNIT, "programs": len(sample), "nodes": sn,
           "sample": f"first {len(sample)} programs of the workload, one scalar generator, one at a time",
           "stage_ms": {k: round(float(v) / 1e6, 3) for k, v in zip(STAGES, stage)},
           "bit_exact_vs_oracle": equal == len(sample), "oracle_equal": equal,
           "cpu_baseline": {"value": sn / cdt, "unit": UNIT, "cores": threads, "kind": "port",
                            "sample": f"the same {len(sample)} programs, {threads} threads",
                            "seconds": round(cdt, 3)}}
    # the same semantics through the batched pipeline (BatchCompiler(scalar=True)) on the
    # first 512 programs, beside the oracle's scalar restatement on all host cores
    from ptilopsis_gb300.batch import BatchCompiler
    bsample = trees[:512]
    bn = sum(t.n for t in bsample)
    with BatchCompiler(device=device, workers=min(32, threads), scalar=True) as bc:
        bc.compile(bsample)
        dev_ns, walls = [], []
        for _ in range(3):
            t0 = time.perf_counter()
            bc.compile(bsample)
            walls.append(time.perf_counter() - t0)
            dev_ns.append(bc.device_ns())
        bwords = [bc.words(k).copy() for k in range(len(bsample))]
    basts = [to_ast(t) for t in bsample]
    t0 = time.perf_counter()
    with ThreadPoolExecutor(threads) as ex:
        bouts = list(ex.map(lambda a: portbind.compile_ast(a, scalar=True), basts))
    bcdt = time.perf_counter() - t0
    bequal = sum(bool(np.array_equal(w, o.words)) for w, o in zip(bwords, bouts))
    out["batched"] = {"value": bn / (float(np.median(dev_ns)) / 1e9), "e2e_value": bn / float(np.median(walls)),
                      "unit": UNIT, "programs": len(bsample), "nodes": bn,
                      "sample": f"first {len(bsample)} programs of the workload in one scalar batch (median of 3)",
                      "bit_exact_vs_oracle": bequal == len(bsample), "oracle_equal": bequal,
                      "cpu_baseline": {"value": bn / bcdt, "unit": UNIT, "cores": threads, "kind": "port",
                                       "sample": f"the same {len(bsample)} programs, {threads} threads",
                                       "seconds": round(bcdt, 3)}}
    return out


def run_single_program(device, config, steps=3, check=True):
    """One configuration's single program (c1: 4.3M nodes, 2,048 functions, a quarter of
    them spilling; c2: 64M nodes, 32,768 functions) through the plain pipeline: device
    time per compile (stage events, median of `steps`), the call with host arrays in and
    out, and the words against the oracle's restatement (one core, outside the timings)."""
    from ptilopsis_gb300 import STAGES, RvGenerator
    from ptilopsis_gb300.synth import config_tree
    tree = config_tree(config)
    n = tree.n
    with RvGenerator(tree, device=device) as gen:
        gen.process()
        dev, stage = [], []
        for _ in range(steps):
            gen.process(profile=True, to_host=False)
            ns = np.array(gen.stage_ns(), dtype=np.float64)
            dev.append(ns.sum() / 1e9)
            stage.append(ns)
        walls = []
        for _ in range(steps):
            t0 = time.perf_counter()
            gen.upload(tree)
            gen.process()
            words = gen.get_instructions()
            table = gen.function_table()
            walls.append(time.perf_counter() - t0)
    k = int(np.argsort(dev)[len(dev) // 2])
    out = {"value": n / dev[k], "e2e_value": n / float(np.median(walls)), "unit": UNIT, "nodes": n,
           "functions": int(len(table["starts"])), "words": int(len(words)),
           "sample": f"one program of {n} nodes (configuration {config}), median of {steps} compiles",
           "stage_ms": {s: round(float(v) / 1e6, 3) for s, v in zip(STAGES, stage[k])}}
    if check:
        from oracle import portbind
        t0 = time.perf_counter()
        ref = portbind.compile_ast(to_ast(tree))
        out["bit_exact_vs_oracle"] = bool(np.array_equal(words, ref.words)) and bool(
            np.array_equal(table["starts"], ref.bufs["fn_start"]))
        out["cpu_baseline"] = {"value": n / (time.perf_counter() - t0), "unit": UNIT, "cores": 1, "kind": "port",
                               "sample": "the same program, one thread"}
    return out


def run_flatten(trees, device, reps=3):
    """AST flattening (ptl_flatten, the GPU's DepthTree construction) on the 16 largest of
    the first 256 programs, each given in a seeded random node order, through the public
    call with host arrays in and out; checked against the original post-order trees, and
    the oracle's single-thread restatement timed on the same inputs."""
    from oracle import portbind
    from ptilopsis_gb300 import flatten
    pick = sorted(trees[:256], key=lambda t: -t.n)[:16]
    cases = []
    for k, t in enumerate(pick):
        rng = np.random.default_rng(0x50544F00 + k)
        perm = rng.permutation(t.n)
        par = np.where(t.parent >= 0, perm[np.maximum(t.parent, 0)], -1).astype(np.int32)
        arrs = []
        for x in (t.type, t.rtype, par, t.child_idx, t.data):
            y = np.empty_like(x)
            y[perm] = x
            arrs.append(y)
        cases.append(arrs)
    nodes = sum(t.n for t in pick)
    for arrs in cases[:2]:
        flatten(*arrs, device=device)  # warm-up
    best, exact = None, True
    for _ in range(reps):
        t0 = time.perf_counter()
        outs = [flatten(*arrs, device=device)[0] for arrs in cases]
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    for t, o in zip(pick, outs):
        exact &= all(np.array_equal(getattr(o, f), getattr(t, f))
                     for f in ("type", "rtype", "parent", "depth", "child_idx", "data")) and o.max_depth == t.max_depth
    t0 = time.perf_counter()
    for arrs in cases:
        portbind.flatten(*arrs)
    cpu = time.perf_counter() - t0
    return {"value": nodes / best, "unit": UNIT, "nodes": nodes,
            "sample": f"16 largest of the first 256 programs, nodes in seeded random order, host arrays in and out "
                      f"(best of {reps})",
            "bit_exact_vs_post_order": bool(exact),
            "cpu_baseline": {"value": nodes / cpu, "unit": UNIT, "cores": 1, "kind": "port",
                             "sample": "the same 16 inputs, the oracle's restatement of DepthTree::construct"}}


def run_batched(args):
    import torch
    rank, world, local = env_rank()
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    from ptilopsis_gb300 import RvGenerator, STAGES
    from ptilopsis_gb300 import build as b
    from ptilopsis_gb300.batch import BatchCompiler
    from ptilopsis_gb300.codegen import kernel_launches
    b.build_all()
    trees = make_workload(args, rank, world)
    nodes = sum(t.n for t in trees)
    dev = torch.device("cuda", local)

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def max_over_ranks(x):
        return reduce_max(x, dist, dev)

    # tile sizes by measurement, on other programs of the same distribution (untimed)
    tiles = tuple(args.tiles) if args.tiles else None
    if tiles is None and not args.no_autotune:
        from concurrent.futures import ThreadPoolExecutor
        from ptilopsis_gb300.batch import autotune
        from ptilopsis_gb300.synth import config_params, generate
        with ThreadPoolExecutor(min(32, os.cpu_count() or 8)) as ex:
            tune = list(ex.map(lambda k: generate(config_params("c3", program=1_000_000 + 512 * rank + k)),
                               range(min(512, args.programs))))
        tuned = autotune(tune, device=local, workers=min(32, os.cpu_count() or 8), save=False)
        tiles = (tuned["elem_tile"], tuned["sweep_tile"])
        del tune
    bc = BatchCompiler(device=local, workers=min(32, os.cpu_count() or 8), tiles=tiles)
    for _ in range(args.warmup):
        bc.compile(trees)
    barrier()
    dev_ms, wall_ms, sort_ms, stage_sum, host_parts = [], [], [], np.zeros(7), np.zeros(3)
    launches0 = kernel_launches()
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            t0 = time.perf_counter()
            bc.compile(trees)
            wall_ms.append(1000.0 * (time.perf_counter() - t0))
            ns = np.array(bc.stage_ns(), dtype=np.float64)
            stage_sum += ns
            hp = bc.host_ns()
            host_parts += np.array([hp["gather_ns"], hp["h2d_ns"], hp["d2h_ns"]], dtype=np.float64)
            dev_ms.append(bc.device_ns() / 1e6)
            sort_ms.append(bc.depth_sort_ns() / 1e6)
        barrier()
    launches = (kernel_launches() - launches0) // args.steps
    ms = max_over_ranks(float(np.mean(dev_ms)))
    e2e_ms = max_over_ranks(float(np.mean(wall_ms)))
    h2d, d2h = bc.copied_bytes()
    value = world * nodes / (ms / 1000.0)
    hp_ms = host_parts / 1e6 / args.steps
    e2e = {"value": world * nodes / (e2e_ms / 1000.0), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
           "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_ms,
           "parts_ms": {"gather_inputs": round(float(hp_ms[0]), 2), "h2d": round(float(hp_ms[1]), 2),
                        "pipeline": round(float(np.mean(dev_ms)), 2), "d2h": round(float(hp_ms[2]), 2)}}

    # per-program sizes for the algorithmic bytes
    tot = {"n": 0, "W": 0, "W2": 0, "W3": 0}
    for k in range(len(trees)):
        for key, v in bc.sizes(k).items():
            tot[key] += v
    stage_ms = stage_sum / 1e6 / args.steps
    dom = int(np.argmax(stage_ms[:6]))
    name = STAGES[dom]
    alg = STAGE_BYTES[name](tot["n"], tot["W"], tot["W2"], tot["W3"])
    achieved = alg / (stage_ms[dom] / 1000.0) / 1e9
    peak, peak_kind = peaks()
    traffic = STAGE_DRAM_BYTES_PER_NODE[name] * tot["n"]
    roofline = {"bound": "hbm", "kernel": f"{name} stage (all programs)", "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic,
                "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum of the stage's kernels on the "
                                   "first 256 programs, per node, times this batch's nodes") if traffic else None,
                "traffic_over_algorithmic": round(traffic / alg, 2) if traffic else None,
                "algorithmic_bytes_per_launch": int(alg),
                "stage_ms": {s: round(float(v), 3) for s, v in zip(STAGES, stage_ms)},
                "depth_sort_ms": round(float(np.mean(sort_ms)), 3),  # part of isn_gen
                **stage_rooflines(stage_ms, tot, peak)}
    # isn_gen's generation passes alone: its algorithmic bytes (inputs, registers, words;
    # the depth order moves none of them) over the stage's time less the depth sort's
    gen_ms = float(stage_ms[STAGES.index("isn_gen")]) - float(np.mean(sort_ms))
    if gen_ms > 0:
        gb = STAGE_BYTES["isn_gen"](tot["n"], tot["W"], tot["W2"], tot["W3"])
        roofline["isn_gen_generation_passes"] = {"ms": round(gen_ms, 3), "algorithmic_bytes": int(gb),
                                                 "achieved_gbs": round(gb / (gen_ms / 1000.0) / 1e9, 1),
                                                 "frac": round(gb / (gen_ms / 1000.0) / 1e9 / peak, 4)}

    # the plain pipeline on a sample of the same programs, one at a time
    sample = trees[:args.plain_sample]
    sn = sum(t.n for t in sample)
    gen = RvGenerator(sample[0], device=local)
    gen.process()
    plain_dev, plain_words = 0.0, []
    plain_stage = np.zeros(len(STAGES))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for t in sample:
        gen.upload(t)
        gen.process(profile=True)
        plain_words.append(gen.get_instructions())
        ns = np.array(gen.stage_ns(), dtype=np.float64)
        plain_stage += ns
        plain_dev += ns.sum() / 1e9
    plain_wall = time.perf_counter() - t0
    gen.close()
    plain = {"value": sn / plain_dev, "e2e_value": sn / plain_wall, "unit": UNIT, "programs": len(sample),
             "nodes": sn, "sample": f"first {len(sample)} programs of the workload, one generator, one at a time",
             "stage_ms": {k: round(float(v) / 1e6, 3) for k, v in zip(STAGES, plain_stage)}}
    # the same programs through 16 generators on 16 host threads at once (each its own
    # stream; host arrays in and out): what a caller compiling many programs through the
    # one-program API gets
    n_conc = 16
    gens = [RvGenerator(sample[0], device=local) for _ in range(min(n_conc, len(sample)))]
    conc_words = [None] * len(sample)

    def conc_worker(g, ks):
        for k in ks:
            g.upload(sample[k])
            g.process()
            conc_words[k] = g.get_instructions()

    import threading
    for g in gens:  # warmed like the one-at-a-time generator: its arenas grow as it goes
        g.process()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ths = [threading.Thread(target=conc_worker, args=(g, range(j, len(sample), len(gens)))) for j, g in enumerate(gens)]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    conc_wall = time.perf_counter() - t0
    for g in gens:
        g.close()
    plain["concurrent_generators"] = {
        "value": sn / conc_wall, "unit": UNIT, "generators": len(gens), "host_threads": len(gens),
        "sample": "the same programs, host arrays in and out, generator j taking programs j, j+16, ...",
        "bit_exact_vs_one_at_a_time": all(np.array_equal(conc_words[k], plain_words[k]) for k in range(len(sample)))}
    same_as_plain = all(np.array_equal(bc.words(k), plain_words[k]) for k in range(len(sample)))
    if rank == 0 and not args.no_cpu_baseline:
        # what one caller with one program at a time gets on the CPU: the oracle's
        # restatement on one core over the same sample, beside the plain pipeline
        rate1, dt1, _ = port_parallel(sample, 1)
        plain["cpu_one_program_at_a_time"] = {"value": rate1, "unit": UNIT, "cores": 1, "kind": "port",
                                              "seconds": round(dt1, 3),
                                              "plain_over_cpu": plain["value"] / rate1}
        # beside the concurrent generators: the oracle on every host core over the same programs
        cores = os.cpu_count() or 1
        rate_all, dt_all, _ = port_parallel(sample, cores)
        plain["concurrent_generators"]["cpu_all_cores"] = {
            "value": rate_all, "unit": UNIT, "cores": cores, "kind": "port", "seconds": round(dt_all, 3),
            "concurrent_over_cpu": plain["concurrent_generators"]["value"] / rate_all}
    oracle_check, cpu_line = None, None
    if rank == 0 and not args.no_cpu_baseline:
        # the oracle on every program of the batch, on all host cores (outside the timed
        # region); its time is the CPU baseline
        threads = os.cpu_count() or 1
        rate, dt, outs = port_parallel(trees, threads)
        oracle_check = compare_all(trees, bc.words, bc.function_table, outs)
        del outs
        cpu_line = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
                    "sample": f"all {len(trees)} programs of the workload ({nodes} nodes), {threads} threads",
                    "seconds": round(dt, 3)}

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded grammar, no datasets)",
            "config": {**batched_config(trees, tot["W3"]),
                       "l2": "inputs and working set (~60 GB) larger than L2; no flush between steps",
                       "parallelism": f"replicas x{world} (each GPU its own batch)"},
            "tiles": {"elem": bc.tiles()[0], "sweep": bc.tiles()[1],
                      "chosen_by": "defaults" if tiles is None else "--tiles" if args.tiles else
                      "autotune on 512 other programs of the same distribution"},
            "e2e": e2e, "plain": plain, "batched_over_plain": value / plain["value"],
            "roofline": roofline, "gpu_launches": int(launches)}
    bc.close()
    if rank == 0:
        line["clocks"] = clocks.summary()
        line["bit_exact_vs_plain"] = bool(same_as_plain)
        if not args.no_serving:
            line["serving"] = run_serving(local, args)
        if not args.no_flatten:
            line["flatten"] = run_flatten(trees, local)
        if not args.no_scalar:
            line["scalar"] = run_scalar(trees, local, args.scalar_sample)
        if not args.no_huge:
            line["large_program"] = run_single_program(local, "c1", check=not args.no_cpu_baseline)
            line["huge_program"] = run_single_program(local, "c2", check=not args.no_cpu_baseline)
        if oracle_check is not None:
            line["bit_exact_vs_oracle"] = oracle_check["equal"] == oracle_check["programs"]
            line["oracle_check"] = oracle_check
            line["cpu_baseline"] = cpu_line
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def run_gb300(args):
    import torch
    rank, world, local = env_rank()
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    from ptilopsis_gb300 import RvGenerator, STAGES
    from ptilopsis_gb300 import build as b
    from ptilopsis_gb300.codegen import kernel_launches
    from ptilopsis_gb300.synth import config_tree
    b.build_all()
    tree = config_tree(args.config, args.scale)
    n = tree.n
    dev = torch.device("cuda", local)
    dtree = tree.to(dev)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    gen = RvGenerator(dtree, device=local)
    for _ in range(args.warmup):
        gen.process(profile=True, to_host=False)
    barrier()
    stage_sum = np.zeros(7)
    step_ms = []
    launches0 = kernel_launches()
    t_wall0 = time.perf_counter()
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            l2_flush(flush)
            torch.cuda.synchronize()
            gen.process(profile=True, to_host=False)
            ns = np.array(gen.stage_ns(), dtype=np.float64)
            stage_sum += ns
            step_ms.append(ns.sum() / 1e6)
        barrier()
    wall_s = time.perf_counter() - t_wall0
    launches = kernel_launches() - launches0
    ms = float(np.mean(step_ms))
    ms_all = ms
    if dist is not None:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_all = float(t.item())
    value = world * n / (ms_all / 1000.0)
    words_dev, n_words = gen.device_instructions()
    W3 = n_words

    # ---- e2e: host buffers through the public API
    pinned = {k: torch.from_numpy(np.ascontiguousarray(getattr(tree, k).view(np.int32) if k == "data" else getattr(tree, k))).pin_memory()
              for k in ("type", "rtype", "parent", "depth", "child_idx", "data")}
    from ptilopsis_gb300 import DepthTree
    htree = DepthTree(max_depth=tree.max_depth, **pinned)
    ftab_entries = 0
    e2e_s = []
    for k in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        gen.upload(htree)
        gen.process(profile=False, to_host=True)
        words = gen.get_instructions()
        ftab = gen.function_table()
        dt = time.perf_counter() - t0
        if k >= args.warmup:
            e2e_s.append(dt)
        ftab_entries = len(ftab["starts"])
    e2e_ms = 1000.0 * float(np.mean(e2e_s))
    if dist is not None:
        t = torch.tensor([e2e_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = float(t.item())
    e2e = {"value": world * n / (e2e_ms / 1000.0), "unit": UNIT, "h2d_bytes_per_step": int(18 * n),
           "d2h_bytes_per_step": int(4 * len(words) + 16 * ftab_entries), "ms_per_step": e2e_ms}

    # ---- roofline of the dominant stage (event-timed on the library's stream)
    stage_ms = stage_sum / 1e6 / args.steps
    sizes = gen_sizes(gen)
    dom = int(np.argmax(stage_ms[:6]))
    name = STAGES[dom]
    alg = STAGE_BYTES[name](n, sizes["W"], sizes["W2"], W3)
    achieved = alg / (stage_ms[dom] / 1000.0) / 1e9
    peak, peak_kind = peaks()
    roofline = {"bound": "hbm", "kernel": f"{name} stage", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_kind, "traffic": None,
                "algorithmic_bytes_per_launch": int(alg),
                "stage_ms": {s: round(float(v), 4) for s, v in zip(STAGES, stage_ms)},
                **stage_rooflines(stage_ms, {"n": n, "W": sizes["W"], "W2": sizes["W2"], "W3": W3}, peak)}

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_all, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded grammar, no datasets)",
            "config": {"workload": f"{args.config}: one synthetic program per GPU, {n} nodes, "
                                   f"{sizes['F']} functions, {W3} output words",
                       "nodes": n, "functions": sizes["F"], "words": W3,
                       "l2": "flushed between steps (256 MB write); working set > L2",
                       "parallelism": f"replicas x{world}"},
            "e2e": e2e, "roofline": roofline, "gpu_launches": int(launches),
            "wall_s_timed": round(wall_s, 3)}
    if rank == 0:
        line["clocks"] = clocks.summary()
        if not args.no_cpu_baseline:
            base, ref = cpu_baseline(tree, f"one full compile of {args.config} ({n} nodes), one thread")
            line["cpu_baseline"] = base
            gen.process(profile=False, to_host=True)
            line["bit_exact_vs_oracle"] = bool(np.array_equal(gen.get_instructions(), ref.words))
        print(json.dumps(line), flush=True)
    gen.close()
    if dist is not None:
        dist.destroy_process_group()


def gen_sizes(gen):
    import ctypes
    from ptilopsis_gb300.codegen import SNAPSHOTS
    out = {}
    for key, snap in (("W", "gen_instr"), ("W2", "ra_instr"), ("F", "fn_start")):
        n = ctypes.c_size_t()
        gen._lib.ptl_generator_snapshot(gen._h, SNAPSHOTS[snap], None, 0, ctypes.byref(n))
        out[key] = int(n.value)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--config", default="c1")
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--mode", default="batched", choices=["batched", "single", "scalar"])
    ap.add_argument("--programs", type=int, default=4096)
    ap.add_argument("--plain-sample", type=int, default=64)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-flatten", action="store_true")
    ap.add_argument("--no-scalar", action="store_true")
    ap.add_argument("--no-huge", action="store_true", help="skip the single large and huge programs (c1, c2)")
    ap.add_argument("--scalar-sample", type=int, default=64)
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--tiles", type=int, nargs=2, metavar=("ELEM", "SWEEP"),
                    help="tile sizes of the batched pipeline instead of autotuning them")
    ap.add_argument("--serve-requests", type=int, default=1000, help="distinct serving requests (the pool)")
    ap.add_argument("--serve-seconds", type=float, default=5.0, help="arrival window per rate")
    ap.add_argument("--serve-drain", type=float, default=10.0, help="seconds after the window before the rest is dropped")
    ap.add_argument("--serve-slots", type=int, default=3, help="server lanes: slots // 2 for small requests, the rest large")
    ap.add_argument("--serve-rates", type=float, nargs="+", default=[1000.0, 10000.0, 50000.0])
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.mode == "batched":
        run_batched(args)
    elif args.mode == "scalar":
        # the scalar generator alone on the first --scalar-sample programs (the `scalar`
        # object of the batched line, printed by itself)
        import torch
        args.programs = args.scalar_sample
        trees = make_workload(args, 0)
        torch.cuda.init()
        print(json.dumps({"mode": "scalar", **run_scalar(trees, 0, len(trees))}), flush=True)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
