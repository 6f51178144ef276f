#!/usr/bin/env python
"""Benchmark: candidate literals scored per second on one GB300.

Workload (default ``batched_step``): one refinement step of 256 candidate
literals over a 32M x 6 binding set (10% positive) and 32 relations of arity
1-3 (log-uniform 1K-8M tuples, Zipf s=1.1 keys over a 2M domain); seeded
synthetic data.  ``--workload single_literal`` runs the 16M x 4 binding set /
4M-tuple relation single-literal operator bench instead.

A step = one batched evaluation of all the step's literals (exact counts).
The partition bits are first chosen by the engine's autotuner.  ``value`` is
literals/s with the binding set resident in HBM, the step replayed from its
captured CUDA graph (``direct`` gives the same step through the plain API
call, with per-stage CUDA-event times); ``e2e`` is the same metric through the
C ABI from pinned host buffers (binding-set upload and count download inside
the timed region); the plain per-literal GPU path is timed beside it
(``per_literal``).  ``serving`` runs the serving loop on 64 requests of
concurrent rule searches (binding sets log-uniform over 10K-20M rows), first
as a burst and then with Poisson arrivals at about 80% load, with p50/p99
latency.  Inputs (768 MB of binding columns) are larger than the 129 MB L2,
so no flush is needed between steps.

``--impl reference`` times the CPU restatement of the reference's operator
chain (the oracle; the reference itself cannot be built on the GPU host) on
all host cores over the whole step (all literals), for at most 3 steps.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import tempfile
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


# Repeats of the wall-clock end-to-end legs (the median is reported).
E2E_REPEATS = 3

# The headline metric, one string for both arms (the lines are compared).
HEADLINE_METRIC = "literals scored/s batched vs per-literal on 1 GB300, exact counts; p99 ms"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", choices=["batched_step", "single_literal", "single_literal_zipf"],
                    default="batched_step")
    ap.add_argument("--scale", type=float, default=1.0,
                    help="fraction of the binding-set size (for quick checks only)")
    ap.add_argument("--cpu-sample", type=int, default=0,
                    help="literals in the CPU-baseline sample (0 = automatic)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-per-literal", action="store_true")
    ap.add_argument("--eval-bits", type=int, default=0,
                    help="binding partition bits of the batched engine (0 = autotuned)")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving-loop leg")
    ap.add_argument("--no-coverage", action="store_true",
                    help="skip the coverage, test-runner and loader legs")
    ap.add_argument("--no-operators", action="store_true",
                    help="skip the leg timing the reference's operators kept at the C ABI")
    ap.add_argument("--no-learn", action="store_true",
                    help="skip the full-scale learn-loop (config 4) leg")
    return ap.parse_args()


def make_workload(args, rank: int):
    from quickfoil_gb300 import workloads
    if args.workload == "batched_step":
        return workloads.batched_step(n_bindings=int(32_000_000 * args.scale), seed=3 + rank)
    return workloads.single_literal(n_bindings=int(16_000_000 * args.scale),
                                    zipf=args.workload.endswith("zipf"), seed=2 + rank)


def workload_config(args, w):
    cfg = {"workload": w.name, "binding_rows": w.num_bindings,
           "binding_columns": len(w.binding_columns), "positive_rows": w.num_positive,
           "relations": len(w.relations), "relation_tuples": w.relation_tuples(),
           "literals": len(w.literals), "key_domain": w.domain,
           "l2_policy": "inputs larger than L2 (binding columns %d MB > 129 MB)"
                        % (w.num_bindings * len(w.binding_columns) * 4 // 2**20)}
    if args.scale != 1.0:
        cfg["scale"] = args.scale
    return cfg


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            # The samples go to a temporary file; the JSON line carries their
            # summary.  QF_CLOCKS_DIR keeps the raw samples elsewhere.
            out_dir = os.environ.get("QF_CLOCKS_DIR") or tempfile.gettempdir()
            os.makedirs(out_dir, exist_ok=True)
            self.path = os.path.join(out_dir, f"clocks_{os.getpid()}.csv")
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.fh,
                stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, flags in rows for i, f in enumerate(flags)
                          if f.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows),
                "sm_max_mhz": max(r[1] for r in rows), "reasons": reasons,
                "samples": len(rows)}


def profiled_traffic(args):
    """DRAM bytes (read + write) per launch of the evaluation kernel on the
    default workload, from the committed ncu summary; None for other
    workloads or when the summary is absent."""
    if args.workload != "batched_step" or args.scale != 1.0:
        return None
    path = os.path.join(ROOT, "profiles", "eval_batched_kernel_batched_step.md")
    try:
        for line in open(path):
            if line.startswith("dram_bytes_per_launch:"):
                return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


def host_cpu():
    """The host CPU's model name and logical core count (lscpu)."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            k, _, v = line.partition(":")
            if k.strip() == "Model name" and model is None:
                model = v.strip()
    except Exception:
        pass
    return {"model": model, "logical_cores": os.cpu_count()}


def measured_peak_hbm():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def join_group_sample(w):
    """The literals of the step that join on one binding column (the
    smallest such group): one Evaluate call's worth, so the sample pays one
    binding-set partition for its literals, about the full step's ratio (a
    partition per join column, 6 for 256 literals)."""
    groups = {}
    for l in w.literals:
        groups.setdefault(l.vars[l.join_pos], []).append(l.as_tuple())
    col, lits = min(groups.items(), key=lambda kv: len(kv[1]))
    return col, lits


def cpu_baseline(w, nthreads: int, sample: int):
    """The oracle (CPU restatement of the reference chain) on a bounded
    sample of the step: by default every literal of one join column
    (join_group_sample), else the first `sample` literals; returns
    (literals/s, seconds, literals, description)."""
    import oracle
    o = oracle.Oracle(w.relations)
    if sample > 0:
        lits = [l.as_tuple() for l in w.literals][:sample]
        what = f"first {len(lits)} of {len(w.literals)} literals of the step"
    else:
        col, lits = join_group_sample(w)
        what = (f"the {len(lits)} literals of the step that join on binding column {col} "
                f"(one Evaluate call: one binding partition for them)")
    o.evaluate(w.binding_columns, w.num_positive, lits[:1], 5, nthreads)  # warm relation cache
    t0 = time.perf_counter()
    o.evaluate(w.binding_columns, w.num_positive, lits, 5, nthreads)
    dt = time.perf_counter() - t0
    o.close()
    return len(lits) / dt, dt, len(lits), what


def run_reference(args):
    """The reference arm: the oracle port of the reference's operator chain
    (the reference itself cannot be built on the GPU host) over the whole
    step -- all of its literals, every binding partition -- on all host
    threads.  A step takes seconds, so at most 3 timed steps after 1 warm-up
    step are run (the JSON line gives the numbers run)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    w = make_workload(args, 0)
    threads = os.cpu_count() or 1
    import oracle
    o = oracle.Oracle(w.relations)
    lits = [l.as_tuple() for l in w.literals]
    if args.cpu_sample > 0:
        lits = lits[:args.cpu_sample]
    warmup, steps = min(args.warmup, 1), max(1, min(args.steps, 3))
    for _ in range(warmup):
        o.evaluate(w.binding_columns, w.num_positive, lits, 5, threads)
    t0 = time.perf_counter()
    for _ in range(steps):
        o.evaluate(w.binding_columns, w.num_positive, lits, 5, threads)
    dt = (time.perf_counter() - t0) / steps
    o.close()
    value = len(lits) / dt
    line = {"impl": "reference", "metric": HEADLINE_METRIC,
            "value": value, "unit": "literals/s", "n_gpus": args.gpus, "steps": steps,
            "warmup": warmup, "steps_requested": args.steps, "warmup_requested": args.warmup,
            "ms_per_step": dt * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32/int64",
            "data": "synthetic (seeded)", "config": workload_config(args, w),
            "cpu_baseline": {"value": value, "unit": "literals/s", "cores": threads,
                             "kind": "port", "host": host_cpu(),
                             "sample": f"the whole step: all {len(lits)} of {len(w.literals)} "
                                       "literals (every binding partition), oracle (C "
                                       "restatement of the reference operator chain), "
                                       f"{threads} threads"},
            "e2e": {"value": value, "unit": "literals/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_gb300(args):
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl")
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)

    def barrier():
        if dist is not None:
            dist.barrier()

    from quickfoil_gb300 import Engine
    from quickfoil_gb300 import _capi as C
    w = make_workload(args, rank)
    eng = Engine(local_rank)
    if args.eval_bits:
        eng.set_option(C.QFG_OPT_EVAL_BITS, args.eval_bits)
    stream = torch.cuda.current_stream(dev)
    eng.set_stream(stream.cuda_stream)
    for rid, cols in enumerate(w.relations):
        eng.register_relation(rid, cols)
    dev_cols = [torch.from_numpy(c).to(dev) for c in w.binding_columns]
    b = eng.bindings(dev_cols, w.num_positive)
    n = len(w.literals)
    lits_c = (C.QfgLiteral * n)(*[l.to_c() for l in w.literals])
    counts = torch.zeros((n, 4), dtype=torch.int64, device=dev)

    # First touch: relation key tables (cached for the run, like the
    # reference's relation partitions).
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    eng.evaluate_step_device(b, lits_c, n, counts.data_ptr())
    torch.cuda.synchronize()
    first_touch_ms = (time.perf_counter() - t0) * 1e3
    traffic = eng.step_traffic(b, w.literals)
    tune = None
    if not args.eval_bits:
        bits, cbits, tms = eng.autotune_step(b, w.literals)
        eng.set_option(C.QFG_OPT_AUTOTUNE, 1)
        tune = dict(eng.autotune_choice(w.num_bindings), ms_per_step=tms)

    for _ in range(args.warmup):
        eng.evaluate_step_device(b, lits_c, n, counts.data_ptr())
    torch.cuda.synchronize()
    eng.set_option(C.QFG_OPT_STAGE_TIMING, 1)
    eng.stage_times(reset=True)
    launches0 = eng.kernel_launches()
    clocks = ClockSampler(local_rank)
    clocks.start()
    barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        eng.evaluate_step_device(b, lits_c, n, counts.data_ptr())
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    launches = eng.kernel_launches() - launches0
    stages = eng.stage_times(reset=True)
    eng.set_option(C.QFG_OPT_STAGE_TIMING, 0)
    ms = ev0.elapsed_time(ev1) / args.steps
    if dist is not None:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    batched_counts = counts.cpu().numpy().copy()

    # The same step replayed from its captured CUDA graph (one launch a step).
    eng.set_option(C.QFG_OPT_USE_GRAPHS, 1)
    for _ in range(args.warmup):
        eng.evaluate_step_device(b, lits_c, n, counts.data_ptr())
    torch.cuda.synchronize()
    glaunch0 = eng.kernel_launches()
    barrier()
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(args.steps):
        eng.evaluate_step_device(b, lits_c, n, counts.data_ptr())
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier()
    glaunches = eng.kernel_launches() - glaunch0
    gms = ev0.elapsed_time(ev1) / args.steps
    if dist is not None:
        t = torch.tensor([gms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        gms = float(t.item())
    graph_equal = bool(np.array_equal(counts.cpu().numpy(), batched_counts))
    eng.set_option(C.QFG_OPT_USE_GRAPHS, 0)

    # Plain per-literal GPU path (one operator chain per literal).
    per_lit = None
    if not args.no_per_literal:
        host_counts = np.zeros((n, 4), dtype=np.int64)
        eng.evaluate_per_literal(b, w.literals)  # warm relation partitions
        eng.set_option(C.QFG_OPT_STAGE_TIMING, 1)
        eng.stage_times(reset=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        host_counts = eng.evaluate_per_literal(b, w.literals)
        pl_s = time.perf_counter() - t0
        pl_stage = eng.stage_times(reset=True)
        eng.set_option(C.QFG_OPT_STAGE_TIMING, 0)
        per_lit = {"value": n / pl_s, "unit": "literals/s", "ms_per_step": pl_s * 1e3,
                   "join_count_kernel_ms": pl_stage["per_literal"][0],
                   "counts_equal_batched": bool(np.array_equal(host_counts, batched_counts))}

    # The API-kept RadixPartition (qfg_radix_partition, the reference layout)
    # on one binding column at 15 radix bits, against 12 bytes a row.
    radix = operators = None
    if args.workload == "batched_step" and rank == 0:
        radix = run_radix_partition(eng, dev_cols[0], stream, torch, measured_peak_hbm()[0])
        if not args.no_operators:
            operators = run_operators(eng, w, b, dev_cols, stream, torch, measured_peak_hbm()[0],
                                      batched_counts)

    # End to end through the C ABI from pinned host buffers.
    pinned = [torch.from_numpy(c).pin_memory() for c in w.binding_columns]
    h2d = sum(c.numel() * 4 for c in pinned)
    d2h = n * 4 * 8
    for _ in range(max(1, min(args.warmup, 2))):
        be = eng.bindings(pinned, w.num_positive)
        eng.evaluate_step(be, w.literals)
        be.close()
    torch.cuda.synchronize()
    barrier()
    # Wall-clock legs on a shared host: each is timed E2E_REPEATS times over
    # the same K steps and the median is reported, with every repeat.
    e2e_counts = None
    e2e_runs = []
    for _ in range(E2E_REPEATS):
        t0 = time.perf_counter()
        for _ in range(args.steps):
            be = eng.bindings(pinned, w.num_positive)
            e2e_counts = eng.evaluate_step(be, w.literals)
            be.close()
        e2e_runs.append((time.perf_counter() - t0) / args.steps)
    e2e_s = statistics.median(e2e_runs)
    if dist is not None:
        t = torch.tensor([e2e_s], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())

    # End to end, pipelined through the serving API: step i+1's binding set
    # uploads on the context stream while step i evaluates on a server slot.
    # One slot: the steps take the GPU one after another while the uploads
    # overlap them; with two slots consecutive steps evaluate concurrently
    # and contend for SMs and L2 (10.80 against 10.61 ms a step on the
    # batched step).  Depth 2: the next step is queued on the slot's stream
    # behind the running one, so no host turnaround separates them.  The
    # server is created once, as a serving process would: its slot's scratch
    # (about 12 GB here) is allocated by the warm-up's first request, not
    # inside the timed steps.
    srv = eng.server(slots=1, depth=2)

    def pipelined(steps):
        prev, got = None, None
        for _ in range(steps):
            be = eng.bindings(pinned, w.num_positive)
            rid = srv.submit(be, w.literals)
            if prev is not None:
                got = srv.result(prev[0]).copy()
                prev[1].close()
            prev = (rid, be)
        got = srv.result(prev[0]).copy()
        prev[1].close()
        return got

    pipelined(max(2, min(args.warmup, 3)))
    torch.cuda.synchronize()
    barrier()
    pipe_runs = []
    for _ in range(E2E_REPEATS):
        t0 = time.perf_counter()
        pipe_counts = pipelined(args.steps)
        pipe_runs.append((time.perf_counter() - t0) / args.steps)
    srv.close()
    pipe_s = statistics.median(pipe_runs)
    if dist is not None:
        t = torch.tensor([pipe_s], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        pipe_s = float(t.item())

    serving = None
    if not args.no_serving and args.workload == "batched_step":
        serving = run_serving(eng, w, dev, torch)
    coverage = loader = testrun = None
    if args.workload == "batched_step" and not args.no_coverage and rank == 0:
        coverage = run_coverage(eng, w, b, dev, torch, measured_peak_hbm()[0], args.no_cpu)
        testrun = run_test_runner(eng, w, dev, torch, args.no_cpu)
        loader = run_loader(eng, dev, torch, measured_peak_hbm()[0], args.no_cpu)
    learn = None
    if args.workload == "batched_step" and not args.no_learn and rank == 0:
        learn = run_learn_loop(torch)

    if rank == 0:
        peak, peak_kind = measured_peak_hbm()
        st_ms = {k: v[0] / args.steps for k, v in stages.items()}
        # The dominant kernel: the persistent evaluation kernel (one launch a
        # step; its own CUDA events).  Stage figures for the rest beside it.
        eval_launches = max(stages["evaluate"][1] / args.steps, 1.0)
        kernel_ms = st_ms["evaluate"] / eval_launches
        achieved = traffic["evaluate"] / eval_launches / (kernel_ms * 1e-3) / 1e9 if kernel_ms > 0 else 0.0
        stage_roof = {k: {"ms": round(st_ms[k], 4), "algorithmic_bytes": traffic[k],
                          "achieved_gbs": traffic[k] / (st_ms[k] * 1e-3) / 1e9,
                          "frac": traffic[k] / (st_ms[k] * 1e-3) / 1e9 / peak}
                      for k in ("bind_partition", "unit_plan", "evaluate") if st_ms.get(k, 0) > 0}
        ncu_traffic = profiled_traffic(args)
        line = {
            "metric": HEADLINE_METRIC,
            "value": n * world / (gms * 1e-3), "unit": "literals/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": gms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int32 keys / int64 counts", "data": "synthetic (seeded)",
            "config": workload_config(args, w),
            "e2e": {"value": n * world / pipe_s, "unit": "literals/s",
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "ms_per_step": pipe_s * 1e3,
                    "ms_per_step_repeats": [round(x * 1e3, 3) for x in pipe_runs],
                    "mode": "pipelined through one long-lived qfg_server (one slot, depth 2): each step uploads its "
                            "binding set from pinned host memory (qfg_bindings_create) while the "
                            "previous step evaluates, counts read back to the host every step",
                    "counts_equal_device_path": bool(np.array_equal(pipe_counts, batched_counts))},
            "e2e_serial": {"value": n * world / e2e_s, "unit": "literals/s",
                           "ms_per_step": e2e_s * 1e3,
                           "ms_per_step_repeats": [round(x * 1e3, 3) for x in e2e_runs],
                           "mode": "upload, qfg_evaluate_step, release, one step after another",
                           "counts_equal_device_path": bool(np.array_equal(e2e_counts, batched_counts))},
            "gpu_launches": glaunches,
            "path": "step replayed from its CUDA graph",
            "direct": {"value": n * world / (ms * 1e-3), "unit": "literals/s", "ms_per_step": ms,
                       "gpu_launches": launches, "counts_equal_graph": graph_equal},
            "stages_ms_per_step": {k: round(v, 4) for k, v in st_ms.items() if v > 0},
            "roofline": {"bound": "hbm", "kernel": "eval_batched_kernel", "achieved": achieved,
                         "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": ncu_traffic,
                         "algorithmic_bytes": traffic["evaluate"] / eval_launches,
                         "launch_ms": kernel_ms, "peak_source": peak_kind},
            "stage_roofline": stage_roof,
            "first_touch_ms": first_touch_ms,
            "autotune": tune,
            "algorithmic_bytes_per_step": traffic,
        }
        if serving is not None:
            line["serving"] = serving
        if radix is not None:
            line["radix_partition"] = radix
        if operators is not None:
            line["operators"] = operators
        if learn is not None:
            line["learn_loop"] = learn
        if coverage is not None:
            line["coverage"] = coverage
        if testrun is not None:
            line["test_runner"] = testrun
        if loader is not None:
            line["loader"] = loader
        if per_lit is not None:
            line["per_literal"] = per_lit
            line["batched_over_per_literal"] = line["value"] / (per_lit["value"] * world)
        if clk is not None:
            line["clocks"] = clk
        if not args.no_cpu:
            v, dt, s, what = cpu_baseline(w, 1, args.cpu_sample)
            line["cpu_baseline"] = {"value": v, "unit": "literals/s", "cores": 1, "kind": "port",
                                    "host": host_cpu(),
                                    "sample": f"{what} ({dt:.1f} s), oracle = C restatement of "
                                              "the reference operator chain, 1 thread like the "
                                              "reference"}
        print(json.dumps(line), flush=True)
    b.close()
    eng.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


def run_radix_partition(eng, values, stream, torch, peak, bits: int = 15, reps: int = 5):
    """qfg_radix_partition (RadixPartition, stable, PartitionTuple output) of
    one 32M-row binding column at 15 radix bits, timed with CUDA events on
    the context stream; checked for a stable partition; HBM fraction on the
    12 bytes a row of a partition's I/O (the key and the row index read, the
    index written)."""
    n = values.numel()
    tuples, offsets = eng.radix_partition(values, bits)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(reps):
        tuples, offsets = eng.radix_partition(values, bits)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / reps
    # stable partition: values grouped by digit, tuple ids ascending within
    # every partition, every row once
    v, t = tuples[:, 0], tuples[:, 1].long()
    digit = v & ((1 << bits) - 1)
    ok = bool(torch.equal(values[t], v)) and bool((digit[1:] >= digit[:-1]).all())
    same = digit[1:] == digit[:-1]
    ok = ok and bool((t[1:][same] > t[:-1][same]).all())
    ok = ok and int(offsets[-1]) == n and bool(torch.equal(
        torch.bincount(digit.long(), minlength=1 << bits).cumsum(0), offsets[1:]))
    alg = 12 * n
    return {"kernel": "qfg_radix_partition (two stable 7/8-bit passes)", "rows": n, "bits": bits,
            "ms": ms, "algorithmic_bytes": alg, "achieved_gbs": alg / (ms * 1e-3) / 1e9,
            "frac": alg / (ms * 1e-3) / 1e9 / peak, "peak": peak, "stable_partition": ok}


def run_operators(eng, w, b, dev_cols, stream, torch, peak, counts, reps: int = 3):
    """The reference's operators kept at the C ABI, each timed with CUDA events
    on the context stream over `reps` calls, at the batched step's sizes:
    BuildHashTableOnPartitions over the 15-bit RadixPartition of one 32M-row
    binding column, BuildHashTableOnTable over the largest relation's first
    column, LeftSemiJoin and RightSemiJoin of that binding column against the
    relation's column, and the label-aware extension of the binding set by
    one of the step's literals.  Bytes are the arrays each call reads and
    writes, once each; the fraction is against the measured copy peak."""
    from quickfoil_gb300 import _capi as C

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(reps):
            out = fn()
        ev1.record(stream)
        torch.cuda.synchronize()
        return ev0.elapsed_time(ev1) / reps, out

    def entry(name, ms, nbytes, **extra):
        gbs = nbytes / (ms * 1e-3) / 1e9
        return dict(name=name, ms=round(ms, 4), bytes=int(nbytes), achieved_gbs=round(gbs, 1),
                    frac=round(gbs / peak, 4), **extra)

    out = []
    col = dev_cols[0]
    n = col.numel()
    bits = 15
    tuples, offsets = eng.radix_partition(col, bits)
    ms, res = timed(lambda: eng.build_hash_table_on_partitions(tuples, offsets, bits))
    buckets, bucket_offsets, masks, nxt = res
    io = 8 * n + 8 * offsets.numel() + 4 * buckets.numel() + 8 * bucket_offsets.numel() + \
        4 * masks.numel() + 4 * nxt.numel()
    out.append(entry("qfg_build_hash_table_on_partitions", ms, io, rows=n, bits=bits))
    rel = max(w.relations, key=lambda r: len(r[0]))
    rkey = torch.from_numpy(rel[0]).to(col.device)
    m = rkey.numel()
    ms, res = timed(lambda: eng.build_hash_table_on_table([rkey]))
    io = 4 * m + 4 * res[0].numel() + 4 * res[1].numel()
    out.append(entry("qfg_build_hash_table_on_table", ms, io, rows=m))
    ms, res = timed(lambda: eng.left_semijoin([col], [rkey]))
    out.append(entry("qfg_left_semijoin", ms, 4 * n + 4 * m + 8 * res[0].numel(), probe_rows=n,
                     build_rows=m, ones=int(res[1])))
    ms, res = timed(lambda: eng.right_semijoin([col], [rkey]))
    out.append(entry("qfg_right_semijoin", ms, 4 * n + 4 * m + 8 * res[0].numel(), probe_rows=n,
                     build_rows=m, ones=int(res[1])))
    # Extension by the step literal with the fewest binding pairs above 1M.
    pairs = counts[:, 2] + counts[:, 3]
    pick = [i for i in np.argsort(pairs) if pairs[i] >= 1_000_000]
    if pick:
        i = int(pick[0])
        lit = w.literals[i]
        npos, nneg = int(counts[i, 2]), int(counts[i, 3])
        nb = eng.extend_bindings(b, lit, npos, nneg)
        nb.close()
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        total = 0.0
        for _ in range(reps):
            ev0.record(stream)
            nb = eng.extend_bindings(b, lit, npos, nneg)
            ev1.record(stream)
            torch.cuda.synchronize()
            total += ev0.elapsed_time(ev1)
            ncols_out = nb.num_columns
            nb.close()
        ms = total / reps
        io = 4 * b.num_columns * b.num_tuples + 4 * ncols_out * (npos + nneg)
        out.append(entry("qfg_extend_bindings", ms, io, rows_in=b.num_tuples,
                         rows_out=npos + nneg, columns_out=ncols_out))
    return out


def run_learn_loop(torch):
    """BASELINE config 4 at full scale (1M pictures): the reference learner's
    recorded run replayed call by call on the device (tests/learn_replay.py,
    every result checked against the reference's), in a fresh engine.  GPU
    seconds of the replayed calls (each timed with a device synchronize on
    both sides) beside the reference's own seconds inside the same calls and
    in Learn as a whole (one x86 core, recorded when the trace was made)."""
    from quickfoil_gb300 import Engine
    from tests import learn_replay
    # A warm-up replay in a first engine loads the kernels; the timed replay
    # runs in a fresh engine, so its relation key tables are built on first
    # use inside the calls, as in a learn run.
    for _ in range(2):
        eng = Engine(torch.cuda.current_device())
        try:
            t0 = time.perf_counter()
            out = learn_replay.replay(eng, torch)
            wall = time.perf_counter() - t0
        finally:
            eng.close()
    ref = out["reference_seconds"]
    ref_calls = ref["evaluate"] + ref["extend"] + ref["coverage"]
    return {"metric": "full-scale learn loop (config 4): seconds in the data-parallel calls",
            "gpu_seconds": out["gpu_seconds_total"], "gpu_seconds_by_call": out["gpu_seconds"],
            "reference_seconds_in_calls": ref_calls, "reference_learn_seconds": ref["learn"],
            "reference_seconds_by_call": ref, "speedup_in_calls": ref_calls / out["gpu_seconds_total"],
            "calls": out["calls"], "knowledge_base": out["knowledge_base"],
            "replay_wall_seconds_incl_checks": wall,
            "results_equal_reference": True, "learnt_clauses": out["reference_clauses"],
            "reference_host": "x86_64 build container, 1 core (the reference cannot run on the GPU host)"}


def run_serving(eng, w, dev, torch, n_requests: int = 64, lits_per_request: int = 64, slots: int = 8):
    """The serving loop (config 5): 64 rule searches' literal batches over
    device-resident binding sets of log-uniform 10K-20M rows x 6 columns
    (10% positive), against the step's relations; a burst (all requests at
    once), then Poisson arrivals at ~80% of the burst throughput."""
    from quickfoil_gb300 import workloads
    rng = np.random.default_rng(11)
    sizes = np.exp(rng.uniform(np.log(10_000), np.log(20_000_000), n_requests)).astype(np.int64)
    gen = torch.Generator(device=dev)
    gen.manual_seed(11)
    reqs = []
    for nrows in sizes:
        cols = [torch.randint(0, w.domain, (int(nrows),), dtype=torch.int32, device=dev, generator=gen)
                for _ in range(6)]
        lits = workloads.random_literals(lits_per_request, w.relations, 6, rng)
        b = eng.bindings(cols, int(nrows) // 10)
        eng.step_scratch_bytes(b, lits)  # builds any key tables these literals need
        reqs.append((b, lits, cols))
    order = np.argsort(sizes)
    check = [int(order[0]), int(order[n_requests // 2]), int(order[-1])]
    alone = {i: eng.evaluate_step(reqs[i][0], reqs[i][1]) for i in check}
    torch.cuda.synchronize()

    # One server for the whole leg, as a serving process keeps it: an
    # unmeasured burst allocates its slots' scratch, then each measured run
    # starts from fresh statistics.
    srv = eng.server(slots=slots)

    def run(arrivals):
        srv.reset_stats()
        t0 = time.perf_counter()
        ids = []
        for i, (b, lits, _) in enumerate(reqs):
            while arrivals is not None and time.perf_counter() - t0 < arrivals[i]:
                srv.poll()
                time.sleep(0.0001)
            ids.append(srv.submit(b, lits))
        srv.drain()
        dt = time.perf_counter() - t0
        st = srv.stats()
        equal = all(np.array_equal(srv.result(ids[i]), alone[i]) for i in check)
        return dt, st, equal

    run(None)  # warm-up
    burst_s, st_b, eq_b = run(None)
    arrivals = np.cumsum(rng.exponential(burst_s / n_requests / 0.8, n_requests))
    pois_s, st_p, eq_p = run(arrivals)
    srv.close()
    for b, _, _ in reqs:
        b.close()
    total = n_requests * lits_per_request
    return {"requests": n_requests, "literals_per_request": lits_per_request, "slots": slots,
            "binding_rows": {"min": int(sizes.min()), "median": int(np.median(sizes)),
                             "max": int(sizes.max()), "total": int(sizes.sum())},
            "burst": {"literals_per_s": total / burst_s, "makespan_ms": burst_s * 1e3,
                      "p50_ms": st_b["p50_ms"], "p99_ms": st_b["p99_ms"],
                      "peak_in_flight": st_b["peak_in_flight"]},
            "poisson": {"literals_per_s": total / pois_s, "makespan_ms": pois_s * 1e3,
                        "offered_load": 0.8, "p50_ms": st_p["p50_ms"], "p99_ms": st_p["p99_ms"],
                        "peak_in_flight": st_p["peak_in_flight"]},
            "counts_equal_alone": bool(eq_b and eq_p)}


def run_coverage(eng, w, b, dev, torch, peak, no_cpu: bool, n_lits: int = 16, reps: int = 5):
    """Coverage on acceptance of the step's first n_lits distinct literals
    appended to the clause whose binding set is the step's (target = binding
    columns 0-1): 2M uncovered positives (half the target tuples of sampled
    positive binding rows, half random) and 4M original negatives (likewise
    from negative rows), covered counts of both and the positives' bit
    vector.  Timed as the learner runs it -- example tables prepared once
    (qfg_examples), one qfg_coverage_examples per literal -- and through the
    plain qfg_coverage that hashes the examples on every call; then the
    compaction of the uncovered positives (qfg_compact_rows).  Every call
    reads its counts back to the host."""
    import oracle
    from quickfoil_gb300 import _capi as C
    rng = np.random.default_rng(5)
    B, P, k = w.binding_columns, w.num_positive, 2
    n = len(B[0])
    npos, nneg = min(1_000_000, P // 2), min(2_000_000, (n - P) // 2)
    pos_rows = rng.choice(P, npos, replace=False)
    neg_rows = P + rng.choice(n - P, nneg, replace=False)
    U = [np.concatenate([B[q][pos_rows], rng.integers(0, w.domain, npos).astype(np.int32)])
         for q in range(k)]
    Ng = [np.concatenate([B[q][neg_rows], rng.integers(0, w.domain, nneg).astype(np.int32)])
          for q in range(k)]
    dU = [torch.from_numpy(c).to(dev) for c in U]
    dN = [torch.from_numpy(c).to(dev) for c in Ng]
    lits = list(dict.fromkeys(w.literals))[:n_lits]
    eu, en = eng.examples(dU), eng.examples(dN)
    for _ in range(3):
        for l in lits:
            eng.coverage_examples(b, l, eu, en)
            eng.coverage(b, l, k, dU, dN)
    torch.cuda.synchronize()

    def timed(fn):
        launches0 = eng.kernel_launches()
        t0 = time.perf_counter()
        out = []
        for _ in range(reps):
            out = [fn(l) for l in lits]
        torch.cuda.synchronize()
        return out, (time.perf_counter() - t0) / (reps * len(lits)), \
            (eng.kernel_launches() - launches0) / (reps * len(lits))

    got, call_s, launches = timed(lambda l: eng.coverage_examples(b, l, eu, en))
    got_plain, plain_s, plain_launches = timed(lambda l: eng.coverage(b, l, k, dU, dN))
    same_paths = all(a[0] == c[0] and torch.equal(a[1], c[1]) for a, c in zip(got, got_plain))
    # device time of the stages (CUDA events around the launches)
    eng.set_option(C.QFG_OPT_STAGE_TIMING, 1)
    eng.stage_times(reset=True)
    for l in lits:
        eng.coverage_examples(b, l, eu, en)
    st = eng.stage_times(reset=True)
    eng.set_option(C.QFG_OPT_STAGE_TIMING, 0)
    scan_ms = st["coverage_scan"][0] / len(lits)
    ex_ms = st["coverage_examples"][0] / len(lits)
    best = max(range(len(got)), key=lambda i: got[i][0][0])  # the literal covering most
    bits0 = got[best][1]
    left = eng.compact_rows(dU, bits0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        left = eng.compact_rows(dU, bits0)
    torch.cuda.synchronize()
    comp_s = (time.perf_counter() - t0) / reps
    eu.close()
    en.close()
    # algorithmic bytes of the pass over the binding rows: every row's
    # bound-key columns (the relation's key set and the examples' stay in L2)
    scan_bytes = float(np.mean([4 * n * sum(1 for v in l.vars if v >= 0) for l in lits]))
    kept = int(left[0].numel())
    comp_bytes = 4 * k * (len(U[0]) + kept) + len(U[0]) // 8
    ok = None
    cpu = None
    if not no_cpu:
        t0 = time.perf_counter()
        m, ok = 0, True
        for l, (counts, bits) in zip(lits, got):
            want = oracle.coverage(B, P, w.relations[l.relation], l.as_tuple(), k, U, Ng)
            ok &= counts == want[0] and np.array_equal(bits.cpu().numpy().view(np.uint64), want[1])
            m += 1
            if time.perf_counter() - t0 > 6.0:
                break
        dt = time.perf_counter() - t0
        cpu = {"value": m / dt, "unit": "coverage calls/s", "cores": 1, "kind": "port",
               "sample": f"first {m} of {len(lits)} literals, full size ({dt:.1f} s), also the "
                         "parity check of those calls"}
    return {"metric": "literal coverage calls/s (covered positives + negatives + bit vector)",
            "value": 1.0 / call_s, "unit": "coverage calls/s", "ms_per_call": call_s * 1e3,
            "path": "qfg_coverage_examples on example tables prepared once",
            "gpu_launches_per_call": launches,
            "plain": {"value": 1.0 / plain_s, "ms_per_call": plain_s * 1e3,
                      "gpu_launches_per_call": plain_launches,
                      "path": "qfg_coverage (example key sets built every call)",
                      "results_equal_prepared": bool(same_paths)},
            "stages_ms_per_call": {"coverage_scan": scan_ms, "coverage_examples": ex_ms},
            "workload": {"binding_rows": n, "binding_positive": P, "target_columns": k,
                         "uncovered_positives": len(U[0]), "negatives": len(Ng[0]),
                         "literals": len(lits), "repeats": reps},
            "roofline": {"bound": "hbm", "kernel": "coverage scan (binding-row pass)",
                         "algorithmic_bytes": scan_bytes,
                         "achieved": scan_bytes / (scan_ms * 1e-3) / 1e9, "peak": peak,
                         "unit": "GB/s", "frac": scan_bytes / (scan_ms * 1e-3) / 1e9 / peak},
            "compaction": {"ms": comp_s * 1e3, "rows_in": len(U[0]), "rows_kept": kept,
                           "algorithmic_bytes": comp_bytes,
                           "achieved_gbs": comp_bytes / comp_s / 1e9,
                           "frac": comp_bytes / comp_s / 1e9 / peak},
            "cpu_baseline": cpu, "counts_equal_oracle": ok}


def run_loader(eng, dev, torch, peak, no_cpu: bool, lines: int = 10_000_000, reps: int = 5):
    """The fact loader (qfg_parse_text, LoadData on the device): a text of
    `lines` facts of two random int32 arguments (about 220 MB), parsed from
    device memory (the `value`) and from host memory with the copy inside
    the timed region (`e2e`); the oracle's parser on the same text is the
    CPU baseline."""
    import ctypes
    import oracle
    from quickfoil_gb300 import _capi as C
    from quickfoil_gb300.workloads import facts_text
    rng = np.random.default_rng(17)
    cols = [rng.integers(-2 ** 31, 2 ** 31, lines).astype(np.int32) for _ in range(2)]
    text = facts_text(cols)
    dtext = torch.from_numpy(np.frombuffer(text, dtype=np.uint8).copy()).to(dev)
    outs = [torch.empty(lines, dtype=torch.int32, device=dev) for _ in range(2)]
    optr = C.ptr_array([o.data_ptr() for o in outs])
    rows, err = ctypes.c_int64(), ctypes.c_int64()
    dptr = ctypes.cast(ctypes.c_void_p(dtext.data_ptr()), ctypes.c_char_p)

    def parse(src, flags):
        C.check(eng.lib.qfg_parse_text(eng.ctx, src, len(text), flags, 2, None, optr, lines,
                                       ctypes.byref(rows), ctypes.byref(err)),
                eng.ctx, "qfg_parse_text")

    for _ in range(2):
        parse(dptr, C.QFG_DEVICE_BORROW)
        parse(text, C.QFG_HOST)
    torch.cuda.synchronize()
    ok = rows.value == lines and all(torch.equal(o.cpu(), torch.from_numpy(c)) for o, c in zip(outs, cols))
    timings = {}
    for name, src, flags in (("device", dptr, C.QFG_DEVICE_BORROW), ("host", text, C.QFG_HOST)):
        t0 = time.perf_counter()
        for _ in range(reps):
            parse(src, flags)
        torch.cuda.synchronize()
        timings[name] = (time.perf_counter() - t0) / reps
    alg = len(text) + 8 * lines  # the text read once, the columns written once
    line = {"metric": "fact text parsed (GB/s of '|'-delimited text)",
            "value": len(text) / timings["device"] / 1e9, "unit": "GB/s",
            "facts_per_s": lines / timings["device"], "ms": timings["device"] * 1e3,
            "e2e": {"value": len(text) / timings["host"] / 1e9, "unit": "GB/s",
                    "ms": timings["host"] * 1e3, "h2d_bytes": len(text),
                    "mode": "qfg_parse_text from pageable host memory, copy included"},
            "text_bytes": len(text), "facts": lines, "arguments": 2,
            "roofline": {"bound": "hbm", "algorithmic_bytes": alg,
                         "achieved": alg / timings["device"] / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": alg / timings["device"] / 1e9 / peak,
                         "note": "wall time of the call: newline pass, line scan, parse, compaction"},
            "columns_equal_input": bool(ok)}
    if not no_cpu:
        t0 = time.perf_counter()
        got = oracle.parse_text(text, 2)
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": len(text) / dt / 1e9, "unit": "GB/s", "cores": 1,
                                "kind": "port", "sample": f"the whole text ({dt:.1f} s)",
                                "columns_equal": bool(all(np.array_equal(g, c) for g, c in zip(got, cols)))}
    return line


def run_test_runner(eng, w, dev, torch, no_cpu: bool, test_rows: int = 4_000_000, reps: int = 3):
    """The device test runner (qfg_run_test, QuickFoilTestRunner::RunTest):
    a test table of `test_rows` two-column rows (binding rows of the step:
    their values meet the step's relations), three clauses of two body
    literals over the step's relations; the oracle's restatement on the same
    inputs is the CPU baseline."""
    import oracle
    from quickfoil_gb300 import workloads
    from quickfoil_gb300.engine import Literal
    rng = np.random.default_rng(23)
    rows = rng.choice(len(w.binding_columns[0]), test_rows, replace=False)
    test = [w.binding_columns[q][rows] for q in range(2)]
    lits = workloads.random_literals(64, w.relations, 2, rng)
    clauses = []
    for i in range(3):
        first = next(l for l in lits[8 * i:] if any(v < 0 for v in l.vars))
        # the second literal joins on the column the first one introduced
        tmpl = lits[40 + i]
        jb = next(j for j, v in enumerate(tmpl.vars) if v >= 0)
        second = Literal(tmpl.relation, tuple(2 if j == jb else v for j, v in enumerate(tmpl.vars)))
        clauses.append([first, second])
    dtest = [torch.from_numpy(c).to(dev) for c in test]
    left = eng.run_test(clauses, dtest)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        left = eng.run_test(clauses, dtest)
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / reps
    line = {"metric": "test rows checked/s (learnt clauses on a test table)",
            "value": test_rows / dt, "unit": "rows/s", "ms": dt * 1e3, "test_rows": test_rows,
            "clauses": [[(l.relation, list(l.vars)) for l in c] for c in clauses],
            "uncovered": left}
    if not no_cpu:
        t0 = time.perf_counter()
        want = oracle.run_test(w.relations, [[(l.relation, l.vars) for l in c] for c in clauses],
                               test)
        cdt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": test_rows / cdt, "unit": "rows/s", "cores": 1,
                                "kind": "port", "sample": f"the same test table ({cdt:.1f} s)"}
        line["uncovered_equal_oracle"] = len(want[0]) == left
    return line


def main():
    args = parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
