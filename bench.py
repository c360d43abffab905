#!/usr/bin/env python
"""Benchmark of the GB300 refinement engine: pins/s per refinement pass.

Workload (default "zipf4m"): all six metrics (CN, TV, TM, MSM, MSV, MSRV), each on
its own resident instance: K = 256, eps = 0.05 (C = (W/K) * 1.05),
4,194,304 vertices and 4,194,304 nets, net sizes Zipf(2.1) clipped to
[2, 10000], pins drawn by a Zipf(1.5) vertex popularity, source = first drawn
pin, vertex weight = degree; 10 refinement passes.  Synthetic and seeded.

A step is one refinement pass of each of the six resident instances; the
instances carry their state between steps and restart from the streaming
initial partition (untimed) every 10 steps, so the default --steps 10 times one
complete 10-pass schedule.  metric = pins * passes / refinement seconds over the
six metrics (the reference's "Refinement took" span).

  value   device-resident: CUDA events on the engine's stream around each
          refinement launch
  e2e     through the C ABI with host buffers: host -> device upload of the
          state, the passes, device -> host copy of the part vector
  --impl reference: the reference's own OpenMP partition_par() (compiled from
          its sources into oracle/_ref) on every host core, on the same
          hypergraph (drawn by the oracle's generator, no product library
          loaded), K and pass schedule.  The reference has no vertex weights
          (it counts vertices), so it runs the unit-weight form of the
          instance; cpu_baseline is the same on the first passes of the
          schedule (a bounded sample)

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
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
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRICS = ["CN", "TV", "TM", "MSM", "MSV", "MSRV"]
# the headline metric, the same string on both arms
METRIC = "pins/s per refine pass (pins x passes / refinement seconds, six metrics)"
WORKLOADS = {
    "zipf4m": dict(nov=4_194_304, noe=4_194_304, alpha=2.1, lo=2, hi=10000, beta=1.5, weight_rule=1, K=256,
               eps=1.05, passes=10, seed=0),
    "uniform16k": dict(nov=16_384, noe=16_384, alpha=0.0, lo=2, hi=16, beta=0.0, weight_rule=0, K=8, eps=1.03,
               passes=5, seed=0),
    # high-K heavy-tail stress of the message and send+receive volume metrics:
    # ~119 M pins, nets up to 100,000 pins, uniform vertex popularity
    "zipf16m_k1024": dict(nov=16_777_216, noe=8_388_608, alpha=1.9, lo=2, hi=100_000, beta=0.0, weight_rule=0,
               K=1024, eps=1.05, passes=10, seed=0, metrics="TM,MSRV"),
}


def metrics_for(w, arg):
    """The metrics a run covers: --metrics, else the workload's own list, else all six."""
    if arg:
        return arg.split(",")
    return w["metrics"].split(",") if "metrics" in w else list(METRICS)


def measured_traffic(kernel, config, scale, metrics=None):
    """DRAM bytes per launch of `kernel` on the full-size workload, from the
    ncu summaries under profiles/: lines `traffic: <kernel> <config> <metric>
    <bytes>` (dram__bytes_read.sum + dram__bytes_write.sum of one captured
    launch of that metric's instance).  The mean over `metrics` (the metrics
    whose launches the kernel ran, one launch each per step); None when a
    metric has no line or the run is not full size."""
    if scale != 1:
        return None
    found = {}
    for md in sorted((ROOT / "profiles").glob("*.md")):
        for line in md.read_text().splitlines():
            f = line.strip().strip("`").split()
            if len(f) == 5 and f[0] == "traffic:" and f[1] == kernel and f[2] == config:
                try:
                    found[f[3]] = int(float(f[4]))
                except ValueError:
                    pass
    want = list(metrics) if metrics else sorted(found)
    if not want or any(m not in found for m in want):
        return None
    return int(sum(found[m] for m in want) / len(want))


def spec_for(fp, w, scale=1, unit_weights=False):
    nov, noe = max(w["nov"] // scale, 1024), max(w["noe"] // scale, 1024)
    if w["alpha"] > 0:
        return fp.GenSpec.zipf(nov, noe, w["alpha"], w["lo"], min(w["hi"], nov), beta=w["beta"],
                               weight_rule=0 if unit_weights else w["weight_rule"], seed=w["seed"])
    return fp.GenSpec.column_net(nov, noe, w["lo"], w["hi"], seed=w["seed"])


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def algorithmic_bytes(metric, hg, ep_len, moved_mask, K):
    """Bytes one refinement pass must move at minimum: vertex CSR, per-pin net offset + part count, the listed parts
    scanned, the part vector, part sizes, and the list slots a move rewrites.
    The TM/MSM/MSV/MSRV passes also read the source and its part per pin, the
    counts of the scanned slots, and one K-row per evaluated vertex (TM/MSM)."""
    sizes = np.diff(hg.nptr).astype(np.int64)
    lam = ep_len.astype(np.int64)
    P = hg.pins
    scanned = int(np.sum(sizes * lam))                 # sum over (v, e) of lambda_e
    deg = np.diff(hg.vptr).astype(np.int64)
    if metric == "CN":
        two = lam == 2
        return 4 * (hg.noe + 1) + 8 * hg.noe + int(np.sum(8 * sizes[two]))
    b = 4 * (hg.nov + 1) + 4 * P + 8 * P + 4 * scanned + 4 * hg.nov + 8 * K
    if moved_mask is not None and moved_mask.any():
        vv = np.nonzero(moved_mask)[0]
        net_lam = lam[hg.vnets.astype(np.int64)]
        cs = np.concatenate([np.zeros(1, np.int64), np.cumsum(net_lam)])
        per_v = cs[hg.vptr[1:].astype(np.int64)] - cs[hg.vptr[:-1].astype(np.int64)]
        b += 16 * int(per_v[vv].sum())
    if metric != "TV":
        b += 8 * P + 4 * scanned + 4 * K
        if metric in ("TM", "MSM"):
            b += 4 * K * hg.nov
    return b


KERNEL_OF = {"TV": "spec_ldg_kernel", "MSV": "spec_ldg_kernel", "MSRV": "spec_ldg_kernel",
             "CN": "spec_cn_kernel", "TM": "spec_msg_kernel", "MSM": "spec_msg_kernel"}


def whole_job(units_per_rank, seconds, device="cpu"):
    """Whole-job throughput of independent replicas: every rank processes the
    same `units_per_rank`, the job takes as long as its slowest rank (an
    all-reduce MAX of `seconds` over the process group when one is up; the
    tensor lives on `device`, "cpu" for gloo, "cuda:N" for nccl), and the value
    is all ranks' units over that time.  Returns (value, max seconds, ranks)."""
    import torch
    import torch.distributed as tdist
    nranks = 1
    if tdist.is_available() and tdist.is_initialized():
        t = torch.tensor([seconds], dtype=torch.float64, device=device)
        tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
        seconds = float(t.item())
        nranks = tdist.get_world_size()
    return units_per_rank * nranks / seconds, seconds, nranks


def time_schedule(eng, stream, hg, w, metrics, passes, steps, warmup, account=True):
    """Resident instances of every metric on hg; W untimed warm-up steps, then
    `steps` timed steps (one pass of each instance per step, restarting from
    the initial partition every `passes` steps).  Returns (instances,
    per-metric seconds per step, per-metric algorithmic bytes per step,
    seconds of host initial partitions)."""
    import torch
    insts = {}
    t_init = time.time()
    for m in metrics:
        inst = eng.instance(hg, w["K"], m, w["eps"])
        inst.initial_partition()
        insts[m] = inst
    t_init = time.time() - t_init
    done = {"n": 0}

    def reset_all():
        for inst in insts.values():
            inst.reset_state()
        done["n"] = 0

    def one_step(timed, acc=None):
        if done["n"] == passes:
            reset_all()
        out = {}
        for m in metrics:
            inst = insts[m]
            if acc is not None:
                ln, _, _ = inst.lists()
                before = inst.partition()
            torch.cuda.synchronize()
            if timed:
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
            inst.refine(1)
            if timed:
                e1.record(stream)
                e1.synchronize()
                out[m] = e0.elapsed_time(e1) / 1e3
            if acc is not None:
                after = inst.partition()
                acc[m].append(algorithmic_bytes(m, hg, ln, before != after, w["K"]))
        done["n"] += 1
        return out

    for _ in range(warmup):
        one_step(False)
    reset_all()
    torch.cuda.synchronize()
    per_metric = {m: [] for m in metrics}
    bytes_acc = {m: [] for m in metrics} if account else None
    for _ in range(steps):
        for m, t in one_step(True, bytes_acc).items():
            per_metric[m].append(t)
    torch.cuda.synchronize()
    return insts, per_metric, bytes_acc, t_init


def run_ours(args):
    import torch
    import fastpartitioner_gb300 as fp

    dist = int(os.environ.get("WORLD_SIZE", "1")) > 1
    rank = int(os.environ.get("RANK", "0"))
    if dist:
        import torch.distributed as tdist
        local = int(os.environ.get("LOCAL_RANK", "0"))
        torch.cuda.set_device(local)
        tdist.init_process_group("nccl")
        device = local
    else:
        device = 0
        torch.cuda.set_device(0)
    w = WORKLOADS[args.config]
    passes = args.passes or w["passes"]
    metrics = metrics_for(w, args.metrics)
    t_gen = time.time()
    hg = fp.generate(spec_for(fp, w, args.scale))
    t_gen = time.time() - t_gen
    stream = torch.cuda.Stream(device=device)
    eng = fp.Engine(device)
    eng.set_stream(stream.cuda_stream)

    if dist:
        tdist.barrier()
    with Clocks(device) as clk:
        insts, per_metric, bytes_acc, t_init = time_schedule(eng, stream, hg, w, metrics, passes, args.steps,
                                                             args.warmup)
    if dist:
        tdist.barrier()
    launches = len(metrics) * args.steps
    total_t = sum(sum(v) for v in per_metric.values())
    value, total_t, nranks = whole_job(hg.pins * len(metrics) * args.steps, total_t, f"cuda:{device}")

    # e2e: the call a user makes per metric -- host state -> device, all passes,
    # part vector -> host -- timed on the wall clock, one schedule.
    e2e_t = 0.0
    h2d = d2h = 0
    for m in metrics:
        inst = insts[m]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        inst.reset_state()
        inst.refine(passes)
        pv = inst.partition()
        t1 = time.perf_counter()
        e2e_t += t1 - t0
        h2d += inst.state_bytes()
        d2h += pv.nbytes
    e2e_value, e2e_t, _ = whole_job(hg.pins * passes * len(metrics), e2e_t, f"cuda:{device}")
    for inst in insts.values():
        inst.close()

    # Roofline per kernel: algorithmic bytes of one launch (one pass of one
    # metric) / its CUDA-event duration; the dominant kernel is the one with the
    # largest share of the timed region.
    peak, peak_kind = peaks()
    kern = {}
    for m in metrics:
        k = kern.setdefault(KERNEL_OF[m], {"t": 0.0, "bytes": 0, "launches": 0, "metrics": []})
        k["t"] += sum(per_metric[m])
        k["bytes"] += sum(bytes_acc[m])
        k["launches"] += len(per_metric[m])
        k["metrics"].append(m)
    per_kernel = {}
    for name, k in kern.items():
        ach = k["bytes"] / k["t"] / 1e9
        per_kernel[name] = {"metrics": k["metrics"], "share": k["t"] / total_t, "launches": k["launches"],
                            "avg_launch_ms": 1e3 * k["t"] / k["launches"],
                            "algorithmic_bytes_per_launch": int(k["bytes"] / k["launches"]),
                            "achieved_gbs": ach, "frac": ach / peak}
    dom = max(per_kernel, key=lambda n: per_kernel[n]["share"])
    traffic = measured_traffic(dom, args.config, args.scale, per_kernel[dom]["metrics"])
    unique = unique_bytes(hg, w["K"])
    dom_metrics = per_kernel[dom]["metrics"]
    uniq_per_launch = sum(unique[m] * len(per_metric[m]) for m in dom_metrics) / per_kernel[dom]["launches"]
    uniq_gbs = uniq_per_launch / (per_kernel[dom]["avg_launch_ms"] / 1e3) / 1e9

    cpu = None
    if not args.no_cpu_baseline and rank == 0:
        cpu = cpu_baseline(w, args, per_metric)
    clocks = clk.summary()
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "pins/s",
        "n_gpus": nranks,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": total_t / args.steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "int32",
        "data": "synthetic (seeded generator, fastpartitioner_gb300/csrc/fp_gen.cpp)",
        "config": {
            "workload": workload_text(args.config, w, hg.nov, hg.noe, hg.pins, passes, metrics,
                                      "degree" if w["weight_rule"] else "unit"),
            "step": STEP_TEXT.format(passes=passes),
            "weights": ("vertex weight = degree; the reference arm and cpu_baseline run the same hypergraph "
                        "with unit weights (the reference counts vertices)") if w["weight_rule"] else "unit",
            "l2": "inputs larger than L2 (per-instance CSRs and lists exceed 129 MB)" if hg.pins > 8_000_000
                  else "inputs smaller than L2",
            "per_metric_pins_per_s": {m: hg.pins * len(v) / sum(v) for m, v in per_metric.items()},
            "per_metric_ms_per_pass": {m: 1e3 * statistics.mean(v) for m, v in per_metric.items()},
            "scale": args.scale,
            "generate_s": round(t_gen, 2),
            "host_initial_partition_s": round(t_init, 2),
            "parallelism": "one instance per metric on one GPU (replicas only across GPUs)",
            "e2e_step": f"per metric: reset_state (host -> device) + refine({passes}) + partition (device -> host)",
        },
        "e2e": {"value": e2e_value, "unit": "pins/s", "h2d_bytes_per_step": h2d // len(metrics),
                "d2h_bytes_per_step": d2h // len(metrics)},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": per_kernel[dom]["achieved_gbs"], "peak": peak,
                     "unit": "GB/s", "frac": per_kernel[dom]["achieved_gbs"] / peak,
                     "peak_kind": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                     else peak_kind, "traffic": traffic,
                     "unique_bytes_per_launch": int(uniq_per_launch), "unique_achieved": uniq_gbs,
                     "unique_frac": uniq_gbs / peak, "per_kernel": per_kernel},
        "cpu_baseline": cpu,
        "clocks": clocks,
    }
    eng.close()
    if dist:
        tdist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line), flush=True)


STEP_TEXT = ("one refinement pass of each metric's resident instance (state carried between steps; "
             "restart from the initial partition every {passes} steps, untimed)")


def workload_text(name, w, nov, noe, pins, passes, metrics, weights):
    """The workload string of either arm (they differ only in the weights)."""
    return (f"{name}: {nov} vertices, {noe} nets, {pins} pins, {weights} weights, K={w['K']}, eps factor "
            f"{w['eps']}, {passes}-pass schedule, metrics {','.join(metrics)}")


def unique_bytes(hg, K):
    """Bytes a pass touches at least once (each array read once, the refined
    arrays written once): vertex CSR, net offsets, part vector, the per-net
    (part, count) lists; the LDG and message metrics also read the sources and
    the net -> pins CSR is not needed; TM / MSM also a K x K count table.  A
    per-pass lower bound against which re-reads of the lists show up."""
    P, nov, noe = hg.pins, hg.nov, hg.noe
    base = 4 * (nov + 1) + 4 * P + 4 * (noe + 1) + 2 * 4 * nov + 2 * 4 * (noe + 2 * P)
    out = {m: base + 4 * noe for m in METRICS}
    out["CN"] = 4 * (noe + 1) + 4 * P + 2 * 4 * nov + 2 * 4 * (noe + 2 * P)
    for m in ("TM", "MSM"):
        out[m] += 4 * K * K
    return out


# The reference's partition_par() is racy: on small instances at K = 256 with 8
# threads, 8 of 20 TV runs and up to 10 of 20 CN runs ended with SIGSEGV (the
# full-size instance ran cleanly).  A run that a signal ended is run again, up
# to this many times, and the number of such runs is reported with the baseline.
REFERENCE_TRIES = 12


def run_reference_retrying(oracle, path, K, metric, passes, threads):
    """oracle.run_reference_file, again after a run that a signal ended;
    returns (result, crashed runs)."""
    crashes = 0
    while True:
        try:
            return oracle.run_reference_file(path, K, metric, passes, threads=threads), crashes
        except oracle.ReferenceRunError as e:
            crashes += 1
            if e.returncode >= 0 or crashes >= REFERENCE_TRIES:
                raise


def instance_file(w, scale, tmpdir):
    """The workload's unit-weight instance drawn by the oracle's generator
    (the product generator's draws, no product library loaded) as an .fphg
    file; returns (path, (nov, noe, pins))."""
    import oracle
    nov, noe = max(w["nov"] // scale, 1024), max(w["noe"] // scale, 1024)
    path = Path(tmpdir) / f"inst_{scale}.fphg"
    if w["alpha"] > 0:
        oracle.generate_fphg(path, nov, noe, w["lo"], min(w["hi"], nov), w["alpha"], w["beta"], 1, 0, w["seed"])
    else:
        oracle.generate_fphg(path, nov, noe, w["lo"], w["hi"], 0.0, 0.0, 0, 1, w["seed"])
    return path, oracle.fphg_header(path)


def reference_schedule(path, K, metrics, steps, passes, threads, kind="reference"):
    """The reference's partition_par() (threads > 1; partition() otherwise) on
    the instance file for `steps` steps of the pass schedule: per metric, runs
    of `passes` passes (the schedule restarts from the stream, as the GPU arm's
    instances do) and a shorter last run for the remainder.  kind "port": the
    oracle's restatement (one thread) where the reference was not built.
    Returns {metric: (passes timed, refinement seconds)} and the crashed runs
    retried."""
    import oracle
    out, crashes = {}, 0
    inst = oracle.FphgInstance(path) if kind == "port" else None
    for m in metrics:
        left, t, n = steps, 0.0, 0
        while left > 0:
            run = min(left, passes)
            if inst is not None:
                t += oracle.run_oracle(inst, K, m, run, eps_factor=1.05)["refine_seconds"]
            else:
                r, c = run_reference_retrying(oracle, path, K, m, run, threads)
                crashes += c
                t += r["refine_seconds"]
            n += run
            left -= run
        out[m] = (n, t)
    return out, crashes


def reference_available():
    try:
        import oracle
        return oracle.reference_available()
    except Exception:
        return False


def cpu_baseline(w, args, per_metric_gpu):
    """The reference's partition_par() with every host thread on the same
    full-size instance, the first --cpu-passes passes of the schedule of each
    metric: a bounded sample of the reference arm's run.  The GPU's time for
    the same passes is reported beside it."""
    kind = "reference" if reference_available() else "port"
    threads = (os.cpu_count() or 1) if kind == "reference" else 1
    metrics = list(per_metric_gpu)
    n = min(args.cpu_passes, args.steps)
    with tempfile.TemporaryDirectory(prefix="fpbench") as td:
        path, (nov, noe, pins) = instance_file(w, args.scale, td)
        res, crashes = reference_schedule(path, w["K"], metrics, n, w["passes"], threads, kind)
    t = sum(v[1] for v in res.values())
    gpu_t = sum(sum(per_metric_gpu[m][:n]) for m in metrics)
    engine = f"partition_par with {threads} threads" if kind == "reference" else "the oracle restatement, one thread"
    return {"value": pins * n * len(metrics) / t, "unit": "pins/s", "cores": threads, "kind": kind,
            "crashed_runs_retried": crashes,
            "per_metric_pins_per_s": {m: pins * k / s for m, (k, s) in res.items()},
            "gpu_same_passes_pins_per_s": pins * n * len(metrics) / gpu_t if gpu_t > 0 else None,
            "sample": f"the same instance ({nov} vertices / {pins} pins, unit weights), passes 1-{n} of the "
                      f"{w['passes']}-pass schedule of each of {','.join(metrics)}, {engine}"}


def run_reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle
    try:
        oracle.build()
    except Exception:
        pass
    w = WORKLOADS[args.config]
    metrics = metrics_for(w, args.metrics)
    passes = args.passes or w["passes"]
    # the reference compiled from its sources, else the oracle's restatement
    kind = "reference" if reference_available() else "port"
    threads = (os.cpu_count() or 1) if kind == "reference" else 1
    with tempfile.TemporaryDirectory(prefix="fpbench") as td:
        # untimed warm-up: the same schedule on a 1/64-scale draw, W passes
        warm_crashes = 0
        if args.warmup:
            wpath, _ = instance_file(w, 64 * args.scale, td)
            _, warm_crashes = reference_schedule(wpath, w["K"], metrics, args.warmup, passes, threads, kind)
        path, (nov, noe, pins) = instance_file(w, args.scale, td)
        res, crashes = reference_schedule(path, w["K"], metrics, args.steps, passes, threads, kind)
        crashes += warm_crashes
    tot_t = sum(t for _, t in res.values())
    value = pins * args.steps * len(metrics) / tot_t
    engine = f"partition_par with {threads} threads" if kind == "reference" else "the oracle restatement, one thread"
    sample = (f"the whole workload ({nov} vertices / {pins} pins): {args.steps} steps = passes 1-{args.steps} of "
              f"the {passes}-pass schedule of each of {','.join(metrics)}, {engine}")
    line = {
        "metric": METRIC,
        "value": value, "unit": "pins/s", "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": tot_t / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic (seeded generator; instance drawn by oracle/fp_oracle_gen.cpp)", "impl": "reference",
        "config": {"workload": workload_text(args.config, w, nov, noe, pins, passes, metrics, "unit"),
                   "weights": "unit: the reference counts vertices and has no vertex weights; the GPU arm runs "
                              "the same hypergraph with the workload's weights",
                   "step": STEP_TEXT.format(passes=passes), "threads": threads,
                   "per_metric_pins_per_s": {m: pins * k / t for m, (k, t) in res.items()},
                   "per_metric_refine_s": {m: t for m, (_, t) in res.items()}},
        "cpu_baseline": {"value": value, "unit": "pins/s", "cores": threads, "kind": kind, "sample": sample,
                         "crashed_runs_retried": crashes},
        "e2e": {"value": value, "unit": "pins/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def same_results(a, b):
    """Whether two runs gave every request the same status, part vector and metrics."""
    for x, y in zip(a, b):
        if x.rid != y.rid or x.status != y.status:
            return False
        if x.status == 0 and (not np.array_equal(x.part_vec, y.part_vec) or x.metrics != y.metrics):
            return False
    return len(a) == len(b)


def run_batch(args):
    """Mixed batch (config: vertices log-uniform in [1e3, 1e6], nets =
    vertices x U[0.5, 2], Zipf(2.2) net sizes up to 2000 pins, K from {2, 4,
    ..., 512}, metric uniform over the six, --batch-passes passes, unit
    weights): --gpu-slots concurrent GPU slots (run_concurrent: own stream, a
    share of the SMs and a device arena each, host preparation on --workers
    threads, largest request first) against the plain per-request loop on the
    same requests; partitions/s on the wall clock, hypergraph construction and
    streaming initial partitions included."""
    import torch
    import fastpartitioner_gb300 as fp
    from fastpartitioner_gb300 import serving as sv
    torch.cuda.set_device(0)
    mk = lambda: sv.mixed_batch(args.batch_n, seed=args.batch_seed, passes=args.batch_passes)
    arena = sv.arena_for(mk())
    slots = sv.gpu_slots(0, args.gpu_slots, arena)
    eng = fp.Engine(0)
    for _ in range(args.warmup):
        sv.run_concurrent(slots, sv.mixed_batch(8, seed=99, vmax=20_000), workers=args.workers)
    conc = sv.run_concurrent(slots, mk(), workers=args.workers)
    plain = sv.run_plain(eng, mk())
    sp, sc = sv.summary(plain), sv.summary(conc)
    eng.close()
    for e in slots:
        e.close()
    line = {
        "metric": "partitions/s (mixed batch, concurrent GPU slots vs plain per-request loop)",
        "value": sc["partitions_per_s"], "unit": "partitions/s", "n_gpus": 1, "steps": 1,
        "warmup": args.warmup, "ms_per_step": 1e3 * sc["makespan_s"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded generator)",
        "config": {"workload": f"mixed batch of {args.batch_n} hypergraphs (seed {args.batch_seed}), "
                               f"{args.batch_passes} passes each", "workers": args.workers,
                   "gpu_slots": args.gpu_slots, "arena_bytes": arena, "plain_loop": sp, "concurrent": sc,
                   "speedup_vs_plain": sc["partitions_per_s"] / sp["partitions_per_s"],
                   "same_alone_and_in_the_mix": same_results(plain, conc)},
    }
    print(json.dumps(line), flush=True)


def run_serve(args):
    """Continuous serving: Poisson arrivals at --rate per second for
    --duration seconds, each request a hypergraph as in the mixed batch with
    vertices log-uniform in [1e3, --serve-vmax], admission by device footprint
    under --budget-gb, refinement on --gpu-slots concurrent GPU slots; against a
    serial queue of plain per-request calls on the same arrivals.  Latency is
    arrival to result."""
    import torch
    import fastpartitioner_gb300 as fp
    from fastpartitioner_gb300 import serving as sv
    torch.cuda.set_device(0)
    n = max(1, int(round(args.rate * args.duration)))
    mk = lambda: sv.poisson_arrivals(sv.mixed_batch(n, seed=args.batch_seed, vmax=args.serve_vmax,
                                                    passes=args.batch_passes), args.rate, seed=1)
    arena = sv.arena_for(mk())
    budget = int(args.budget_gb * 2**30)
    nslots = max(1, min(args.gpu_slots, budget // arena))
    slots = sv.gpu_slots(0, nslots, arena)
    for _ in range(args.warmup):
        sv.run_concurrent(slots, sv.mixed_batch(8, seed=99, vmax=20_000), workers=args.workers)
    srv = sv.Server(slots, budget_bytes=budget - nslots * arena, workers=args.workers, slots=args.slots)
    served = srv.run(mk())
    eng = fp.Engine(0)
    serial = sv.run_plain(eng, mk())
    ss, sq = sv.summary(served), sv.summary(serial)
    eng.close()
    for e in slots:
        e.close()
    line = {
        "metric": "p99 latency (continuous serving vs a serial plain-GPU queue)",
        "value": ss["p99_latency_s"], "unit": "s", "n_gpus": 1, "steps": 1, "warmup": args.warmup,
        "ms_per_step": 1e3 * ss["makespan_s"], "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded generator, Poisson arrivals)",
        "config": {"workload": f"{n} requests at {args.rate}/s, vertices log-uniform in [1e3, {args.serve_vmax}], "
                               f"{args.batch_passes} passes", "budget_gb": args.budget_gb,
                   "workers": args.workers, "admission_slots": args.slots, "gpu_slots": nslots,
                   "arena_bytes": arena, "served": ss, "serial_queue": sq,
                   "peak_reserved_gb": srv.peak_reserved / 2**30,
                   "same_alone_and_in_the_mix": same_results(sorted(serial, key=lambda r: r.rid), served)},
    }
    print(json.dumps(line), flush=True)


def run_stream(args):
    """Streaming initial partitions of the workload: the device stream
    (fp_set_stream_mode device: csrc/fp_stream.cu) against the host stream on
    the same instance, per metric (--metrics; default TV, MSV, MSRV, the ones
    that stream on the device by default).  Seconds of fp_initial_partition on
    the wall clock, the state's copy to the host included; every state array
    compared."""
    import torch
    import fastpartitioner_gb300 as fp
    torch.cuda.set_device(0)
    w = WORKLOADS[args.config]
    metrics = args.metrics.split(",") if args.metrics else ["TV", "MSV", "MSRV"]
    hg = fp.generate(spec_for(fp, w, args.scale))
    fields = ("part_vec", "ep_ends", "ep_parts", "ep_cnt", "part_sizes", "marker", "send", "recv", "conn", "msgs")
    per = {}
    with fp.Engine(0) as eng:
        for m in metrics:
            with eng.instance(hg, w["K"], m, w["eps"]) as inst:
                if args.stream_walk >= 0:
                    inst.set_stream_walk(bool(args.stream_walk))
                t = {}
                st = {}
                for where in ["device"] * (args.warmup + 1) + ["host"]:
                    inst.set_stream(where)
                    torch.cuda.synchronize()
                    t0 = time.perf_counter()
                    inst.initial_partition()
                    torch.cuda.synchronize()
                    t[where] = time.perf_counter() - t0
                    if where == "device" and not inst.streamed_on_device():
                        raise RuntimeError(f"{m}: the instance does not qualify for the device stream")
                    st[where] = inst.get_state()
                x = inst.stats()
                per[m] = {"device_s": t["device"], "host_s": t["host"],
                          "same": all(np.array_equal(st["device"][f], st["host"][f]) for f in fields),
                          "windows": x["windows"], "whole_grid_windows": x["heavy_rounds"],
                          "cut_size_flip": x["cut_size"], "cut_conflict": x["cut_conflict"]}
    dev = sum(v["device_s"] for v in per.values())
    host = sum(v["host_s"] for v in per.values())
    line = {
        "metric": "initial partition seconds (device stream; host stream beside it)", "value": dev, "unit": "s",
        "n_gpus": 1, "steps": 1, "warmup": args.warmup, "ms_per_step": 1e3 * dev, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic (seeded generator)",
        "config": {"workload": workload_text(args.config, w, hg.nov, hg.noe, hg.pins, 0, metrics, "degree"),
                   "stream_walk": args.stream_walk, "host_s": host, "per_metric": per,
                   "same_as_host": all(v["same"] for v in per.values())},
    }
    print(json.dumps(line), flush=True)


def run_transforms(args):
    """The hypergraph transforms on the device against their host forms:
    createInverse (fp_create_inverse) and CN thinning (fp_thin_nets_device,
    mean factor 2, 100 pins) on the workload, the BFS visiting order
    (fp_bfs_order_device) on a 1 M-vertex Zipf hypergraph (the host BFS walks
    every (vertex, net, pin) triple: hours at the workload's size).  Seconds on
    the wall clock, host <-> device copies included; results compared."""
    import torch
    import fastpartitioner_gb300 as fp
    torch.cuda.set_device(0)
    w = WORKLOADS[args.config]
    hg = fp.generate(spec_for(fp, w, args.scale))
    g2 = fp.generate(fp.GenSpec.zipf(1_000_000 // args.scale, 1_000_000 // args.scale, 2.1, 2, 2000, beta=1.2,
                                     seed=31))

    def timed(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        return r, time.perf_counter() - t0

    def bfs(fn, *a):
        """Raw call (a vertex left unreached is FP_ERR_UNSUPPORTED, with the
        reached prefix of the ordering still written): (status, ordering)."""
        import ctypes as C
        out = np.empty(g2.nov, np.int32)
        far = np.empty(2, np.int32)
        v = g2.view()
        rc = fn(*a, C.byref(v), 7, out.ctypes.data, far.ctypes.data)
        return rc, out, far

    out = {}
    with fp.Engine(0) as eng:
        for _ in range(args.warmup):
            eng.create_inverse(hg.nov, hg.noe, hg.vptr, hg.vnets)
        (rp, ci), td = timed(lambda: eng.create_inverse(hg.nov, hg.noe, hg.vptr, hg.vnets))
        hv, th = timed(lambda: fp.Hypergraph.from_vertices(hg.nov, hg.noe, hg.vptr, hg.vnets))
        out["create_inverse"] = {"device_s": td, "host_s": th, "pins": int(hg.pins),
                                 "same": bool(np.array_equal(rp, hv.nptr) and np.array_equal(ci, hv.npins))}
        a, td = timed(lambda: eng.thin(hg, 2, 100))
        b, th = timed(lambda: hg.thin(2, 100))
        out["thin_nets"] = {"device_s": td, "host_s": th, "kept_nets": int(a.noe),
                            "same": all(np.array_equal(getattr(a, f), getattr(b, f))
                                        for f in ("vptr", "vnets", "nptr", "npins", "src"))}
        from fastpartitioner_gb300 import lib
        (rd, od, fd), td = timed(lambda: bfs(lib().fp_bfs_order_device, eng._ctx))
        (rh, oh, fh), th = timed(lambda: bfs(lib().fp_bfs_order))
        out["bfs_order"] = {"device_s": td, "host_s": th, "nov": g2.nov, "pins": int(g2.pins),
                            "reached": int((oh >= 0).sum()), "status": int(rh),
                            "same": bool(rd == rh and np.array_equal(od, oh) and np.array_equal(fd, fh))}
    line = {
        "metric": "createInverse pins/s on the device (thinning and BFS ordering beside it)",
        "value": hg.pins / out["create_inverse"]["device_s"], "unit": "pins/s", "n_gpus": 1, "steps": 1,
        "warmup": args.warmup, "ms_per_step": 1e3 * out["create_inverse"]["device_s"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "uint32", "data": "synthetic (seeded generator)",
        "config": {"workload": workload_text(args.config, w, hg.nov, hg.noe, hg.pins, 0, [], "degree"),
                   "per_transform": out, "same_as_host": all(v["same"] for v in out.values())},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="zipf4m", choices=sorted(WORKLOADS))
    ap.add_argument("--scale", type=int, default=1, help="divide vertex/net counts (quick runs)")
    ap.add_argument("--passes", type=int, default=0)
    ap.add_argument("--metrics", default="")
    ap.add_argument("--cpu-passes", type=int, default=2,
                    help="cpu_baseline: passes of each metric's schedule (a bounded sample)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--mode", default="refine", choices=["refine", "batch", "serve", "stream", "transforms"],
                    help="refine: the pins/s line; batch / serve: the many-request runners; stream: device vs "
                         "host initial partitions; transforms: device createInverse, thinning, BFS order")
    ap.add_argument("--batch-n", type=int, default=64)
    ap.add_argument("--batch-seed", type=int, default=0)
    ap.add_argument("--batch-passes", type=int, default=8)
    ap.add_argument("--workers", type=int, default=os.cpu_count() or 8)
    ap.add_argument("--rate", type=float, default=20.0)
    ap.add_argument("--duration", type=float, default=5.0)
    ap.add_argument("--serve-vmax", type=int, default=4_000_000)
    ap.add_argument("--budget-gb", type=float, default=150.0)
    ap.add_argument("--slots", type=int, default=32, help="serve: requests admitted at once")
    ap.add_argument("--gpu-slots", type=int, default=4, help="batch / serve: concurrent GPU slots")
    ap.add_argument("--stream-walk", type=int, default=-1,
                    help="stream: 1 / 0 walks changed decisions in the device stream's windows or not "
                         "(default: the library's per-metric choice)")
    args = ap.parse_args()
    if args.mode == "batch":
        run_batch(args)
    elif args.mode == "serve":
        run_serve(args)
    elif args.mode == "stream":
        run_stream(args)
    elif args.mode == "transforms":
        run_transforms(args)
    elif args.impl == "reference":
        run_reference_arm(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
