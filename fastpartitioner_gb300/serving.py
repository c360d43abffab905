"""Many partition requests on one GPU: a plain per-request loop, a pipelined
batch runner and a continuous serving loop.

A request is one hypergraph, K, metric, balance factor and number of
refinement passes; its result is the refined part vector and the six metric
values, the same as one fp_instance_create / fp_initial_partition / fp_refine /
fp_metrics / fp_get_partition sequence (the reference's partition_gpu(),
TV/partition.h:19, once per request).

* run_plain: that sequence, one request after another.  The streaming initial
  partition runs on the host between the GPU passes, so the GPU idles while it
  runs; it is the baseline the other two are measured against.
* run_pipelined: host work of later requests (building the hypergraph, the
  streaming initial partition, fp_stream_partition) runs on worker threads
  while the GPU refines earlier ones.  Every GPU call is made from the calling
  thread, in request order, on the engine's stream; a request's state enters
  its instance through fp_set_state, which gives the device state that
  fp_initial_partition gives.
* run_concurrent: as run_pipelined, with several GPU slots.  A slot is an
  engine of its own (context and stream) whose grids are sized for a share of
  the SMs (fp_ctx_set_sm_limit) and whose instances live in a device arena
  (fp_ctx_set_arena, no cudaMalloc / cudaFree per request, which would wait
  for the other slots' work); one host thread per slot takes the next prepared
  request, largest first, so small requests run on the device side by side.
* Server: requests arrive over time (Poisson arrivals); each is admitted when
  a preparation slot is free and its device footprint (fp_instance_footprint)
  fits the device-memory budget, is prepared on the workers and refined on the
  GPU as soon as a GPU slot is free (one slot: in arrival order).  Latency is
  arrival to result.

Results do not depend on the runner: a request's part vector and metrics are
those of the request alone.
"""
from __future__ import annotations

import math
import threading
import time
from collections import deque
from concurrent.futures import ThreadPoolExecutor, wait
from dataclasses import dataclass
from typing import Callable, Optional

import numpy as np

from . import ERR_INVALID, ERR_NOMEM, FastPartError, GenSpec, Hypergraph, footprint, generate, stream_partition

METRIC_NAMES = ("TV", "CN", "TM", "MSM", "MSV", "MSRV")


@dataclass
class Request:
    """One partition request: a hypergraph (or the seeded generator spec that
    builds it), K, metric, balance factor and refinement passes.  `arrival` is
    seconds from the start of a serving run."""
    rid: int
    K: int
    metric: str
    passes: int
    eps: float = 1.05
    hg: Optional[Hypergraph] = None
    spec: Optional[GenSpec] = None
    arrival: float = 0.0

    def hypergraph(self) -> Hypergraph:
        return self.hg if self.hg is not None else generate(self.spec)


@dataclass
class Result:
    rid: int
    status: int                          # 0, or the library's negative status code
    part_vec: Optional[np.ndarray] = None
    metrics: Optional[dict] = None
    pins: int = 0
    device_bytes: int = 0
    t_arrival: float = 0.0               # seconds from the start of the run
    t_ready: float = 0.0                 # host preparation done
    t_start: float = 0.0                 # first GPU call
    t_done: float = 0.0                  # result read back
    error: str = ""                      # a failure that was not the library's

    @property
    def latency(self) -> float:
        return self.t_done - self.t_arrival


@dataclass
class Prepared:
    request: Request
    hg: Optional[Hypergraph] = None
    state: Optional[dict] = None
    status: int = 0
    t_ready: float = 0.0
    error: str = ""


def _failed(p: Prepared, e: BaseException) -> None:
    """Marks a preparation failed: the library's status, FP_ERR_NOMEM for a
    host allocation failure, FP_ERR_INVALID for anything else (kept as text)."""
    if isinstance(e, FastPartError):
        p.status = e.status
    else:
        p.status = ERR_NOMEM if isinstance(e, MemoryError) else ERR_INVALID
        p.error = repr(e)
    p.hg = p.state = None


# ---- workloads -------------------------------------------------------------

def mixed_batch(n: int, seed: int = 0, vmin: int = 1_000, vmax: int = 1_000_000, passes: int = 8,
                Ks=(2, 4, 8, 16, 32, 64, 128, 256, 512), metrics=METRIC_NAMES, eps: float = 1.05,
                alpha: float = 2.2, size_hi: int = 2000) -> list:
    """n independent requests of uneven size: vertices log-uniform in
    [vmin, vmax], nets = vertices x U[0.5, 2], net sizes Zipf(alpha) clipped to
    [2, size_hi] with uniformly drawn pins, K and metric uniform over `Ks` and
    `metrics`, unit weights.  Hypergraphs are built when a runner prepares them."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        nov = int(round(math.exp(rng.uniform(math.log(vmin), math.log(vmax)))))
        noe = max(1, int(round(nov * rng.uniform(0.5, 2.0))))
        K = int(rng.choice(np.asarray(Ks)))
        m = str(rng.choice(np.asarray(metrics)))
        spec = GenSpec.zipf(nov, noe, alpha, 2, min(size_hi, nov), seed=int(rng.integers(1 << 31)))
        out.append(Request(rid=i, K=K, metric=m, passes=passes, eps=eps, spec=spec))
    return out


def poisson_arrivals(requests: list, rate: float, seed: int = 1) -> list:
    """Stamps the requests with Poisson arrival times at `rate` per second (in
    request order) and returns them."""
    rng = np.random.default_rng(seed)
    t = 0.0
    for r in requests:
        t += rng.exponential(1.0 / rate)
        r.arrival = t
    return requests


# ---- runners ---------------------------------------------------------------

def _prepare(r: Request, clock: Callable[[], float], t0: float) -> Prepared:
    p = Prepared(request=r)
    try:
        p.hg = r.hypergraph()
        p.state = stream_partition(p.hg, r.K, r.metric, r.eps)
    except Exception as e:      # a failed request is a result, not an abort
        _failed(p, e)
    p.t_ready = clock() - t0
    return p


def _refine_on_gpu(engine, p: Prepared, clock, t0) -> Result:
    """The GPU part of one request, from a host-prepared stream state."""
    r = p.request
    res = Result(rid=r.rid, status=p.status, t_arrival=r.arrival, t_ready=p.t_ready, error=p.error)
    res.t_start = clock() - t0
    if p.status == 0:
        res.pins = p.hg.pins
        try:
            with engine.instance(p.hg, r.K, r.metric, r.eps) as inst:
                res.device_bytes = inst.device_bytes()
                st = p.state
                base = ("part_vec", "ep_starts", "ep_ends", "ep_parts", "ep_cnt")
                inst.set_state(*(st[k] for k in base), **{k: v for k, v in st.items() if k not in base})
                inst.refine(r.passes)
                res.metrics = inst.metrics()
                res.part_vec = inst.partition()
        except Exception as e:      # the serving loop must go on to release what it holds
            q = Prepared(request=r)
            _failed(q, e)
            res.status, res.error = q.status, q.error
            res.part_vec = res.metrics = None
    res.t_done = clock() - t0
    return res


def run_plain(engine, requests: list, clock: Callable[[], float] = time.perf_counter) -> list:
    """One request after another: build, instance, streaming initial partition
    (host), passes (GPU), metrics and part vector, release."""
    t0 = clock()
    out = []
    for r in requests:
        res = Result(rid=r.rid, status=0, t_arrival=max(r.arrival, 0.0))
        delay = r.arrival - (clock() - t0)
        if delay > 0:
            time.sleep(delay)
        res.t_start = clock() - t0
        try:
            hg = r.hypergraph()
            res.pins = hg.pins
            with engine.instance(hg, r.K, r.metric, r.eps) as inst:
                res.device_bytes = inst.device_bytes()
                inst.initial_partition()
                res.t_ready = clock() - t0
                inst.refine(r.passes)
                res.metrics = inst.metrics()
                res.part_vec = inst.partition()
        except Exception as e:
            p = Prepared(request=r)
            _failed(p, e)
            res.status, res.error = p.status, p.error
        res.t_done = clock() - t0
        out.append(res)
    return out


def run_pipelined(engine, requests: list, workers: int = 8, lookahead: Optional[int] = None,
                  clock: Callable[[], float] = time.perf_counter) -> list:
    """Host preparation of up to `lookahead` requests ahead on `workers`
    threads; GPU work in request order on the calling thread."""
    lookahead = lookahead or 2 * workers
    t0 = clock()
    out = []
    with ThreadPoolExecutor(max_workers=workers) as ex:
        futs = deque()
        it = iter(requests)
        for r in it:
            futs.append(ex.submit(_prepare, r, clock, t0))
            if len(futs) >= lookahead:
                break
        while futs:
            p = futs.popleft().result()
            nxt = next(it, None)
            if nxt is not None:
                futs.append(ex.submit(_prepare, nxt, clock, t0))
            out.append(_refine_on_gpu(engine, p, clock, t0))
    return out


ARENA_SLACK = 1 << 16   # fp_instance_footprint + this always fits an arena (256-byte aligned buffers)


def gpu_slots(device: int, slots: int, arena_bytes: int, sm_share: float = 0.8):
    """`slots` engines on `device` for concurrent refinement: each sized for an
    equal part of `sm_share` of the SMs (the grid-wide engines need all CTAs of
    a launch resident; the concurrent grids must fit the device together), each
    with an arena of `arena_bytes`."""
    import torch
    from . import Engine
    sms = torch.cuda.get_device_properties(device).multi_processor_count
    per = max(1, int(sms * sm_share) // slots)
    out = []
    for _ in range(slots):
        e = Engine(device)
        e.set_sm_limit(per)
        e.set_arena(arena_bytes)
        out.append(e)
    return out


def arena_for(requests: list) -> int:
    """An arena size that fits every request of the list."""
    need = 0
    for r in requests:
        hg = r.hypergraph()
        need = max(need, footprint(hg.nov, hg.noe, hg.pins, r.K, r.metric))
    return need + ARENA_SLACK


def _size_key(r: Request) -> int:
    if r.hg is not None:
        return r.hg.pins
    sp = r.spec
    return sp.noe * (sp.size_lo + sp.size_hi) // 2 if sp is not None else 0


def run_concurrent(engines: list, requests: list, workers: int = 8, lookahead: Optional[int] = None,
                   largest_first: bool = True, clock: Callable[[], float] = time.perf_counter) -> list:
    """Host preparation on `workers` threads, GPU work on one thread per engine
    (gpu_slots): every slot takes the next prepared request, the largest first
    unless told otherwise.  Results in request-id order."""
    order = sorted(requests, key=lambda r: -_size_key(r)) if largest_first else list(requests)
    lookahead = lookahead or 2 * max(workers, len(engines))
    t0 = clock()
    out = []
    lock = threading.Lock()
    with ThreadPoolExecutor(max_workers=workers) as ex:
        futs = deque()
        it = iter(order)
        for r in it:
            futs.append(ex.submit(_prepare, r, clock, t0))
            if len(futs) >= lookahead:
                break

        def slot(engine):
            mine = []
            while True:
                with lock:
                    if not futs:
                        return mine
                    f = futs.popleft()
                    nxt = next(it, None)
                    if nxt is not None:
                        futs.append(ex.submit(_prepare, nxt, clock, t0))
                p = f.result()
                mine.append(_refine_on_gpu(engine, p, clock, t0))

        with ThreadPoolExecutor(max_workers=len(engines)) as gpu:
            for part in gpu.map(slot, engines):
                out.extend(part)
    return sorted(out, key=lambda x: x.rid)


class Server:
    """Continuous serving on one GPU.

    Requests are admitted in arrival order once they have arrived and fewer
    than `slots` admitted requests are unfinished.  A worker builds the
    request's hypergraph, then reserves its device footprint
    (fp_instance_footprint, known before the instance exists) against
    `budget_bytes`.  Reservations are taken strictly in admission order, so a
    large request is not overtaken indefinitely.  A request whose footprint
    alone exceeds the budget is rejected with FP_ERR_NOMEM.  The worker then
    runs the streaming initial partition, and the thread that calls run()
    refines the prepared requests on the GPU in admission order, releasing
    each reservation when its result is read back.

    Reserving in admission order cannot deadlock: the executor starts tasks in
    submission order, so the request whose turn it is has started, and the
    reservations it waits for belong to earlier requests, which the GPU
    finishes in that same order."""

    ERR_NOMEM = ERR_NOMEM

    def __init__(self, engine, budget_bytes: int, workers: int = 8, slots: int = 32,
                 clock: Callable[[], float] = time.perf_counter, footprint_fn=footprint):
        # one engine (requests refined in admission order on the calling
        # thread) or a list of GPU slots (gpu_slots: a prepared request goes to
        # the next free slot, and requests overlap on the device)
        self.engines = list(engine) if isinstance(engine, (list, tuple)) else [engine]
        self.engine = self.engines[0]
        self.budget = int(budget_bytes)
        self.workers = workers
        self.slots = slots
        self.clock = clock
        self.footprint_fn = footprint_fn
        self.peak_reserved = 0
        self.peak_admitted = 0

    def run(self, requests: list) -> list:
        reqs = sorted(requests, key=lambda r: (r.arrival, r.rid))
        t0 = self.clock()
        cv = threading.Condition()
        book = {"reserved": 0, "turn": 0}

        def prepare(idx: int, r: Request):
            p = Prepared(request=r)
            need = 0
            try:
                p.hg = r.hypergraph()
                need = self.footprint_fn(p.hg.nov, p.hg.noe, p.hg.pins, r.K, r.metric)
            except Exception as e:  # the turn below is taken whatever happened
                _failed(p, e)
            with cv:
                while book["turn"] != idx or (p.status == 0 and need <= self.budget and
                                              book["reserved"] + need > self.budget):
                    cv.wait()
                if p.status == 0 and need > self.budget:
                    p.status = self.ERR_NOMEM
                if p.status == 0:
                    book["reserved"] += need
                    self.peak_reserved = max(self.peak_reserved, book["reserved"])
                else:
                    need = 0
                book["turn"] += 1
                cv.notify_all()
            if p.status == 0:
                try:
                    p.state = stream_partition(p.hg, r.K, r.metric, r.eps)
                except Exception as e:
                    _failed(p, e)
            p.t_ready = self.clock() - t0
            return p, need

        out = []
        free = deque(self.engines)   # GPU slots not refining
        running = set()              # GPU futures

        def on_gpu(engine, p, need):
            try:
                return _refine_on_gpu(engine, p, self.clock, t0)
            finally:
                p.hg = p.state = None
                with cv:
                    book["reserved"] -= need
                    cv.notify_all()

        def finish(fs):
            for f in fs:
                engine, res = f.result()
                out.append(res)
                free.append(engine)
                running.discard(f)

        with ThreadPoolExecutor(max_workers=self.workers) as ex, \
                ThreadPoolExecutor(max_workers=len(self.engines)) as gpu:
            queue = deque(reqs)      # not yet admitted
            admitted = deque()       # futures, admission order
            idx = 0
            while queue or admitted or running:
                finish([f for f in list(running) if f.done()])
                now = self.clock() - t0
                while queue and queue[0].arrival <= now and len(admitted) + len(running) < self.slots:
                    admitted.append(ex.submit(prepare, idx, queue.popleft()))
                    idx += 1
                    self.peak_admitted = max(self.peak_admitted, len(admitted) + len(running))
                if admitted and admitted[0].done() and free:
                    p, need = admitted.popleft().result()
                    engine = free.popleft()
                    running.add(gpu.submit(lambda e=engine, q=p, n=need: (e, on_gpu(e, q, n))))
                    continue
                # wait for the head's preparation, a GPU slot, or the next
                # arrival if it could be admitted now
                timeout = None
                if queue and len(admitted) + len(running) < self.slots:
                    timeout = max(0.0, queue[0].arrival - (self.clock() - t0))
                pending = list(running) + ([admitted[0]] if admitted and free else [])
                if pending:
                    wait(pending, timeout=timeout, return_when="FIRST_COMPLETED")
                elif timeout:
                    time.sleep(timeout)
            finish(list(running))
        return sorted(out, key=lambda x: x.rid)


def summary(results: list) -> dict:
    """Throughput and latency of a run: partitions/s over the makespan (first
    arrival to last result), pins/s, p50 / p99 latency, failures."""
    ok = [r for r in results if r.status == 0]
    if not results:
        return {"requests": 0}
    span = max(r.t_done for r in results) - min(r.t_arrival for r in results)
    lat = np.array([r.latency for r in ok]) if ok else np.zeros(1)
    return {"requests": len(results), "completed": len(ok), "failed": len(results) - len(ok),
            "makespan_s": span, "partitions_per_s": len(ok) / span if span > 0 else float("inf"),
            "pins_per_s": sum(r.pins for r in ok) / span if span > 0 else float("inf"),
            "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99))}
