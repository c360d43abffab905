"""Host logic of the batch and serving runners (fastpartitioner_gb300.serving),
on CPU with a stand-in engine: every GPU call made from the calling thread,
one instance alive at a time, results per request the same alone and in the
mix, admission within the device-memory budget, arrival order kept."""
import threading

import numpy as np
import pytest

import fastpartitioner_gb300 as fp
from fastpartitioner_gb300 import serving as sv


class FakeInstance:
    """Stands in for an engine instance: the host stream as the state, an
    identity refinement, metrics recounted with numpy."""

    def __init__(self, eng, hg, K, metric, eps):
        self.eng, self.hg, self.K, self.metric, self.eps = eng, hg, K, metric, eps
        self.pv = None
        eng.calls.append(("create", threading.get_ident()))
        eng.alive += 1
        eng.max_alive = max(eng.max_alive, eng.alive)

    def _call(self, what):
        self.eng.calls.append((what, threading.get_ident()))

    def device_bytes(self):
        self._call("bytes")
        return fp.footprint(self.hg.nov, self.hg.noe, self.hg.pins, self.K, self.metric)

    def initial_partition(self):
        self._call("initial")
        self.pv = fp.stream_partition(self.hg, self.K, self.metric, self.eps)["part_vec"]

    def set_state(self, part_vec, ep_starts, ep_ends, ep_parts, ep_cnt, **optional):
        self._call("set_state")
        assert set(optional) <= {"part_sizes", "marker", "send", "recv", "conn", "msgs"}
        self.pv = np.array(part_vec)

    def refine(self, passes):
        self._call("refine")

    def metrics(self):
        self._call("metrics")
        sizes = np.diff(self.hg.nptr).astype(np.int64)
        net = np.repeat(np.arange(self.hg.noe), sizes)
        lam = np.bincount(np.unique(net * self.K + self.pv[self.hg.npins]) // self.K, minlength=self.hg.noe)
        return {"TV": int(np.sum(lam - 1)), "CN": int(np.sum(lam > 1))}

    def partition(self):
        self._call("partition")
        return self.pv.copy()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.eng.alive -= 1
        self._call("close")


class FakeEngine:
    def __init__(self, device=0):
        self.calls, self.alive, self.max_alive = [], 0, 0

    def close(self):
        pass

    def instance(self, hg, K, metric, eps=1.05):
        return FakeInstance(self, hg, K, metric, eps)


def small_batch(n, seed=0):
    return sv.mixed_batch(n, seed=seed, vmin=200, vmax=4000, passes=3, Ks=(2, 4, 8, 16, 32))


def test_mixed_batch_shapes():
    reqs = sv.mixed_batch(64, seed=3)
    assert [r.rid for r in reqs] == list(range(64))
    for r in reqs:
        assert 1000 <= r.spec.nov <= 1_000_000
        assert 0.5 * r.spec.nov - 1 <= r.spec.noe <= 2 * r.spec.nov + 1
        assert r.K in (2, 4, 8, 16, 32, 64, 128, 256, 512) and r.metric in sv.METRIC_NAMES
        assert r.spec.size_alpha == 2.2 and r.spec.size_hi == min(2000, r.spec.nov)
    again = sv.mixed_batch(64, seed=3)
    assert [(r.K, r.metric, r.spec.nov, r.spec.seed) for r in reqs] == \
           [(r.K, r.metric, r.spec.nov, r.spec.seed) for r in again]
    arr = [r.arrival for r in sv.poisson_arrivals(reqs, rate=200.0, seed=1)]
    assert all(b > a for a, b in zip(arr, arr[1:]))
    assert 0.15 < arr[-1] < 0.5          # 64 arrivals at 200/s


def test_pipelined_equals_plain_and_keeps_gpu_calls_on_the_caller():
    reqs = small_batch(24)
    plain_eng, pipe_eng = FakeEngine(), FakeEngine()
    plain = sv.run_plain(plain_eng, reqs)
    pipe = sv.run_pipelined(pipe_eng, reqs, workers=4)
    me = threading.get_ident()
    for eng in (plain_eng, pipe_eng):
        assert {tid for _, tid in eng.calls} == {me}
        assert eng.max_alive == 1
    assert [r.rid for r in pipe] == [r.rid for r in reqs]
    for a, b in zip(plain, pipe):
        assert a.status == b.status == 0
        np.testing.assert_array_equal(a.part_vec, b.part_vec)
        assert a.metrics == b.metrics and a.pins == b.pins
        assert b.t_ready <= b.t_start <= b.t_done
    # the pipelined runner loads the host stream's state; the plain one streams itself
    assert {c for c, _ in pipe_eng.calls} >= {"set_state"} and "initial" not in {c for c, _ in pipe_eng.calls}


def test_server_admission_budget_order_and_results():
    reqs = sv.poisson_arrivals(small_batch(30, seed=5), rate=400.0, seed=2)
    alone = {r.rid: r for r in sv.run_plain(FakeEngine(), [sv.Request(**{**q.__dict__, "arrival": 0.0})
                                                             for q in reqs])}
    foot = {r.rid: fp.footprint(*(lambda h: (h.nov, h.noe, h.pins))(r.hypergraph()), r.K, r.metric) for r in reqs}
    vals = sorted(foot.values())
    assert vals[-1] > vals[-2]
    budget = (vals[-1] + vals[-2]) // 2    # every request but the largest fits
    srv = sv.Server(FakeEngine(), budget_bytes=budget, workers=4, slots=6)
    out = srv.run(reqs)
    assert [r.rid for r in out] == sorted(foot)
    assert srv.peak_reserved <= budget and srv.peak_admitted <= 6
    for r in out:
        if foot[r.rid] > budget:
            assert r.status == sv.Server.ERR_NOMEM and r.part_vec is None
            continue
        assert r.status == 0
        np.testing.assert_array_equal(r.part_vec, alone[r.rid].part_vec)
        assert r.metrics == alone[r.rid].metrics
        assert r.t_arrival <= r.t_ready <= r.t_start <= r.t_done and r.latency >= 0
    assert sum(r.status == sv.Server.ERR_NOMEM for r in out) == 1
    served = sorted((r for r in out if r.status == 0), key=lambda r: (r.t_arrival, r.rid))
    assert all(a.t_done <= b.t_done for a, b in zip(served, served[1:]))   # arrival order kept
    s = sv.summary(out)
    assert s["requests"] == 30 and s["completed"] + s["failed"] == 30
    assert s["p50_latency_s"] <= s["p99_latency_s"] and s["partitions_per_s"] > 0


def test_server_tight_budget_serialises_without_deadlock():
    """A budget that fits one request at a time: every request still completes,
    in arrival order, with one reservation held at a time."""
    reqs = sv.poisson_arrivals(small_batch(12, seed=7), rate=1000.0, seed=3)
    foot = [fp.footprint(*(lambda h: (h.nov, h.noe, h.pins))(r.hypergraph()), r.K, r.metric) for r in reqs]
    srv = sv.Server(FakeEngine(), budget_bytes=max(foot), workers=4, slots=8)
    out = srv.run(reqs)
    assert all(r.status == 0 for r in out) and len(out) == 12
    assert srv.peak_reserved <= max(foot)


def test_footprint_is_monotone_and_validates():
    base = fp.footprint(10_000, 10_000, 50_000, 64, "TV")
    assert base > 0
    assert fp.footprint(20_000, 10_000, 50_000, 64, "TV") > base
    assert fp.footprint(10_000, 10_000, 90_000, 64, "TV") > base
    assert fp.footprint(10_000, 10_000, 50_000, 128, "TV") > base
    # TM/MSM hold K x K counts and masks; the LDG metrics hold move records per pin
    assert fp.footprint(1000, 1000, 3000, 1024, "TM") > fp.footprint(1000, 1000, 3000, 1024, "CN") + 4 * 1024 * 1024
    assert fp.footprint(1000, 1000, 10_000_000, 8, "MSV") > fp.footprint(1000, 1000, 10_000_000, 8, "TM")
    for bad in ((0, 10, 10, 8, "TV"), (10, 10, 10, 1, "TV"), (10, 10, 10, 5000, "TV"), (10, 10, -1, 8, "TV")):
        with pytest.raises(fp.FastPartError):
            fp.footprint(*bad)


def test_bench_batch_and_serve_lines(monkeypatch, capsys):
    """bench.py --mode batch / serve end to end with the stand-in engine: one
    JSON line each, results the same alone and in the mix."""
    import json
    import sys
    from pathlib import Path
    import torch
    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    import bench
    monkeypatch.setattr(fp, "Engine", FakeEngine)
    monkeypatch.setattr(torch.cuda, "set_device", lambda d: None)
    orig = sv.mixed_batch
    monkeypatch.setattr(sv, "mixed_batch", lambda n, seed=0, vmax=1_000_000, passes=8, **kw:
                        orig(n, seed=seed, vmin=200, vmax=4000, passes=passes, Ks=(2, 4, 8, 16, 32)))
    monkeypatch.setattr(sv, "gpu_slots", lambda device, n, arena, **kw: [FakeEngine() for _ in range(n)])
    args = bench.argparse.Namespace(batch_n=10, batch_seed=0, batch_passes=2, workers=3, warmup=1, rate=200.0,
                                    duration=0.05, serve_vmax=4000, budget_gb=1.0, slots=4, gpu_slots=2)
    bench.run_batch(args)
    bench.run_serve(args)
    lines = [json.loads(x) for x in capsys.readouterr().out.strip().splitlines()]
    assert len(lines) == 2
    b, v = lines
    assert b["unit"] == "partitions/s" and b["value"] > 0 and b["config"]["same_alone_and_in_the_mix"] is True
    assert b["config"]["plain_loop"]["completed"] == 10
    assert v["unit"] == "s" and v["higher_is_better"] is False and v["config"]["same_alone_and_in_the_mix"] is True
    assert v["config"]["served"]["requests"] == 10 and v["config"]["peak_reserved_gb"] <= 1.0
    assert b["config"]["gpu_slots"] == 2 and v["config"]["gpu_slots"] >= 1


class BrokenRequest(sv.Request):
    def hypergraph(self):
        raise ValueError("no payload")


@pytest.mark.parametrize("runner", ["plain", "pipelined", "server"])
def test_a_failing_request_is_a_result(runner):
    """A request whose hypergraph cannot be built fails alone: its result
    carries FP_ERR_INVALID and the error text, the others complete, and the
    serving loop's turn order does not stall on it."""
    reqs = sv.poisson_arrivals(small_batch(9, seed=8), rate=500.0, seed=5)
    bad = reqs[3]
    reqs[3] = BrokenRequest(**bad.__dict__)
    eng = FakeEngine()
    if runner == "plain":
        out = sv.run_plain(eng, reqs)
    elif runner == "pipelined":
        out = sv.run_pipelined(eng, reqs, workers=3)
    else:
        out = sv.Server(eng, budget_bytes=1 << 40, workers=3, slots=4).run(reqs)
    by = {r.rid: r for r in out}
    assert len(by) == 9
    assert by[bad.rid].status == fp.ERR_INVALID and "no payload" in by[bad.rid].error
    assert all(r.status == 0 for rid, r in by.items() if rid != bad.rid)


class FailingRefineEngine(FakeEngine):
    """refine() fails for one K: a GPU-side failure of one request."""

    def instance(self, hg, K, metric, eps=1.05):
        inst = super().instance(hg, K, metric, eps)
        if K == 16:
            def boom(passes):
                raise RuntimeError("device lost")
            inst.refine = boom
        return inst


def test_gpu_side_failure_releases_the_request():
    reqs = sv.poisson_arrivals(small_batch(10, seed=9), rate=800.0, seed=6)
    foot = max(fp.footprint(*(lambda h: (h.nov, h.noe, h.pins))(r.hypergraph()), r.K, r.metric) for r in reqs)
    out = sv.Server(FailingRefineEngine(), budget_bytes=foot, workers=3, slots=4).run(reqs)
    assert len(out) == 10
    for r, q in zip(out, sorted(reqs, key=lambda x: x.rid)):
        if q.K == 16:
            assert r.status == fp.ERR_INVALID and "device lost" in r.error and r.part_vec is None
        else:
            assert r.status == 0


def test_concurrent_slots_equal_plain_one_instance_per_slot():
    """run_concurrent: every slot (engine) makes its calls from one thread of
    its own and holds one instance at a time; results equal the plain loop's."""
    reqs = small_batch(30, seed=7)
    plain = sv.run_plain(FakeEngine(), reqs)
    engines = [FakeEngine() for _ in range(3)]
    conc = sv.run_concurrent(engines, reqs, workers=4)
    assert [r.rid for r in conc] == [r.rid for r in reqs]
    for a, b in zip(plain, conc):
        assert a.status == b.status == 0
        np.testing.assert_array_equal(a.part_vec, b.part_vec)
        assert a.metrics == b.metrics
    used = [e for e in engines if e.calls]
    assert len(used) >= 2
    for e in used:
        assert len({tid for _, tid in e.calls}) == 1 and e.max_alive == 1
    assert len({e.calls[0][1] for e in used}) == len(used)   # one thread per slot


def test_server_with_gpu_slots_keeps_budget_and_results():
    reqs = sv.poisson_arrivals(small_batch(24, seed=9), rate=300.0, seed=3)
    alone = {r.rid: r for r in sv.run_plain(FakeEngine(), [sv.Request(**{**q.__dict__, "arrival": 0.0})
                                                             for q in reqs])}
    foot = [fp.footprint(*(lambda h: (h.nov, h.noe, h.pins))(r.hypergraph()), r.K, r.metric) for r in reqs]
    budget = 3 * max(foot)
    engines = [FakeEngine() for _ in range(3)]
    srv = sv.Server(engines, budget_bytes=budget, workers=4, slots=6)
    out = srv.run(reqs)
    assert srv.peak_reserved <= budget
    assert [r.rid for r in out] == sorted(r.rid for r in reqs)
    for r in out:
        assert r.status == 0
        np.testing.assert_array_equal(r.part_vec, alone[r.rid].part_vec)
        assert r.metrics == alone[r.rid].metrics
        assert r.t_arrival <= r.t_start <= r.t_done
    for e in engines:
        assert e.max_alive <= 1
