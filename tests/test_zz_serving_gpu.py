"""Batch and serving runners on the GPU (fastpartitioner_gb300.serving):

* an instance's device allocations equal fp_instance_footprint for its sizes,
  for every metric;
* each request's part vector and metrics are the same alone (the plain
  per-request loop) and in the mix (the pipelined batch runner and the
  serving loop with Poisson arrivals and a device-memory budget).
"""
import pytest

from conftest import METRICS

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("metric", METRICS)
def test_footprint_equals_device_allocations(fp, gpu_engine, metric):
    for spec, K in ((fp.GenSpec.zipf(3000, 2000, 2.1, 2, 300, beta=1.5, seed=61), 16),
                    (fp.GenSpec.column_net(1500, 2500, 2, 9, seed=62), 512)):
        hg = fp.generate(spec)
        with gpu_engine.instance(hg, K, metric) as inst:
            assert inst.device_bytes() == fp.footprint(hg.nov, hg.noe, hg.pins, K, metric), (metric, K)


def test_results_same_alone_and_in_the_mix(fp, gpu_engine):
    from fastpartitioner_gb300 import serving as sv

    def batch():
        return sv.mixed_batch(12, seed=11, vmin=1_000, vmax=30_000, passes=3)

    alone = sv.run_plain(gpu_engine, batch())
    mixed = sv.run_pipelined(gpu_engine, batch(), workers=4)
    reqs = sv.poisson_arrivals(batch(), rate=40.0, seed=4)
    budget = 3 * max(fp.footprint(*(lambda h: (h.nov, h.noe, h.pins))(r.hypergraph()), r.K, r.metric)
                     for r in reqs)
    srv = sv.Server(gpu_engine, budget_bytes=budget, workers=4, slots=4)
    served = srv.run(reqs)
    assert srv.peak_reserved <= budget
    for a, b, c in zip(alone, mixed, served):
        assert a.rid == b.rid == c.rid
        assert a.status == b.status == c.status, a.rid
        if a.status:
            continue
        assert (a.part_vec == b.part_vec).all() and (a.part_vec == c.part_vec).all(), a.rid
        assert a.metrics == b.metrics == c.metrics, a.rid
        assert a.device_bytes == b.device_bytes == c.device_bytes
