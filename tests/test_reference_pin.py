"""The oracle against the reference binary on fresh seeded inputs (runs where the
reference sources were available to build oracle/_ref; skipped elsewhere)."""
import numpy as np
import pytest

from conftest import METRICS

SPECS = [
    ("colnet", lambda fp, s: fp.GenSpec.column_net(1500, 1500, 2, 16, seed=100 + s)),
    ("zipf", lambda fp, s: fp.GenSpec.zipf(1200, 1200, 2.1, 2, 300, beta=1.5, seed=200 + s)),
    ("zipf_uniform_pins", lambda fp, s: fp.GenSpec.zipf(1000, 1000, 1.9, 2, 150, seed=300 + s)),
    ("sparse", lambda fp, s: fp.GenSpec.column_net(600, 600, 2, 3, seed=400 + s)),
]
KS = {"colnet": (2, 6, 24), "zipf": (2, 6, 24), "zipf_uniform_pins": (2, 6, 24), "sparse": (16, 64)}


@pytest.mark.parametrize("name,mk", SPECS, ids=[s[0] for s in SPECS])
@pytest.mark.parametrize("seed", range(4))
def test_oracle_equals_reference(fp, orc, name, mk, seed):
    if not orc.reference_available():
        pytest.skip("reference harness not built (reference sources unavailable)")
    hg = fp.generate(mk(fp, seed))
    for m in METRICS:
        for K in KS[name]:
            o = orc.run_oracle(hg, K, m, 4)
            r = orc.run_reference(hg, K, m, 4)
            assert o["status"] == 0
            np.testing.assert_array_equal(o["part_vec_init"], r["part_vec_init"], err_msg=f"{m} {K}")
            np.testing.assert_array_equal(o["part_vec"], r["part_vec"], err_msg=f"{m} {K}")
            np.testing.assert_array_equal(orc.flat_lists(hg, o["ep_len"], o["ep_part"]), r["lists"],
                                          err_msg=f"{m} {K}")
            assert o["metrics_final"] == r["metrics_final"], (m, K)


# The benchmark's workload shapes at sizes the reference finishes in seconds:
# uniform16k at full size (eps factor 1.05, which the reference fixes,
# TV/partition.cpp:159) and zipf16m_k1024 at 1/64 scale (K = 1024, nets up to
# 100,000 pins).  The six metrics run on threads (each is a subprocess).
SHAPES = [("uniform16k", 1, 5), ("zipf16m_k1024", 64, 2)]


@pytest.mark.parametrize("name,scale,passes", SHAPES, ids=[s[0] for s in SHAPES])
def test_oracle_equals_reference_on_workload_shapes(fp, orc, name, scale, passes):
    if not orc.reference_available():
        pytest.skip("reference harness not built (reference sources unavailable)")
    from concurrent.futures import ThreadPoolExecutor
    import bench
    w = bench.WORKLOADS[name]
    hg = fp.generate(bench.spec_for(fp, w, scale, unit_weights=True))
    K = w["K"]

    def both(m):
        return orc.run_oracle(hg, K, m, passes), orc.run_reference(hg, K, m, passes)

    with ThreadPoolExecutor(len(METRICS)) as ex:
        for m, (o, r) in zip(METRICS, ex.map(both, METRICS)):
            assert o["status"] == 0, m
            np.testing.assert_array_equal(o["part_vec_init"], r["part_vec_init"], err_msg=m)
            np.testing.assert_array_equal(o["part_vec"], r["part_vec"], err_msg=m)
            np.testing.assert_array_equal(orc.flat_lists(hg, o["ep_len"], o["ep_part"]), r["lists"], err_msg=m)
            assert o["metrics_init"] == r["metrics_init"], m
            assert o["metrics_final"] == r["metrics_final"], m
