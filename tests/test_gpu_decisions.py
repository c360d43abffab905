"""Decision-level parity: with the decision log on (fp_set_decision_log), the
grid-wide engine records, for every vertex (every net for CN) of a refine
call's last pass, the decision the reference takes at its turn -- destination,
gain, loss, moved -- and each record equals the oracle's, which restates the
reference's loops (TV/partition.cpp:318-380, MGV/partition.cpp:294-362,
MSRV/partition.cpp:308-400, TM/partition.cpp:330-450, MSM/partition.cpp:
388-518, CN/partition.cpp:262-377).  Refined pass by pass, every pass's
records are compared, on the reference's fixture instances, on uniform16k as
specified and on instances with CTA- and grid-evaluated vertices."""
import numpy as np
import pytest

from conftest import METRICS, golden_cases, load_golden

pytestmark = pytest.mark.gpu
FIELDS = ("dest", "gain", "loss", "moved")


def compare_passes(fp, orc, eng, hg, K, metric, passes, eps=1.05, classes=None, tag=""):
    """Refines one pass at a time with the log on and compares each pass's
    records with the oracle's run of that many passes."""
    with eng.instance(hg, K, metric, eps) as inst:
        if classes:
            inst.set_classes(*classes)
        inst.set_decision_log(True)
        inst.initial_partition()
        for p in range(1, passes + 1):
            inst.refine(1)
            got = inst.decisions()
            want = orc.run_oracle(hg, K, metric, p, eps_factor=eps, records=True)
            for f in FIELDS:
                np.testing.assert_array_equal(got[f], want[f"rec_{f}"], err_msg=f"{tag} {metric} pass {p} {f}")
        np.testing.assert_array_equal(inst.partition(), want["part_vec"], err_msg=f"{tag} {metric}")


@pytest.mark.parametrize("path", golden_cases()[:3], ids=lambda p: p.stem)
@pytest.mark.parametrize("metric", METRICS)
def test_decisions_on_fixture_instances(fp, orc, gpu_engine, path, metric):
    hg, passes, Ks, _ = load_golden(path)
    for K in Ks:
        compare_passes(fp, orc, gpu_engine, hg, K, metric, min(passes, 3), tag=f"{path.stem} K={K}")


@pytest.mark.parametrize("metric", METRICS)
def test_decisions_on_uniform16k(fp, orc, gpu_engine, metric):
    """uniform16k as specified: 16,384 x 16,384 column-net pattern, 2-16 pins
    per net, K = 8, eps factor 1.03, five passes."""
    hg = fp.generate(fp.GenSpec.column_net(16384, 16384, 2, 16, seed=0))
    compare_passes(fp, orc, gpu_engine, hg, 8, metric, 5, eps=1.03, tag="uniform16k")


@pytest.mark.parametrize("metric", METRICS)
def test_decisions_with_cta_and_grid_vertices(fp, orc, gpu_engine, metric):
    """Tiny class bounds put many vertices (nets for CN) in CTA and whole-grid
    evaluation, whose records come from other code than the warps'."""
    hg = fp.generate(fp.GenSpec.zipf(8000, 8000, 2.1, 2, 1500, beta=1.5, weight_rule=1, seed=71))
    compare_passes(fp, orc, gpu_engine, hg, 32, metric, 2, classes=(16, 64), tag="classes")


def test_decision_log_states(fp, gpu_engine):
    """Off by default (FP_ERR_STATE), and the single-CTA walk keeps no records
    (FP_ERR_UNSUPPORTED)."""
    hg = fp.generate(fp.GenSpec.column_net(2048, 2048, 2, 16, seed=5))
    with gpu_engine.instance(hg, 8, "TV") as inst:
        inst.initial_partition()
        inst.refine(1)
        with pytest.raises(fp.FastPartError) as e:
            inst.decisions()
        assert e.value.status == fp.ERR_STATE
        inst.set_decision_log(True)
        inst.set_engine("sequential")
        inst.refine(1)
        with pytest.raises(fp.FastPartError) as e:
            inst.decisions()
        assert e.value.status == fp.ERR_UNSUPPORTED
