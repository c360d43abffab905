"""Failure detection on the device, with no GPU fault: every grid-wide wait of
the refinement engine is bounded.  A test hook (fp_debug_barrier_fault) makes
the last CTA of the launch leave at one barrier without arriving, as a CTA
that stopped would; the other CTAs' polls run out after a short limit, the
kernel returns, and fp_refine reports FP_ERR_DEVICE_TIMEOUT.  The context stays
usable: after fp_reset_state the same instance refines to the oracle's result."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("metric", ["TV", "MSV", "CN", "TM"])
def test_barrier_timeout_is_reported_and_the_instance_recovers(fp, orc, gpu_engine, metric):
    hg = fp.generate(fp.GenSpec.zipf(6000, 6000, 2.1, 2, 800, beta=1.5, seed=81))
    K, passes = 16, 2
    want = orc.run_oracle(hg, K, metric, passes)
    with gpu_engine.instance(hg, K, metric) as inst:
        inst.initial_partition()
        inst.debug_barrier_fault(leave_at=2, poll_limit=1 << 14)
        t0 = time.perf_counter()
        with pytest.raises(fp.FastPartError) as err:
            inst.refine(passes)
        assert err.value.status == fp.ERR_DEVICE_TIMEOUT, metric
        assert time.perf_counter() - t0 < 30.0
        inst.debug_barrier_fault(0, 0)                   # hook off again
        inst.reset_state()
        inst.refine(passes)
        np.testing.assert_array_equal(inst.partition(), want["part_vec"], err_msg=metric)
        assert inst.metrics() == want["metrics_final"], metric
