"""The drop-in boundary's state layout, on the CPU: what the reference's own
partition_gpu() hands to its GPU wrapper after the initial stream (recorded by
the harness's stand-in wrapper, oracle/ref_harness.cpp) is exactly what the
library's host stream writes (fp_stream_partition), array for array, and
fp_check_state -- the check fp_set_state applies -- accepts it as a shim passes
it.  ep_ends is the reference's lambda(e), a count (TV/partition.cpp:1066-1075),
and the reference's own metric code (shared/metric.cpp) reads the library's
state to the oracle's values."""
import numpy as np
import pytest

WRAPPED = ["TV", "CN", "TM", "MSV", "MSRV"]    # MSM has no partition_gpu_wrapper (MSM/msm.cpp:67)
CASES = [("zipf", 3000, 8), ("zipf", 3000, 32), ("colnet", 2048, 16)]


def case(fp, kind, n, seed):
    if kind == "zipf":
        return fp.generate(fp.GenSpec.zipf(n, n, 2.1, 2, 200, beta=1.3, seed=seed))
    return fp.generate(fp.GenSpec.column_net(n, n, 2, 16, seed=seed))


def need_ref(orc, metric="TV"):
    if not orc.reference_available(metric):
        pytest.skip("reference harness not built (reference sources unavailable)")


def shim_optional(w):
    """The optional arrays the INTEGRATION.md shims pass for each wrapper."""
    opt = {"part_sizes": w["psizes"]}
    for k in ("marker", "send", "conn", "msgs"):
        if k in w:
            opt[k] = w[k]
    return opt


@pytest.mark.parametrize("metric", WRAPPED)
@pytest.mark.parametrize("kind,n,K", CASES)
def test_stream_state_is_the_wrappers_input(fp, orc, metric, kind, n, K):
    need_ref(orc, metric)
    hg = case(fp, kind, n, 5 + K)
    w = orc.run_reference_wrapper_state(hg, K, metric)
    s = fp.stream_partition(hg, K, metric)
    for ref_name, name in (("part_vec", "part_vec"), ("psizes", "part_sizes"), ("ep_start", "ep_starts"),
                           ("ep_ends", "ep_ends"), ("ep_parts", "ep_parts"), ("ep_cnt", "ep_cnt")):
        np.testing.assert_array_equal(s[name], w[ref_name], err_msg=f"{metric} {name}")
    for k in ("marker", "send", "conn", "msgs"):
        if k in w:
            np.testing.assert_array_equal(s[k], w[k], err_msg=f"{metric} {k}")
    # the reference's state passes the check fp_set_state applies
    fp.check_state(hg, K, metric, w["part_vec"], w["ep_start"], w["ep_ends"], w["ep_parts"], w["ep_cnt"],
                   **shim_optional(w))


@pytest.mark.parametrize("metric", ["TV", "TM"])
def test_check_state_rejects_what_is_not_the_recount(fp, orc, metric):
    need_ref(orc, metric)
    hg = case(fp, "zipf", 3000, 12)
    K = 8
    w = orc.run_reference_wrapper_state(hg, K, metric)
    base = dict(part_vec=w["part_vec"], ep_starts=w["ep_start"], ep_ends=w["ep_ends"], ep_parts=w["ep_parts"],
                ep_cnt=w["ep_cnt"])
    fp.check_state(hg, K, metric, **base)

    def rejected(**change):
        arrs = {k: v.copy() for k, v in base.items()}
        opt = change.pop("optional", {})
        arrs.update(change)
        with pytest.raises(fp.FastPartError):
            fp.check_state(hg, K, metric, **arrs, **opt)

    starts = w["ep_start"].astype(np.int64)
    rejected(ep_ends=(starts + w["ep_ends"]).astype(np.int32))          # end offsets instead of lambda(e)
    cnt = w["ep_cnt"].copy()
    cnt[starts[1]] += 1
    rejected(ep_cnt=cnt)                                                 # a count off by one
    ends = w["ep_ends"].copy()
    ends[0] += 1
    rejected(ep_ends=ends)                                               # a list longer than its parts
    pv = w["part_vec"].copy()
    pv[0] = K
    rejected(part_vec=pv)                                                # a part id out of range
    sizes = w["psizes"].copy()
    sizes[0] += 1
    rejected(optional={"part_sizes": sizes})                             # sizes that are not the recount
    st = base["ep_starts"].copy()
    st[1] += 1
    rejected(ep_starts=st)                                               # starts that are not the offsets


@pytest.mark.parametrize("metric", ["TV", "CN", "TM", "MSM", "MSV", "MSRV"])
def test_reference_metric_code_reads_the_library_state(fp, orc, metric):
    """shared/metric.cpp's evaluators, handed fp_stream_partition's arrays,
    give the oracle's pre-refinement metrics: the layout is the reference's."""
    if not (orc.REF_DIR / "libref_metrics.so").exists():
        pytest.skip("reference metric library not built")
    hg = case(fp, "zipf", 3000, 21)
    K = 16
    s = fp.stream_partition(hg, K, metric)
    got = orc.reference_metrics(hg, K, s["part_vec"], s["ep_starts"], s["ep_ends"], s["ep_parts"], s["ep_cnt"])
    want = orc.run_oracle(hg, K, metric, 1)["metrics_init"]
    assert got["TV_lambda"] == got["TV"]
    assert {k: got[k] for k in want} == want
