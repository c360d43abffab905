"""fp_metrics_noalloc: the six metrics computed from a refinement state that
the caller keeps in its own device memory, with no device memory allocated by
the library -- for callers that cannot have the library allocate (a loop that
has reserved its whole device-memory budget up front, or memory owned by
another allocator, where an extra cudaMalloc / cudaFree pair fragments the
pool and cudaFree waits for the whole device).

It must give exactly the values of fp_metrics (the instance API, which
allocates its scratch) on the same state, call after call: every call shares
one fixed scratch array, so the second call checks that nothing of the first
is left over.  This file is collected last, so a run that stops at the first
failure has already run every other test.
"""
import numpy as np
import pytest

from conftest import METRICS  # noqa: F401


def test_noalloc_rejects_k_above_its_maximum(fp):
    """K above the fixed array's maximum is refused before any CUDA call."""
    rc = fp.lib().fp_metrics_noalloc(fp.NOALLOC_MAX_K + 1, 10, 10, 20, None, None, None, None, None, None, None)
    assert rc == -5   # FP_ERR_UNSUPPORTED


def device_state(torch, hg, st, dev):
    """The state arrays fp_metrics_noalloc reads, as int32 device tensors
    (allocated here by the test, not by the library)."""
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a).astype(np.int32)).to(dev)
    ep_len = st["ep_ends"]                     # lambda(e) per net
    return dict(nptr=t(hg.nptr.astype(np.int64)), src=t(hg.src), part_vec=t(st["part_vec"]), ep_len=t(ep_len),
                ep_part=t(st["ep_parts"]))


def run_noalloc(fp, torch, hg, K, arrs, out, stream):
    fp.metrics_noalloc(K, hg.nov, hg.noe, hg.pins, arrs["nptr"].data_ptr(), arrs["src"].data_ptr(),
                       arrs["part_vec"].data_ptr(), arrs["ep_len"].data_ptr(), arrs["ep_part"].data_ptr(),
                       out.data_ptr(), stream.cuda_stream)
    stream.synchronize()
    return dict(zip(fp.OUTPUT_ORDER, map(int, out.cpu().tolist())))


@pytest.mark.gpu
@pytest.mark.parametrize("metric,K", [("MSV", 64), ("TM", 256), ("TV", 1024)])
def test_noalloc_metrics_equal_fp_metrics_two_calls(fp, gpu_engine, metric, K):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    hg = fp.generate(fp.GenSpec.zipf(20000, 20000, 2.1, 2, 2000, beta=1.5, seed=61))
    with gpu_engine.instance(hg, K, metric) as inst:
        inst.initial_partition()
        st0, want0 = inst.get_state(), inst.metrics()
        inst.refine(2)
        st1, want1 = inst.get_state(), inst.metrics()
    out = torch.full((6,), -7, dtype=torch.int64, device=dev)
    stream = torch.cuda.current_stream(dev)
    # two calls in a row on different states; integer values, so equality is exact
    for st, want in ((st0, want0), (st1, want1)):
        got = run_noalloc(fp, torch, hg, K, device_state(torch, hg, st, dev), out, stream)
        assert got == want, metric
    # and once more on the first state, after the second has used the array
    assert run_noalloc(fp, torch, hg, K, device_state(torch, hg, st0, dev), out, stream) == want0


@pytest.mark.gpu
def test_noalloc_flags_an_inconsistent_state(fp, gpu_engine):
    """A part id outside [0, K) is reported as -1 in all six outputs (the
    kernel skips it instead of indexing past its array)."""
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    hg = fp.generate(fp.GenSpec.zipf(5000, 5000, 2.1, 2, 500, beta=1.5, seed=62))
    K = 32
    with gpu_engine.instance(hg, K, "TV") as inst:
        inst.initial_partition()
        st, want = inst.get_state(), inst.metrics()
    bad = dict(st)
    bad["ep_parts"] = st["ep_parts"].copy()
    bad["ep_parts"][st["ep_starts"][0]] = K + 5
    out = torch.zeros(6, dtype=torch.int64, device=dev)
    stream = torch.cuda.current_stream(dev)
    assert set(run_noalloc(fp, torch, hg, K, device_state(torch, hg, bad, dev), out, stream).values()) == {-1}
    assert run_noalloc(fp, torch, hg, K, device_state(torch, hg, st, dev), out, stream) == want
