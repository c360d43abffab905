"""The streaming initial partitions on the device (csrc/fp_stream.cu) against
the host streams (fp_stream_partition, the restatement of
TV/partition.cpp:207-264, MGV/partition.cpp:122-189, MSRV/partition.cpp:
123-196, CN/partition.cpp:132-221, TM/partition.cpp:87-250 and
MSM/partition.cpp:146-309 that the oracle and the reference's own outputs
pin): the whole fp_state -- part vector, every net's ordered (part, count)
list, part sizes, TV's marker, the MSV / MSRV volumes, the TM / MSM K x K
connection counts and messages -- bit for bit.

The device stream runs when every vertex without nets weighs 0 (vertex weight =
degree) and K <= 1024; the cases cover vertices without nets before, between
and after the others, vertices in 4096 nets or more (a window of their own,
placed by the whole grid, back to back), and K from 4 to 1024.  Refinement
after the device stream is checked against the oracle as well."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STREAMED = ("TV", "MSV", "MSRV", "CN", "TM", "MSM")
FIELDS = ("part_vec", "ep_ends", "ep_parts", "ep_cnt", "part_sizes", "marker", "send", "recv")
MSG_FIELDS = ("conn", "msgs")


def fields(metric):
    return FIELDS + (MSG_FIELDS if metric in ("TM", "MSM") else ())


def degree_weighted(hg):
    hg.weights = np.ascontiguousarray(np.diff(hg.vptr).astype(np.int32))
    return hg


def heavy_case(fp, seed):
    """30,000 vertices, 9,000 nets: vertex 5 in every net, vertices 6 and 100
    in the even / odd nets (4,500 each), plus 10-30 random pins from vertices
    200 and up; vertices 0-4, 7-99 and 101-199 have no nets."""
    rng = np.random.default_rng(seed)
    nets = []
    for e in range(9000):
        k = int(rng.integers(10, 31))
        others = rng.choice(np.arange(200, 30000), size=k, replace=False)
        nets.append(np.concatenate([[5, 6 if e % 2 == 0 else 100], others]).astype(np.uint32))
    nptr = np.cumsum([0] + [len(n) for n in nets]).astype(np.uint32)
    return degree_weighted(fp.Hypergraph.from_nets(30000, nptr, np.concatenate(nets)))


CASES = [
    ("zipf20k_K8", lambda fp: fp.generate(fp.GenSpec.zipf(20000, 15000, 2.0, 2, 400, beta=1.0, weight_rule=1,
                                                          seed=81)), 8),
    ("zipf20k_K256", lambda fp: fp.generate(fp.GenSpec.zipf(20000, 15000, 2.0, 2, 400, beta=1.0, weight_rule=1,
                                                            seed=82)), 256),
    ("zipf60k_K64", lambda fp: fp.generate(fp.GenSpec.zipf(60000, 60000, 1.9, 2, 3000, beta=1.5, weight_rule=1,
                                                           seed=83)), 64),
    ("colnet_degw_K1024", lambda fp: degree_weighted(fp.generate(fp.GenSpec.column_net(6000, 6000, 2, 30,
                                                                                        seed=84))), 1024),
    ("heavy30k_K16", lambda fp: heavy_case(fp, 85), 16),
    ("heavy30k_K4", lambda fp: heavy_case(fp, 86), 4),
]


def device_state(eng, hg, K, metric, where="device"):
    with eng.instance(hg, K, metric) as inst:
        inst.set_stream(where)
        inst.initial_partition()
        on_dev = inst.streamed_on_device()
        st = inst.get_state()
    return on_dev, st


@pytest.mark.parametrize("name,mk,K", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("metric", STREAMED)
def test_device_stream_matches_host_stream(fp, gpu_engine, name, mk, K, metric):
    hg = mk(fp)
    want = fp.stream_partition(hg, K, metric)
    on_dev, got = device_state(gpu_engine, hg, K, metric)
    assert on_dev, "the instance qualifies for the device stream"
    for f in fields(metric):
        np.testing.assert_array_equal(got[f], want[f], err_msg=f"{name} {metric} {f}")
    np.testing.assert_array_equal(got["ep_starts"], hg.nptr[:-1].astype(np.int32))
    host_dev, host = device_state(gpu_engine, hg, K, metric, where="host")
    assert not host_dev
    for f in fields(metric):
        np.testing.assert_array_equal(host[f], want[f], err_msg=f"host {name} {metric} {f}")


@pytest.mark.parametrize("metric", STREAMED)
def test_refinement_after_the_device_stream(fp, orc, gpu_engine, metric):
    """initial_partition on the device, three passes, reset_state (the copy of
    the device stream's result kept on the host), three passes again: both
    runs equal the oracle's."""
    hg = heavy_case(fp, 87)
    K, passes = 16, 3
    o = orc.run_oracle(hg, K, metric, passes)
    assert o["status"] == 0
    with gpu_engine.instance(hg, K, metric) as inst:
        inst.set_stream("device")
        inst.initial_partition()
        assert inst.streamed_on_device()
        np.testing.assert_array_equal(inst.partition(), o["part_vec_init"])
        for _ in range(2):
            inst.refine(passes)
            np.testing.assert_array_equal(inst.partition(), o["part_vec"], err_msg=metric)
            assert inst.metrics() == o["metrics_final"], metric
            inst.reset_state()
            np.testing.assert_array_equal(inst.partition(), o["part_vec_init"])


def test_device_stream_only_where_it_qualifies(fp, gpu_engine):
    """Unit weights with vertices without nets and K above 1024 stream on the
    host; by default CN, TM and MSM do too."""
    unit = fp.generate(fp.GenSpec.zipf(5000, 4000, 2.0, 2, 200, beta=1.0, seed=88))
    assert (np.diff(unit.vptr) == 0).any()
    degw = fp.generate(fp.GenSpec.zipf(5000, 4000, 2.0, 2, 200, beta=1.0, weight_rule=1, seed=88))
    for hg, K, metric, dev, where in ((unit, 8, "TV", False, "device"), (degw, 2048, "MSV", False, "device"),
                                      (degw, 8, "CN", True, "device"), (degw, 8, "CN", False, "auto"),
                                      (degw, 8, "TM", True, "device"), (degw, 8, "TM", False, "auto"),
                                      (degw, 16, "MSM", True, "device"), (degw, 8, "MSRV", True, "auto")):
        with gpu_engine.instance(hg, K, metric) as inst:
            inst.set_stream(where)
            inst.initial_partition()
            assert inst.streamed_on_device() == dev, (K, metric)
            if not dev:
                continue
            st = inst.get_state()
        want = fp.stream_partition(hg, K, metric)
        for f in fields(metric):
            np.testing.assert_array_equal(st[f], want[f], err_msg=f)


@pytest.mark.parametrize("metric", ("TV", "CN", "MSRV"))
def test_stream_walk_setting_leaves_the_result(fp, gpu_engine, metric):
    """fp_set_stream_walk (walk the changed decisions in a window, or end the
    window at the first) is tuning only: the same state either way."""
    hg = heavy_case(fp, 89)
    states = []
    for walk in (0, 1):
        with gpu_engine.instance(hg, 16, metric) as inst:
            inst.set_stream("device")
            inst.set_stream_walk(bool(walk))
            inst.initial_partition()
            assert inst.streamed_on_device()
            states.append(inst.get_state())
    for f in fields(metric):
        np.testing.assert_array_equal(states[0][f], states[1][f], err_msg=f"{metric} {f}")


@pytest.mark.parametrize("metric", ("TV", "MSV", "MSRV"))
def test_window_setting_leaves_the_refinement(fp, orc, gpu_engine, metric):
    """fp_set_window (window length after a cut) is tuning only."""
    hg = fp.generate(fp.GenSpec.zipf(20000, 15000, 2.0, 2, 400, beta=1.0, weight_rule=1, seed=90))
    o = orc.run_oracle(hg, 64, metric, 3)
    assert o["status"] == 0
    with gpu_engine.instance(hg, 64, metric) as inst:
        inst.initial_partition()
        for wmin, grow in ((0, 2), (256, 4), (4096, 1)):
            inst.reset_state()
            inst.set_window(wmin, grow)
            inst.refine(3)
            np.testing.assert_array_equal(inst.partition(), o["part_vec"], err_msg=f"{metric} {wmin} {grow}")
            assert inst.metrics() == o["metrics_final"], (metric, wmin, grow)
