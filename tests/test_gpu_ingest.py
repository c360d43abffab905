"""The hypergraph transforms on the device (csrc/fp_ingest.cu) against their
host forms, which the reference pins (tests/test_ingest_reference.py,
tests/test_bfs_order.py, tests/test_cn_thinning.py):

* fp_create_inverse (createInverse, shared/utils.cpp:32-56): the net -> pins
  CSR with each net's pins ascending, at the benchmark's full size (21.35 M
  pins, nets up to 10,000 pins) and on nets of every sort class (up to 32
  pins, up to 4,096, longer; a net of 100,000 pins);
* fp_thin_nets_device (CN/cn.cpp:201-268): every array of the thinned
  hypergraph;
* fp_bfs_order_device (shared/utils.cpp:433-536): the ordering and both
  farthest vertices, and the same FP_ERR_UNSUPPORTED with the same partial
  ordering when a vertex is not reached."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def inverse_reference(nov, noe, vptr, vnets):
    """createInverse in numpy: pins of each net in ascending vertex id."""
    owner = np.repeat(np.arange(nov, dtype=np.uint32), np.diff(vptr.astype(np.int64)))
    order = np.argsort(vnets, kind="stable")
    nptr = np.concatenate([[0], np.cumsum(np.bincount(vnets, minlength=noe))]).astype(np.uint32)
    return nptr, owner[order]


def big_net_case(fp, seed):
    """2,000 nets of 2-40 pins, 200 of 33-4,096, 3 of 5,000-20,000 and one of
    100,000 pins over 150,000 vertices, pins drawn unsorted."""
    rng = np.random.default_rng(seed)
    nov = 150_000
    sizes = np.concatenate([rng.integers(2, 41, 2000), rng.integers(33, 4097, 200), rng.integers(5000, 20001, 3),
                            [100_000]])
    rng.shuffle(sizes)
    nets = [rng.choice(nov, size=int(k), replace=False).astype(np.uint32) for k in sizes]
    nptr = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint32)
    return fp.Hypergraph.from_nets(nov, nptr, np.concatenate(nets))


@pytest.mark.parametrize("case", ["zipf4m", "big_nets", "colnet"])
def test_create_inverse_matches_the_host(fp, gpu_engine, case):
    import bench
    if case == "zipf4m":
        hg = fp.generate(bench.spec_for(fp, bench.WORKLOADS["zipf4m"], 1))
    elif case == "big_nets":
        hg = big_net_case(fp, 5)
    else:
        hg = fp.generate(fp.GenSpec.column_net(20_000, 30_000, 2, 60, seed=6))
    want_ptr, want_pins = inverse_reference(hg.nov, hg.noe, hg.vptr, hg.vnets)
    rp, ci = gpu_engine.create_inverse(hg.nov, hg.noe, hg.vptr, hg.vnets)
    np.testing.assert_array_equal(rp, want_ptr)
    np.testing.assert_array_equal(ci, want_pins)
    # the library's own net -> pins CSR of a hypergraph built from vertices
    hv = fp.Hypergraph.from_vertices(hg.nov, hg.noe, hg.vptr, hg.vnets)
    np.testing.assert_array_equal(rp, hv.nptr)
    np.testing.assert_array_equal(ci, hv.npins)


def test_create_inverse_rejects_bad_input(fp, gpu_engine):
    from fastpartitioner_gb300 import FastPartError
    vptr = np.array([0, 2, 3], np.uint32)
    with pytest.raises(FastPartError):
        gpu_engine.create_inverse(2, 2, vptr, np.array([0, 2, 1], np.uint32))   # net 2 >= noe
    with pytest.raises(FastPartError):
        gpu_engine.create_inverse(2, 3, np.array([0, 3, 2], np.uint32), np.array([0, 1, 2], np.uint32))
    # empty nets are allowed: their ranges are empty
    rp, ci = gpu_engine.create_inverse(2, 4, vptr, np.array([0, 3, 3], np.uint32))
    np.testing.assert_array_equal(rp, [0, 1, 1, 1, 3])
    np.testing.assert_array_equal(ci, [0, 0, 1])


THIN = [
    ("zipf_50k", lambda fp: fp.generate(fp.GenSpec.zipf(50_000, 40_000, 2.0, 2, 3000, beta=1.2, seed=21)), 2, 40),
    ("zipf_50k_loose", lambda fp: fp.generate(fp.GenSpec.zipf(50_000, 40_000, 2.0, 2, 3000, beta=1.2, seed=22)), 8,
     1000),
    ("colnet", lambda fp: fp.generate(fp.GenSpec.column_net(8000, 9000, 2, 30, seed=23)), 1, 12),
]


@pytest.mark.parametrize("name,mk,mean,minp", THIN, ids=[t[0] for t in THIN])
def test_thin_matches_the_host(fp, gpu_engine, name, mk, mean, minp):
    hg = mk(fp)
    want = hg.thin(mean, minp)
    got = gpu_engine.thin(hg, mean, minp)
    assert (got.nov, got.noe, got.pins) == (want.nov, want.noe, want.pins)
    for f in ("vptr", "vnets", "nptr", "npins", "src"):
        np.testing.assert_array_equal(getattr(got, f), getattr(want, f), err_msg=f)


def raw_bfs(fn, *args, nov):
    out = np.empty(nov, np.int32)
    far = np.empty(2, np.int32)
    rc = fn(*args, out.ctypes.data, far.ctypes.data)
    return rc, far.tolist(), out


BFS = [
    ("zipf_200k", lambda fp: fp.generate(fp.GenSpec.zipf(200_000, 200_000, 2.1, 2, 2000, beta=1.2, seed=31))),
    ("colnet_50k", lambda fp: fp.generate(fp.GenSpec.column_net(50_000, 50_000, 2, 20, seed=32))),
    ("big_nets", lambda fp: big_net_case(fp, 33)),
]


@pytest.mark.parametrize("name,mk", BFS, ids=[b[0] for b in BFS])
def test_bfs_order_matches_the_host(fp, gpu_engine, name, mk):
    from fastpartitioner_gb300 import lib
    hg = mk(fp)
    v = hg.view()
    for start in (0, hg.nov // 3, hg.nov - 1):
        rc_h, far_h, ord_h = raw_bfs(lib().fp_bfs_order, C.byref(v), int(start), nov=hg.nov)
        rc_d, far_d, ord_d = raw_bfs(lib().fp_bfs_order_device, gpu_engine._ctx, C.byref(v), int(start), nov=hg.nov)
        assert rc_d == rc_h, (name, start)
        assert far_d == far_h, (name, start)
        np.testing.assert_array_equal(ord_d, ord_h, err_msg=f"{name} start {start}")
