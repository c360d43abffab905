"""CN thinning (-m 1 -n MIN -z MEAN) against the reference's own CN driver
(CN/cn.cpp, compiled into oracle/_ref/ref_cn_driver): fp_thin_nets gives the
driver's thinned hypergraph, the CN partition of it (here the oracle, which the
GPU engine equals bit for bit) gives the driver's part vector, and the six
metrics of the full hypergraph under that part vector are the driver's."""
import ctypes
import ctypes.util
import re
import subprocess

import numpy as np
import pytest

import fastpartitioner_gb300 as fp
import oracle

DRIVER = oracle.REF_DIR / "ref_cn_driver"
pytestmark = pytest.mark.skipif(not DRIVER.exists(), reason="reference CN driver not built (reference sources unavailable)")


def driver_sources(hg):
    """The CN driver's sources: rand() % degree per net, glibc's generator
    with its default seed (CN/cn.cpp:186-199)."""
    libc = ctypes.CDLL(ctypes.util.find_library("c"))
    libc.srand(1)
    src = np.empty(hg.noe, np.int32)
    for e in range(hg.noe):
        deg = int(hg.nptr[e + 1] - hg.nptr[e])
        src[e] = hg.npins[hg.nptr[e] + libc.rand() % deg]
    return src


def full_metrics(hg, part_vec, K):
    """The driver's metrics() (CN/cn.cpp:17-94) of the full hypergraph."""
    sizes = np.diff(hg.nptr).astype(np.int64)
    net_of_pin = np.repeat(np.arange(hg.noe), sizes)
    key = np.unique(net_of_pin * K + part_vec[hg.npins])
    net, part = key // K, key % K
    lam = np.bincount(net, minlength=hg.noe)
    spart = part_vec[hg.src][net]
    other = part != spart
    send = np.bincount(spart[other], minlength=K)
    recv = np.bincount(part[other], minlength=K)
    pairs = np.unique(spart[other] * K + part[other])
    msgs = np.bincount(pairs // K, minlength=K)
    return {"TV": int(np.sum(lam - 1)), "CN": int(np.sum(lam > 1)), "TM": int(pairs.size),
            "MGM": int(msgs.max()), "MGV": int(send.max()), "MGAV": int((send + recv).max())}


CASES = [
    ("zipf_a", dict(nov=3000, noe=2000, alpha=2.1, hi=80, beta=1.2, seed=5), 8, 2, 2, 10),
    ("zipf_b", dict(nov=4000, noe=3000, alpha=1.8, hi=200, beta=1.0, seed=6), 16, 3, 3, 25),
    ("zipf_c", dict(nov=2500, noe=1800, alpha=2.5, hi=40, beta=1.5, seed=7), 4, 1, 1, 6),
]


@pytest.mark.parametrize("name,spec,K,passes,mean,minp", CASES, ids=[c[0] for c in CASES])
def test_cn_thinning_matches_the_reference_driver(tmp_path, name, spec, K, passes, mean, minp):
    g0 = fp.generate(fp.GenSpec.zipf(spec["nov"], spec["noe"], spec["alpha"], 2, spec["hi"], beta=spec["beta"],
                                     seed=spec["seed"]))
    path = tmp_path / "g.hg"
    fp.write_patohlike(g0, path)
    res = subprocess.run([str(DRIVER), "-f", str(path), "-k", str(K), "-r", "1", "-i", str(passes), "-m", "1",
                          "-n", str(minp), "-z", str(mean)], capture_output=True, text=True, timeout=600,
                         cwd=tmp_path)
    assert res.returncode == 0, res.stdout[-2000:] + res.stderr[-2000:]
    out = res.stdout
    m = re.search(r"Nov = (\d+)\s+noe = (\d+)\s+pins = (\d+)", out)
    ref_part = np.loadtxt(tmp_path / f"g.hg.fastpart.{K}", dtype=np.int64).astype(np.int32)
    block = out[out.rindex("Metrics Computed"):]
    ref_metrics = {k: int(v) for k, v in re.findall(r"^(TV|CN|TM|MGM|MGV|MGAV): (-?\d+)$", block, re.M)}

    hg = fp.read_patohlike(path, transpose=True)
    hg.src = driver_sources(hg)
    thin = hg.thin(mean, minp)
    assert (thin.nov, thin.noe, thin.pins) == tuple(int(x) for x in m.groups()), name
    o = oracle.run_oracle(thin, K, "CN", passes)
    assert o["status"] == 0
    np.testing.assert_array_equal(o["part_vec"], ref_part, err_msg=name)
    assert full_metrics(hg, o["part_vec"], K) == ref_metrics, name


def test_thin_keeps_order_pins_and_sources():
    hg = fp.generate(fp.GenSpec.zipf(1500, 1000, 2.0, 2, 50, beta=1.2, seed=9))
    t = hg.thin(2, 8)
    sizes = np.diff(hg.nptr)
    mean = np.float64(np.float32(hg.pins) / np.float32(hg.noe))
    kept = np.flatnonzero((sizes < 2 * mean) & (sizes < 8))
    assert t.noe == kept.size and t.nov == hg.nov
    for new, e in enumerate(kept[:200]):
        np.testing.assert_array_equal(t.npins[t.nptr[new]:t.nptr[new + 1]], hg.npins[hg.nptr[e]:hg.nptr[e + 1]])
        assert t.src[new] == hg.src[e]
    renum = -np.ones(hg.noe, np.int64)
    renum[kept] = np.arange(kept.size)
    for v in range(0, hg.nov, 37):
        nets = renum[hg.vnets[hg.vptr[v]:hg.vptr[v + 1]]]
        np.testing.assert_array_equal(t.vnets[t.vptr[v]:t.vptr[v + 1]], nets[nets >= 0])
