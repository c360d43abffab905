"""Host-side hypergraph handling: the generator and the PaToH-like file format."""
import numpy as np
import pytest

from conftest import ROOT  # noqa: F401


def test_generator_is_deterministic(fp):
    a = fp.generate(fp.GenSpec.column_net(1000, 900, 2, 16, seed=3))
    b = fp.generate(fp.GenSpec.column_net(1000, 900, 2, 16, seed=3))
    c = fp.generate(fp.GenSpec.column_net(1000, 900, 2, 16, seed=4))
    for k in ("vptr", "vnets", "nptr", "npins", "src"):
        np.testing.assert_array_equal(getattr(a, k), getattr(b, k))
    assert not np.array_equal(a.npins, c.npins)


def test_column_net_distribution(fp):
    hg = fp.generate(fp.GenSpec.column_net(5000, 4000, 2, 16, seed=0))
    sizes = np.diff(hg.nptr)
    assert sizes.min() >= 2 and sizes.max() <= 16
    assert abs(sizes.mean() - 9.0) < 0.3
    for e in range(0, hg.noe, 97):
        pins = hg.npins[hg.nptr[e]:hg.nptr[e + 1]]
        assert len(set(pins.tolist())) == len(pins)            # without replacement
        assert hg.src[e] == pins.min()                          # lowest-id pin
        assert np.all(np.diff(pins.astype(np.int64)) > 0)       # sorted pattern
    # vertex -> nets is the transpose, nets ascending per vertex
    for v in range(0, hg.nov, 101):
        nets = hg.vnets[hg.vptr[v]:hg.vptr[v + 1]]
        assert np.all(np.diff(nets.astype(np.int64)) > 0)
        for e in nets:
            assert v in hg.npins[hg.nptr[e]:hg.nptr[e + 1]]


def test_zipf_distribution(fp):
    hg = fp.generate(fp.GenSpec.zipf(20000, 20000, 2.1, 2, 10000, beta=1.5, weight_rule=1, seed=0))
    sizes = np.diff(hg.nptr)
    assert sizes.min() >= 2 and sizes.max() <= 10000
    # clipped Zipf(2.1) from 1: mean about 5
    assert 3.5 < sizes.mean() < 7.0
    deg = np.diff(hg.vptr)
    assert np.array_equal(hg.weights, deg)                      # weight = degree
    assert deg.max() > 20 * deg.mean()                          # heavy-tailed popularity
    assert hg.validate() == 0


def test_patohlike_roundtrip(fp, tmp_path):
    hg = fp.generate(fp.GenSpec.column_net(300, 250, 2, 9, seed=2))
    path = tmp_path / "g.hg"
    fp.write_patohlike(hg, path)
    back = fp.read_patohlike(path, transpose=True)
    assert (back.nov, back.noe) == (hg.nov, hg.noe)
    np.testing.assert_array_equal(back.nptr, hg.nptr)
    np.testing.assert_array_equal(back.npins, hg.npins)
    np.testing.assert_array_equal(back.vptr, hg.vptr)
    np.testing.assert_array_equal(back.vnets, hg.vnets)


def test_patohlike_one_based_and_cache(fp, tmp_path):
    path = tmp_path / "one.hg"
    # 1-based file, 4 vertices, 3 nets
    path.write_text("1 4 3 7\n1 2\n2 3 4\n1 4\n")
    g = fp.read_patohlike(path, transpose=True, write_cache=True)
    assert (g.nov, g.noe, g.pins) == (4, 3, 7)
    np.testing.assert_array_equal(g.npins, [0, 1, 1, 2, 3, 0, 3])
    assert (tmp_path / "one.hg.plbin").exists()
    # the cache wins over the text, as in the reference (hypergraph_rw.cpp:102-106)
    path.write_text("1 4 3 6\n1 2\n2 3\n1 4\n")
    g2 = fp.read_patohlike(path, transpose=True)
    np.testing.assert_array_equal(g2.npins, g.npins)


def test_patohlike_lines_as_vertices(fp, tmp_path):
    path = tmp_path / "sq.hg"
    path.write_text("0 3 3 5\n0 1\n1 2\n0\n")
    g = fp.read_patohlike(path, transpose=False)
    # lines are vertices: vertex 0 has nets {0, 1}, vertex 1 {1, 2}, vertex 2 {0}
    np.testing.assert_array_equal(g.vptr, [0, 2, 4, 5])
    np.testing.assert_array_equal(g.vnets, [0, 1, 1, 2, 0])
    # net -> pins is the inverse with ascending vertices
    np.testing.assert_array_equal(g.nptr, [0, 2, 4, 5])
    np.testing.assert_array_equal(g.npins, [0, 2, 0, 1, 1])


def test_graph_from_vertices_is_the_inverse(fp):
    """Net -> pins built from vertex -> nets equals the original net CSR (pins
    ascending per net), and sources default to the lowest-id pin."""
    hg = fp.generate(fp.GenSpec.zipf(3000, 2500, 2.1, 2, 300, beta=1.5, seed=9))
    g2 = fp.Hypergraph.from_vertices(hg.nov, hg.noe, hg.vptr, hg.vnets, hg.src)
    np.testing.assert_array_equal(g2.nptr, hg.nptr)
    for e in range(0, hg.noe, 97):
        a = np.sort(hg.npins[hg.nptr[e]:hg.nptr[e + 1]])
        np.testing.assert_array_equal(g2.npins[g2.nptr[e]:g2.nptr[e + 1]], a)
    np.testing.assert_array_equal(g2.src, hg.src)
    g3 = fp.Hypergraph.from_vertices(hg.nov, hg.noe, hg.vptr, hg.vnets)
    lo = np.minimum.reduceat(g3.npins, g3.nptr[:-1].astype(np.int64))
    np.testing.assert_array_equal(g3.src, lo)
    with pytest.raises(fp.FastPartError):
        bad = hg.vnets.copy()
        bad[0] = hg.noe
        fp.Hypergraph.from_vertices(hg.nov, hg.noe, hg.vptr, bad)


# The hypergraph and partition of the reference's README (its Figures 1 and 2):
# N1 = {v1, v2, v3}, N2 = {v1, v6, v7, v8}, N3 = {v3, v4, v5}, N4 = {v6, v7};
# P1 = {v1, v2}, P2 = {v3, v4, v5}, P3 = {v6, v7, v8}, K = 4 (one part empty).
# N1 and N2 are cut, N3 and N4 are not: TV = 2, CN = 2.
README_NETS = [[0, 1, 2], [0, 5, 6, 7], [2, 3, 4], [5, 6]]
README_PARTS = [0, 0, 1, 1, 1, 2, 2, 2]


def recount_metrics(hg, part_vec, K):
    """The six metrics of a part vector, from the net -> pins CSR and the sources
    (shared/metric.cpp:3-391, CN/cn.cpp:17-94)."""
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
            "MSM": int(msgs.max()), "MSV": int(send.max()), "MSRV": int((send + recv).max())}


def test_readme_example_metrics():
    import fastpartitioner_gb300 as fp
    nptr = np.cumsum([0] + [len(n) for n in README_NETS]).astype(np.uint32)
    hg = fp.Hypergraph.from_nets(8, nptr, np.concatenate([np.array(n, np.uint32) for n in README_NETS]))
    m = recount_metrics(hg, np.array(README_PARTS), 4)
    assert m["TV"] == 2 and m["CN"] == 2
    # sources are each net's lowest pin: v1, v1, v3, v6; P1 sends to P2 (N1) and P3 (N2)
    assert list(hg.src) == [0, 0, 2, 5]
    assert m == {"TV": 2, "CN": 2, "TM": 2, "MSM": 2, "MSV": 2, "MSRV": 2}
