"""BFS visiting order (the reference's -o 1) on the host: fp_bfs_order against
the reference's own createInverse + bfsFarthest_queue_par x 2 +
bfsOrdering_queue_par (one thread) compiled into oracle/_ref, plus the
properties of a BFS order that hold without the reference."""
import ctypes as C

import numpy as np
import pytest

import fastpartitioner_gb300 as fp
import oracle
from fastpartitioner_gb300 import _ptr, lib


def connected(nov, extra, max_size, seed, shuffle_pins=False):
    """A path of two-pin nets (so every vertex is reached) plus random nets."""
    rng = np.random.default_rng(seed)
    nets = [[i, i + 1] for i in range(nov - 1)]
    for _ in range(extra):
        nets.append(rng.choice(nov, size=int(rng.integers(2, max_size + 1)), replace=False).tolist())
    order = rng.permutation(len(nets))
    nets = [nets[i] for i in order]
    if not shuffle_pins:
        nets = [sorted(n) for n in nets]
    nptr = np.cumsum([0] + [len(n) for n in nets]).astype(np.uint32)
    npins = np.concatenate([np.array(n, np.uint32) for n in nets])
    return fp.Hypergraph.from_nets(nov, nptr, npins)


def raw_bfs(hg, start):
    out = np.empty(hg.nov, np.int32)
    far = np.empty(2, np.int32)
    v = hg.view()
    rc = lib().fp_bfs_order(C.byref(v), int(start), _ptr(out), _ptr(far))
    return rc, int(far[0]), int(far[1]), out


def bfs_levels(hg, root):
    dist = np.full(hg.nov, -1, np.int64)
    dist[root] = 0
    frontier = [root]
    while frontier:
        nxt = []
        for v in frontier:
            for e in hg.vnets[hg.vptr[v]:hg.vptr[v + 1]]:
                for u in hg.npins[hg.nptr[e]:hg.nptr[e + 1]]:
                    if dist[u] < 0:
                        dist[u] = dist[v] + 1
                        nxt.append(int(u))
        frontier = nxt
    return dist


CASES = [
    ("path_plus_random", lambda: connected(400, 300, 6, 1)),
    ("unsorted_pins", lambda: connected(300, 500, 8, 2, shuffle_pins=True)),
    ("dense", lambda: connected(200, 1500, 12, 3)),
    ("zipf_partly_reached", lambda: fp.generate(fp.GenSpec.zipf(3000, 3000, 2.1, 2, 200, beta=1.5, seed=4))),
]


@pytest.mark.parametrize("name,mk", CASES, ids=[c[0] for c in CASES])
def test_bfs_order_matches_the_reference(name, mk):
    if not (oracle.REF_DIR / "ref_bfs").exists():
        pytest.skip("reference BFS harness not built (reference sources unavailable)")
    hg = mk()
    rng = np.random.default_rng(7)
    for start in [0, hg.nov - 1, *rng.integers(0, hg.nov, size=4).tolist()]:
        f1, f2, ref = oracle.run_reference_bfs(hg, start)
        rc, g1, g2, got = raw_bfs(hg, start)
        assert (g1, g2) == (f1, f2), (name, start)
        np.testing.assert_array_equal(got, ref, err_msg=f"{name} start={start}")
        assert rc == (0 if (ref >= 0).all() else -5), (name, start)


@pytest.mark.parametrize("seed", [10, 11])
def test_bfs_order_is_a_breadth_first_permutation(seed):
    hg = connected(500, 400, 7, seed)
    order = hg.bfs_order(3)
    assert sorted(order.tolist()) == list(range(hg.nov))
    dist = bfs_levels(hg, int(order[0]))
    assert (np.diff(dist[order]) >= 0).all(), "levels must not decrease along the order"
    # the root is a farthest vertex from the previous farthest one
    rc, f1, f2, _ = raw_bfs(hg, 3)
    assert rc == 0 and f2 == order[0]
    d1 = bfs_levels(hg, f1)
    assert d1[f2] == d1.max() and f2 == int(np.flatnonzero(d1 == d1.max())[0])


def test_bfs_order_errors():
    hg = fp.Hypergraph.from_nets(6, np.array([0, 2, 4], np.uint32), np.array([0, 1, 2, 3], np.uint32))
    with pytest.raises(fp.FastPartError) as ei:   # vertices 4 and 5 are never reached
        hg.bfs_order(0)
    assert ei.value.status == -5
    rc, _, _, out = raw_bfs(hg, 0)
    assert rc == -5 and (out[2:] == -1).all() and sorted(out[:2].tolist()) == [0, 1]
    ok = connected(50, 10, 4, 0)
    for bad in (-1, 50):
        with pytest.raises(fp.FastPartError):
            ok.bfs_order(bad)
