"""The streaming initial partitions on the host (fp_stream_partition, the same
code fp_initial_partition runs): against the reference's own initial part
vectors (golden fixtures) and against the oracle's full initial state (part
vector, ordered lists, counts, sizes, volumes / messages)."""
import numpy as np
import pytest

import fastpartitioner_gb300 as fp
import oracle
from conftest import METRICS, golden_cases, load_golden


@pytest.mark.parametrize("path", golden_cases(), ids=lambda p: p.stem)
def test_stream_matches_reference_fixtures(path):
    hg, passes, Ks, z = load_golden(path)
    for m in METRICS:
        for K in Ks:
            s = fp.stream_partition(hg, K, m)
            np.testing.assert_array_equal(s["part_vec"], z[f"{m}_{K}_part_vec_init"], err_msg=f"{m}_{K}")


CASES = [
    ("zipf_5k_K64", lambda: fp.generate(fp.GenSpec.zipf(5000, 5000, 2.1, 2, 1000, beta=1.5, seed=13)), 64, 1.05, False),
    ("colnet_4k_K8", lambda: fp.generate(fp.GenSpec.column_net(4096, 4096, 2, 16, seed=11)), 8, 1.05, False),
    ("zipf_3k_K16_weighted", lambda: fp.generate(fp.GenSpec.zipf(3000, 3000, 2.1, 2, 500, beta=1.5, weight_rule=1,
                                                                   seed=21)), 16, 1.03, True),
]


@pytest.mark.parametrize("name,mk,K,eps,shuffle", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("metric", METRICS)
def test_stream_matches_oracle(name, mk, K, eps, shuffle, metric):
    hg = mk()
    if shuffle:
        hg.ordering = np.random.default_rng(5).permutation(hg.nov).astype(np.int32)
    s = fp.stream_partition(hg, K, metric, eps)
    o = oracle.run_oracle(hg, K, metric, 0, eps_factor=eps)
    assert o["status"] == 0
    np.testing.assert_array_equal(s["part_vec"], o["part_vec_init"])
    np.testing.assert_array_equal(s["ep_starts"], hg.nptr[:-1].astype(np.int32))
    np.testing.assert_array_equal(s["ep_ends"], o["ep_len_init"])   # lambda(e), the reference's layout
    np.testing.assert_array_equal(s["ep_parts"], o["ep_part_init"])
    np.testing.assert_array_equal(s["ep_cnt"], o["ep_cnt_init"])
    w = np.ones(hg.nov, np.int64) if hg.weights is None else hg.weights.astype(np.int64)
    np.testing.assert_array_equal(s["part_sizes"], np.bincount(s["part_vec"], weights=w, minlength=K))


def test_stream_rejects_bad_arguments():
    hg = fp.generate(fp.GenSpec.column_net(256, 256, 2, 8, seed=1))
    for K, metric, eps in ((1, "TV", 1.05), (5000, "TV", 1.05), (8, 7, 1.05), (8, "TV", 0.0)):
        with pytest.raises((fp.FastPartError, ValueError)):
            fp.stream_partition(hg, K, metric, eps)


MORE = [
    ("colnet_2k_K3", lambda: fp.generate(fp.GenSpec.column_net(2048, 2048, 2, 12, seed=31)), 3, 1.05),
    ("zipf_8k_K100_weighted", lambda: fp.generate(fp.GenSpec.zipf(8000, 6000, 2.1, 2, 900, beta=1.5, weight_rule=1,
                                                                    seed=32)), 100, 1.05),
    ("zipf_6k_K1000", lambda: fp.generate(fp.GenSpec.zipf(6000, 5000, 1.9, 2, 300, seed=33)), 1000, 1.05),
    ("zipf_5k_K37_tight", lambda: fp.generate(fp.GenSpec.zipf(5000, 5000, 2.5, 2, 60, beta=1.2, seed=34)), 37, 1.01),
    # eps factor above TV's 1.1 clamp: TV's stream is unsupported, the others run
    ("zipf_3k_K16_loose", lambda: fp.generate(fp.GenSpec.zipf(3000, 3000, 2.1, 2, 200, beta=1.5, seed=35)), 16, 1.3),
]


@pytest.mark.parametrize("name,mk,K,eps", MORE, ids=[c[0] for c in MORE])
@pytest.mark.parametrize("metric", METRICS)
def test_stream_matches_oracle_odd_K_and_status(name, mk, K, eps, metric):
    """K off powers of two (the least-loaded tree's padding), K = 1000, zero
    vertex weights (isolated vertices under degree weights), a tight balance
    factor; where the oracle reports an unsupported input (a TV stream part above
    max_pw), the library reports the same status."""
    hg = mk()
    o = oracle.run_oracle(hg, K, metric, 0, eps_factor=eps)
    assert (o["status"] != 0) == (name == "zipf_3k_K16_loose" and metric == "TV")
    if o["status"] != 0:
        assert o["status"] == -3                    # the oracle's "unsupported"
        with pytest.raises(fp.FastPartError) as ei:
            fp.stream_partition(hg, K, metric, eps)
        assert ei.value.status == fp.ERR_UNSUPPORTED
        return
    s = fp.stream_partition(hg, K, metric, eps)
    np.testing.assert_array_equal(s["part_vec"], o["part_vec_init"])
    np.testing.assert_array_equal(s["ep_ends"], o["ep_len_init"])   # lambda(e), the reference's layout
    np.testing.assert_array_equal(s["ep_parts"], o["ep_part_init"])
    np.testing.assert_array_equal(s["ep_cnt"], o["ep_cnt_init"])
