"""The CPU oracle against the reference's own outputs (committed fixtures made by
tests/golden/make_golden.py from the reference compiled from its sources)."""
import numpy as np
import pytest

from conftest import METRICS, golden_cases, load_golden

OUT = ["TV", "CN", "TM", "MSM", "MSV", "MSRV"]


@pytest.mark.parametrize("path", golden_cases(), ids=lambda p: p.stem)
def test_oracle_matches_reference_fixtures(fp, orc, path):
    hg, passes, Ks, z = load_golden(path)
    for m in METRICS:
        for K in Ks:
            key = f"{m}_{K}"
            o = orc.run_oracle(hg, K, m, passes)
            assert o["status"] == 0, key
            np.testing.assert_array_equal(o["part_vec_init"], z[f"{key}_part_vec_init"], err_msg=key)
            np.testing.assert_array_equal(o["part_vec"], z[f"{key}_part_vec"], err_msg=key)
            np.testing.assert_array_equal(o["ep_len"], z[f"{key}_ep_len"], err_msg=key)
            np.testing.assert_array_equal(orc.flat_lists(hg, o["ep_len"], o["ep_part"]), z[f"{key}_lists"],
                                          err_msg=key)
            assert [o["metrics_init"][k] for k in OUT] == list(z[f"{key}_metrics_init"]), key
            assert [o["metrics_final"][k] for k in OUT] == list(z[f"{key}_metrics_final"]), key


def test_fixtures_exercise_moves(fp, orc):
    """The fixtures are only useful if refinement actually moves vertices for
    every metric somewhere in the set."""
    moved = {m: 0 for m in METRICS}
    for path in golden_cases():
        hg, passes, Ks, z = load_golden(path)
        for m in METRICS:
            for K in Ks:
                moved[m] += int(np.sum(z[f"{m}_{K}_part_vec"] != z[f"{m}_{K}_part_vec_init"]))
    assert all(v > 0 for v in moved.values()), moved


def test_list_invariants_of_fixtures(fp, orc):
    """checkMe (MSM/partition.cpp:2-68): the ordered lists hold every part of a
    net's pins exactly once, with the right counts."""
    for path in golden_cases():
        hg, passes, Ks, z = load_golden(path)
        for m in METRICS:
            for K in Ks:
                pv = z[f"{m}_{K}_part_vec"]
                ln = z[f"{m}_{K}_ep_len"]
                flat = z[f"{m}_{K}_lists"]
                off = 0
                for e in range(hg.noe):
                    parts = set(pv[hg.npins[hg.nptr[e]:hg.nptr[e + 1]]].tolist())
                    listed = flat[off:off + ln[e]].tolist()
                    off += ln[e]
                    assert len(listed) == len(set(listed)) and set(listed) == parts
