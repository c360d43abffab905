"""PaToH-like ingestion against the reference's own reader: fp_read_patohlike
and the reference's read_patohlike (shared/hypergraph_rw.cpp:97-242, compiled
into oracle/_ref/ref_read) give the same line CSR, write byte-identical
<file>.plbin caches, and read each other's caches."""
import shutil

import numpy as np
import pytest

import fastpartitioner_gb300 as fp
import oracle

pytestmark = pytest.mark.skipif(not (oracle.REF_DIR / "ref_read").exists(),
                                reason="reference reader harness not built (reference sources unavailable)")


def text_of(lines, nov, base=0, noe=None, pins=None):
    noe = len([ln for ln in lines if ln]) if noe is None else noe
    pins = sum(len(ln) for ln in lines) if pins is None else pins
    body = "\n".join(" ".join(str(x + base) for x in ln) for ln in lines)
    return f"{base} {nov} {noe} {pins}\n{body}\n"


def generated(seed, square=False):
    hg = fp.generate(fp.GenSpec.zipf(600 if square else 700, 600 if square else 500, 2.1, 2, 40, beta=1.2,
                                     seed=seed))
    return [hg.npins[hg.nptr[e]:hg.nptr[e + 1]].tolist() for e in range(hg.noe)], hg.nov


CASES = {
    "zero_based_empty_line": (text_of([[0, 1, 2], [2, 3], [], [4, 5, 0], [1, 5]], 6)),
    "one_based": (text_of([[0, 1, 2], [2, 3], [4, 5, 0], [1, 5]], 6, base=1)),
    "more_nets_declared": (text_of([[0, 1, 2], [2, 3], [4, 5, 0], [1, 5]], 6, noe=7)),
    "square": (text_of([[0, 1], [1, 2, 3], [3, 4], [0, 4, 2], [1, 3]], 5)),
    "generated_square": text_of(*generated(3, square=True)),
    "generated_1": text_of(*generated(1)),
    "generated_2": text_of(*generated(2), base=1),
}


def copies(tmp_path, text):
    out = []
    for d in ("ref", "ours"):
        (tmp_path / d).mkdir()
        p = tmp_path / d / "g.hg"
        p.write_text(text)
        out.append(p)
    return out


@pytest.mark.parametrize("name", sorted(CASES))
def test_reader_and_cache_match_the_reference(tmp_path, name):
    ref_path, our_path = copies(tmp_path, CASES[name])
    r = oracle.run_reference_read(ref_path)
    assert r["ok"], name
    g = fp.read_patohlike(our_path, transpose=True, write_cache=True)
    assert (g.nov, g.noe, g.pins) == (r["nov"], r["noe"], r["pins"]), name
    np.testing.assert_array_equal(g.nptr, r["col_ptr"], err_msg=name)
    np.testing.assert_array_equal(g.npins, r["row_ind"], err_msg=name)
    np.testing.assert_array_equal(np.diff(g.vptr), r["appear"], err_msg=name)
    assert ref_path.with_suffix(".hg.plbin").read_bytes() == our_path.with_suffix(".hg.plbin").read_bytes(), name
    # lines as vertices (TM / MSM / MGV / MSRV drivers, TM/tm.cpp:65): the same
    # CSR, other side.  Those drivers index the line CSR with the header's
    # vertex count, so only a square file is defined; others are rejected.
    if r["nov"] == r["noe"]:
        h = fp.read_patohlike(our_path, transpose=False)
        np.testing.assert_array_equal(h.vptr, r["col_ptr"], err_msg=name)
        np.testing.assert_array_equal(h.vnets, r["row_ind"], err_msg=name)
    else:
        with pytest.raises(fp.FastPartError) as ei:
            fp.read_patohlike(our_path, transpose=False)
        assert ei.value.status == -1


def test_each_reads_the_others_cache(tmp_path):
    text = CASES["generated_1"]
    ref_path, our_path = copies(tmp_path, text)
    oracle.run_reference_read(ref_path)                          # writes ref/g.hg.plbin
    fp.read_patohlike(our_path, transpose=True, write_cache=True)  # writes ours/g.hg.plbin
    # swap the caches and make the text unreadable: both must use the cache
    a, b = ref_path.with_suffix(".hg.plbin"), our_path.with_suffix(".hg.plbin")
    tmp = tmp_path / "swap"
    shutil.copy(a, tmp)
    shutil.copy(b, a)
    shutil.copy(tmp, b)
    for p in (ref_path, our_path):
        p.write_text("garbage\n")
    r = oracle.run_reference_read(ref_path)
    g = fp.read_patohlike(our_path, transpose=True)
    assert r["ok"]
    np.testing.assert_array_equal(g.nptr, r["col_ptr"])
    np.testing.assert_array_equal(g.npins, r["row_ind"])


def test_pin_count_mismatch_fails_in_both(tmp_path):
    ref_path, our_path = copies(tmp_path, text_of([[0, 1, 2], [2, 3]], 4, pins=9))
    assert not oracle.run_reference_read(ref_path)["ok"]
    with pytest.raises(fp.FastPartError):
        fp.read_patohlike(our_path, transpose=True)
