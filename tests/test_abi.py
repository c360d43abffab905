"""The C ABI library: it loads, exports every entry point include/fastpart.h
declares, and its host-only parts behave (no compute call needs a GPU here)."""
import ctypes as C
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT


def declared_symbols():
    text = (ROOT / "include" / "fastpart.h").read_text()
    return sorted(set(re.findall(r"^(?:int|const char\*)\s+(fp_\w+)\s*\(", text, re.M)))


def test_header_declares_the_api():
    syms = declared_symbols()
    for must in ("fp_ctx_create", "fp_instance_create", "fp_refine", "fp_metrics", "fp_partition_gpu",
                 "fp_read_patohlike", "fp_validate"):
        assert must in syms


def test_library_exports_every_declared_symbol(fp):
    lib = C.CDLL(str(fp.library_path()))
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", str(fp.library_path())], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (fp_\w+)", out))
    assert set(declared_symbols()) <= exported


def test_strerror(fp):
    L = fp.lib()
    assert L.fp_strerror(0) == b"ok"
    assert b"invalid" in L.fp_strerror(-1)
    assert L.fp_strerror(-999) == b"unknown status"


def test_validate_accepts_generated(fp):
    hg = fp.generate(fp.GenSpec.column_net(300, 300, 2, 10, seed=5))
    assert hg.validate() == 0


def _clone(fp, hg, **kw):
    d = dict(nov=hg.nov, noe=hg.noe, vptr=hg.vptr.copy(), vnets=hg.vnets.copy(), nptr=hg.nptr.copy(),
             npins=hg.npins.copy(), src=hg.src.copy(), weights=None, ordering=None)
    d.update(kw)
    return fp.Hypergraph(**d)


def test_validate_rejects_malformed(fp):
    hg = fp.generate(fp.GenSpec.column_net(200, 200, 2, 10, seed=6))
    bad_src = hg.src.copy()
    # a source that is not a pin of its net
    e = 0
    pins = set(hg.npins[hg.nptr[e]:hg.nptr[e + 1]].tolist())
    bad_src[e] = next(v for v in range(hg.nov) if v not in pins)
    assert _clone(fp, hg, src=bad_src).validate() == -1
    # a net id out of range
    vn = hg.vnets.copy()
    vn[0] = hg.noe
    assert _clone(fp, hg, vnets=vn).validate() == -1
    # an ordering that is not a permutation
    order = np.arange(hg.nov, dtype=np.int32)
    order[1] = 0
    assert _clone(fp, hg, ordering=order).validate() == -1
    # negative weight
    w = np.ones(hg.nov, np.int32)
    w[3] = -1
    assert _clone(fp, hg, weights=w).validate() == -1
    # net -> pins that is not the transpose of vertex -> nets
    np2 = hg.npins.copy()
    np2[0], np2[-1] = np2[-1], np2[0]
    if hg.npins[0] != hg.npins[-1]:
        assert _clone(fp, hg, npins=np2).validate() == -1


def test_no_gpu_is_an_error_not_a_fallback(fp):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(fp.FastPartError) as ei:
        fp.Engine(0)
    assert ei.value.status == -2
