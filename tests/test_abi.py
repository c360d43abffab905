"""The C ABI library: it loads, exports every entry point include/fastpart.h
declares, and its host-only parts behave (no compute call needs a GPU here)."""
import ctypes as C
import re
import subprocess
import sys

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


def test_python_status_codes_match_the_header(fp):
    text = (ROOT / "include" / "fastpart.h").read_text()
    codes = re.findall(r"#define FP_(OK|ERR_\w+)\s+(-?\d+)", text)
    assert len(codes) == 8
    for name, val in codes:
        assert getattr(fp, name) == int(val), name


def _plbin(path, noe, nov, pins, body=b""):
    import struct
    path.write_bytes(struct.pack("<IIq", noe, nov, pins) + body)


def test_corrupt_inputs_are_rejected_not_fatal(fp, tmp_path):
    """Headers with counts beyond int32 or the pin limit, caches shorter than
    their header says, and CSR offsets that go backwards give a status code;
    none makes the library allocate from the header or read past a buffer."""
    import struct
    cases = {
        "huge_noe": (0x7FFFFFFF, 10, 4, b""),
        "noe_above_int32": (0x80000001, 10, 4, b""),
        "pins_above_limit": (2, 10, 1 << 40, b""),
        "no_vertices": (1, 0, 2, struct.pack("<III", 2, 0, 1)),
        "truncated": (2, 10, 4, struct.pack("<III", 2, 0, 1)),
        "id_out_of_range": (1, 10, 2, struct.pack("<III", 2, 0, 11)),
    }
    for name, (noe, nov, pins, body) in cases.items():
        txt = tmp_path / f"{name}.hg"
        txt.write_text("garbage\n")                     # the cache is read first
        _plbin(tmp_path / f"{name}.hg.plbin", noe, nov, pins, body)
        with pytest.raises(fp.FastPartError) as ei:
            fp.read_patohlike(txt, transpose=True)
        assert ei.value.status == fp.ERR_IO, name
    for name, header in {"pins_huge": "0 5 2 1099511627776", "nov_huge": "0 5000000000 2 4",
                         "negative_nov": "0 -5 2 4"}.items():
        p = tmp_path / f"{name}.hg"
        p.write_text(header + "\n0 1\n2 3\n")
        with pytest.raises(fp.FastPartError) as ei:
            fp.read_patohlike(p, transpose=True)
        assert ei.value.status == fp.ERR_IO, name
    lib = fp.lib()
    g = C.c_void_p()
    back = np.array([0, 3, 2, 4], np.uint32)             # net 1 ends before it starts
    pins = np.array([0, 1, 2, 3], np.uint32)
    assert lib.fp_graph_from_nets(5, 3, back.ctypes.data, pins.ctypes.data, None, C.byref(g)) == fp.ERR_INVALID
    off = np.array([1, 2, 4], np.uint32)                 # offsets not starting at 0
    assert lib.fp_graph_from_nets(5, 2, off.ctypes.data, pins.ctypes.data, None, C.byref(g)) == fp.ERR_INVALID
    assert lib.fp_graph_from_vertices(2, 3, off.ctypes.data, pins.ctypes.data, None, C.byref(g)) == fp.ERR_INVALID


def test_failed_host_allocation_is_a_status_not_an_abort(fp):
    """Under an address-space limit, a hypergraph too large to build gives
    FP_ERR_NOMEM from the C ABI (a C++ exception never crosses it)."""
    code = (
        "import resource, sys\n"
        f"sys.path.insert(0, {str(ROOT)!r})\n"
        "import fastpartitioner_gb300 as fp\n"
        "fp.lib()\n"
        "resource.setrlimit(resource.RLIMIT_AS, (3 << 30, 3 << 30))\n"
        "try:\n"
        "    fp.generate(fp.GenSpec.column_net(400_000_000, 400_000_000, 2, 16, seed=1))\n"
        "    print('built')\n"
        "except fp.FastPartError as e:\n"
        "    print('status', e.status)\n"
    )
    res = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr[-2000:]
    assert res.stdout.strip() == f"status {fp.ERR_NOMEM}"


def test_footprint_lists_every_instance_allocation():
    """fp_instance_footprint mirrors fp_instance_create's device allocations:
    one size term per dalloc call (a loop of n terms counts n), so an
    allocation added to one and not the other fails here.  The GPU tests check
    the byte totals against fp_instance_device_bytes."""
    src = (ROOT / "fastpartitioner_gb300" / "csrc" / "fp_api.cu").read_text()
    create = src[src.index("int fp_instance_create("):src.index("int fp_instance_device_bytes(")]
    foot = src[src.index("int fp_instance_footprint("):src.index("int fp_instance_destroy(")]
    # the metric scratch is one term of its own (metrics_scratch_bytes), whether
    # it comes from cudaMalloc or from the context's arena through dalloc
    n_alloc = len(re.findall(r"\bdalloc\(in,", create)) - len(re.findall(r"\bdalloc\(in, &q, metrics_scratch", create))
    n_terms = sum(int(m.group(2)) if m.group(2) else 1
                  for m in re.finditer(r"(for \(int k = 0; k < (\d+); k\+\+\) )?\badd\(", foot))
    assert n_alloc > 40 and n_terms == n_alloc
    assert "metrics_scratch_bytes(K)" in create and "metrics_scratch_bytes(K)" in foot
