"""CPU oracle for the GB300 refinement engine -- TEST INFRASTRUCTURE ONLY.

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU legs, never by the
product package.  Two checkers live here:

* ``run_oracle`` -- libfporacle.so, a single-threaded C++ restatement of the
  reference's sequential partition() for the six metrics (fp_oracle.cpp).
* ``run_reference`` -- the reference's own partition() / partition_par(),
  compiled from its sources by oracle/Makefile into oracle/_ref/ and driven by
  ref_harness.cpp.  Used to pin the restatement and to time the reference.
"""
from __future__ import annotations

import ctypes as C
import os
import re
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "libfporacle.so"
REF_DIR = HERE / "_ref"

METRIC_IDS = {"CN": 0, "TV": 1, "TM": 2, "MSM": 3, "MSV": 4, "MSRV": 5}
REF_BIN = {"TV": "ref_tv", "CN": "ref_cn", "TM": "ref_tm", "MSM": "ref_msm", "MSV": "ref_mgv", "MSRV": "ref_msrv"}
OUTPUT_ORDER = ["TV", "CN", "TM", "MSM", "MSV", "MSRV"]
_PRINT_NAMES = {"TV": "TV", "CN": "CN", "TM": "TM", "MSM": "MGM", "MSV": "MGV", "MSRV": "MGAV"}


class _Hg(C.Structure):
    _fields_ = [("nov", C.c_int), ("noe", C.c_int), ("pins", C.c_longlong),
                ("vptr", C.c_void_p), ("vnets", C.c_void_p), ("nptr", C.c_void_p),
                ("npins", C.c_void_p), ("src", C.c_void_p), ("weights", C.c_void_p),
                ("ordering", C.c_void_p)]


class _Run(C.Structure):
    _fields_ = [("metric", C.c_int), ("K", C.c_int), ("eps_factor", C.c_double),
                ("passes", C.c_int), ("refine", C.c_int),
                ("part_vec_init", C.c_void_p), ("ep_len_init", C.c_void_p),
                ("ep_part_init", C.c_void_p), ("ep_cnt_init", C.c_void_p),
                ("part_vec", C.c_void_p), ("ep_len", C.c_void_p), ("ep_part", C.c_void_p),
                ("ep_cnt", C.c_void_p), ("metrics_init", C.c_longlong * 6),
                ("metrics_final", C.c_longlong * 6), ("moves", C.c_longlong * 64),
                ("refine_seconds", C.c_double), ("status", C.c_int),
                ("rec_dest", C.c_void_p), ("rec_gain", C.c_void_p), ("rec_loss", C.c_void_p),
                ("rec_moved", C.c_void_p)]


def build(quiet: bool = True) -> None:
    """Builds libfporacle.so (required) and, where the reference sources are
    reachable, the reference harness binaries (optional: the tests that need
    one skip when it is missing, so a harness that does not build only warns)."""
    res = subprocess.run(["make", "-C", str(HERE), "-j8", "oracle"], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")
    if not quiet:
        print(res.stdout)
    ref = subprocess.run(["make", "-C", str(HERE), "-j8", "-k", "ref"], capture_output=True, text=True)
    if ref.returncode != 0:
        print(f"warning: some reference harnesses did not build:\n{ref.stdout[-2000:]}\n{ref.stderr[-2000:]}",
              file=sys.stderr)
    elif not quiet:
        print(ref.stdout)


_lib = None


def _oracle():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        _lib = C.CDLL(str(LIB))
        _lib.fpo_partition.argtypes = [C.POINTER(_Hg), C.POINTER(_Run)]
        _lib.fpo_partition.restype = C.c_int
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


def run_oracle(hg, K: int, metric: str, passes: int, eps_factor: float = 1.05, refine: bool = True,
               records: bool = False):
    """Runs the restated reference pipeline (stream + passes + metrics).
    Returns a dict of numpy arrays and metric dicts; with records, also the
    decision records of the last pass (rec_dest, rec_gain, rec_loss,
    rec_moved: one entry per vertex, per net for CN)."""
    m = METRIC_IDS[metric.upper()]
    nov, noe, pins = hg.nov, hg.noe, hg.pins
    nrec = noe if metric.upper() == "CN" else nov
    shapes = [("part_vec_init", nov), ("ep_len_init", noe), ("ep_part_init", pins), ("ep_cnt_init", pins),
              ("part_vec", nov), ("ep_len", noe), ("ep_part", pins), ("ep_cnt", pins)]
    if records:
        shapes += [("rec_dest", nrec), ("rec_gain", nrec), ("rec_loss", nrec), ("rec_moved", nrec)]
    out = {k: np.full(n, -2, np.int32) if k.startswith("rec_") else np.empty(n, np.int32) for k, n in shapes}
    h = _Hg(nov, noe, pins, _p(hg.vptr), _p(hg.vnets), _p(hg.nptr), _p(hg.npins), _p(hg.src),
            _p(hg.weights), _p(hg.ordering))
    r = _Run()
    r.metric, r.K, r.eps_factor, r.passes, r.refine = m, K, eps_factor, passes, int(refine)
    for k, a in out.items():
        setattr(r, k, a.ctypes.data)
    rc = _oracle().fpo_partition(C.byref(h), C.byref(r))
    out["status"] = rc
    out["metrics_init"] = dict(zip(OUTPUT_ORDER, list(r.metrics_init)))
    out["metrics_final"] = dict(zip(OUTPUT_ORDER, list(r.metrics_final)))
    out["moves"] = np.array(list(r.moves)[:passes], np.int64)
    out["refine_seconds"] = r.refine_seconds
    return out


def reference_available(metric: str = "TV") -> bool:
    return (REF_DIR / REF_BIN[metric.upper()]).exists()


def _read_capture(path: Path, nov: int, noe: int):
    raw = np.fromfile(path, dtype=np.int32)
    assert raw[0] == nov and raw[1] == noe, "capture header mismatch"
    part_vec = raw[2:2 + nov].copy()
    ep_len = raw[2 + nov:2 + nov + noe].copy()
    flat = raw[2 + nov + noe:].copy()
    return part_vec, ep_len, flat


class ReferenceRunError(RuntimeError):
    """The reference harness exited non-zero; `returncode` < 0 is the signal
    that ended it."""

    def __init__(self, returncode: int, message: str):
        super().__init__(message)
        self.returncode = returncode


def run_reference(hg, K: int, metric: str, passes: int, threads: int = 1, capture: bool = True,
                  timeout: float = 3600):
    """Runs the reference's own partition() (threads == 1) or partition_par()
    on `hg` through the harness.  Returns its printed metrics, its
    'Refinement took' seconds and, with capture, the part vector and ordered part
    lists after the initial stream and after refinement."""
    metric = metric.upper()
    exe = REF_DIR / REF_BIN[metric]
    if not exe.exists():
        raise FileNotFoundError(f"{exe} not built (reference sources unavailable)")
    with tempfile.TemporaryDirectory(prefix="fpref") as td:
        inst = Path(td) / "inst.fphg"
        hg.save_fphg(inst)
        prefix = str(Path(td) / "cap") if capture else "-"
        env = dict(os.environ)
        env.setdefault("OMP_NUM_THREADS", str(max(threads, 1)))
        res = subprocess.run([str(exe), str(inst), str(K), str(passes), str(threads), prefix],
                             capture_output=True, text=True, timeout=timeout, env=env, cwd=td)
        if res.returncode != 0:
            raise ReferenceRunError(res.returncode, f"reference run failed ({res.returncode}):\n"
                                                    f"{res.stdout[-2000:]}\n{res.stderr[-2000:]}")
        text = res.stdout
        out = {"stdout": text}
        before, after = {}, {}
        for key in OUTPUT_ORDER:
            pn = _PRINT_NAMES[key]
            mb = re.search(rf"^{pn} : (-?\d+)$", text, re.M)
            ma = re.search(rf"^After Refinement {pn} : (-?\d+)$", text, re.M)
            if mb:
                before[key] = int(mb.group(1))
            if ma:
                after[key] = int(ma.group(1))
        out["metrics_init"], out["metrics_final"] = before, after
        mt = re.search(r"^Refinement took : ([0-9.eE+-]+) seconds", text, re.M)
        out["refine_seconds"] = float(mt.group(1)) if mt else None
        if capture:
            caps = sorted((p for p in Path(td).glob("cap.*") if p.suffix[1:].isdigit() and p.name.count(".") == 1),
                          key=lambda p: int(p.suffix[1:]))
            if caps:
                out["part_vec_init"], out["ep_len_init"], out["lists_init"] = _read_capture(caps[0], hg.nov, hg.noe)
            if len(caps) > 1:
                out["part_vec"], out["ep_len"], out["lists"] = _read_capture(caps[-1], hg.nov, hg.noe)
        return out


def run_reference_bfs(hg, start: int, timeout: float = 600):
    """The reference's BFS ordering (-o 1: createInverse, bfsFarthest_queue_par
    twice, bfsOrdering_queue_par, one thread) from vertex `start`, through the
    ref_bfs harness.  Returns (first farthest, second farthest, ordering with
    -1 past the reached vertices)."""
    exe = REF_DIR / "ref_bfs"
    if not exe.exists():
        raise FileNotFoundError(f"{exe} not built (reference sources unavailable)")
    with tempfile.TemporaryDirectory(prefix="fpbfs") as td:
        inst = Path(td) / "inst.fphg"
        hg.save_fphg(inst)
        env = dict(os.environ, OMP_NUM_THREADS="1")
        res = subprocess.run([str(exe), str(inst), str(int(start))], capture_output=True, text=True,
                             timeout=timeout, env=env, cwd=td)
        if res.returncode != 0:
            raise RuntimeError(f"reference bfs failed ({res.returncode}): {res.stderr[-2000:]}")
        vals = np.array(res.stdout.split(), dtype=np.int64)
        return int(vals[0]), int(vals[1]), vals[2:2 + hg.nov].astype(np.int32)


def run_reference_read(path, timeout: float = 600) -> dict:
    """The reference's read_patohlike on `path` (it reads <path>.plbin when
    present and writes it otherwise), through the ref_read harness: ok, nov,
    noe, pins and the line CSR (col_ptr, row_ind) with the per-id counts."""
    exe = REF_DIR / "ref_read"
    if not exe.exists():
        raise FileNotFoundError(f"{exe} not built (reference sources unavailable)")
    with tempfile.TemporaryDirectory(prefix="fpread") as td:
        out = Path(td) / "out.bin"
        res = subprocess.run([str(exe), str(path), str(out)], capture_output=True, text=True, timeout=timeout)
        if res.returncode != 0:
            raise RuntimeError(f"reference read failed ({res.returncode}): {res.stderr[-2000:]}")
        raw = out.read_bytes()
    ok, nov, noe = np.frombuffer(raw[:12], np.int32)
    pins = int(np.frombuffer(raw[12:20], np.int64)[0])
    r = {"ok": bool(ok), "nov": int(np.uint32(nov)), "noe": int(np.uint32(noe)), "pins": pins}
    if ok:
        arr = np.frombuffer(raw[20:], np.uint32)
        n, m = r["noe"] + 1, pins
        r["col_ptr"], r["row_ind"], r["appear"] = arr[:n], arr[n:n + m], arr[n + m:n + m + r["nov"]]
    return r


def flat_lists(hg, ep_len, ep_part):
    """Concatenation of every net's listed parts, in list order (the form the
    reference capture stores)."""
    starts = hg.nptr[:-1].astype(np.int64)
    idx = np.concatenate([np.arange(s, s + n) for s, n in zip(starts, ep_len)]) if len(ep_len) else np.zeros(0, np.int64)
    return ep_part[idx.astype(np.int64)] if idx.size else np.zeros(0, np.int32)


def run_reference_wrapper_state(hg, K: int, metric: str, timeout: float = 600) -> dict:
    """Runs the reference's own partition_gpu() (TV, CN, TM, MSV, MSRV) through
    the harness, whose stand-in partition_gpu_wrapper records the state arrays
    partition_gpu() hands to its GPU wrapper after the initial stream: the
    exact input a drop-in shim receives.  Returns them by name (part_vec,
    psizes, ep_start, ep_ends, ep_parts, ep_cnt, and marker / send / conn /
    msgs where the metric's wrapper takes them)."""
    metric = metric.upper()
    exe = REF_DIR / REF_BIN[metric]
    if metric == "MSM" or not exe.exists():
        raise FileNotFoundError(f"no partition_gpu harness for {metric}")
    with tempfile.TemporaryDirectory(prefix="fpwrap") as td:
        inst = Path(td) / "inst.fphg"
        hg.save_fphg(inst)
        prefix = str(Path(td) / "cap")
        res = subprocess.run([str(exe), str(inst), str(K), "1", "0", prefix], capture_output=True, text=True,
                             timeout=timeout, cwd=td)
        if res.returncode != 0:
            raise ReferenceRunError(res.returncode, f"reference partition_gpu failed ({res.returncode}):\n"
                                                    f"{res.stdout[-2000:]}\n{res.stderr[-2000:]}")
        raw = Path(prefix + ".wrap").read_bytes()
    out, pos = {}, 0
    while pos < len(raw):
        name = raw[pos:pos + 8].rstrip(b"\0").decode()
        n = int(np.frombuffer(raw, np.int64, 1, pos + 8)[0])
        out[name] = np.frombuffer(raw, np.int32, n, pos + 16).copy()
        pos += 16 + 4 * n
    return out


_ref_metrics_lib = None


def reference_metrics(hg, K: int, part_vec, ep_starts, ep_ends, ep_parts, ep_cnt) -> dict:
    """The reference's own metric evaluators (shared/metric.cpp, built into
    oracle/_ref/libref_metrics.so) on a state in the reference's layout:
    TV, CN, TM, MSM, MSV, MSRV as partition_gpu() computes them after
    refinement, plus TV_lambda = TV(ep_ends), its pre-refinement form."""
    global _ref_metrics_lib
    if _ref_metrics_lib is None:
        path = REF_DIR / "libref_metrics.so"
        if not path.exists():
            raise FileNotFoundError(f"{path} not built (reference sources unavailable)")
        L = C.CDLL(str(path))
        L.ref_metrics.argtypes = [C.c_int, C.c_int, C.c_int, C.c_longlong] + [C.c_void_p] * 10
        L.ref_metrics.restype = C.c_int
        _ref_metrics_lib = L
    a = lambda x, dt: np.ascontiguousarray(x, dtype=dt)
    sizes = np.diff(hg.nptr).astype(np.uint32)
    arrs = [a(hg.vptr, np.uint32), a(hg.vnets, np.uint32), sizes, a(hg.src, np.int32), a(part_vec, np.int32),
            a(ep_starts, np.int32), a(ep_ends, np.int32), a(ep_parts, np.int32), a(ep_cnt, np.int32)]
    out = np.zeros(7, np.int64)
    _ref_metrics_lib.ref_metrics(K, hg.nov, hg.noe, hg.pins, *[x.ctypes.data for x in arrs], out.ctypes.data)
    d = dict(zip(OUTPUT_ORDER, map(int, out[:6])))
    d["TV_lambda"] = int(out[6])
    return d


def generate_fphg(path, nov: int, noe: int, size_lo: int, size_hi: int, size_alpha: float = 0.0,
                  pin_beta: float = 0.0, src_rule: int = 0, sort_pins: int = 1, seed: int = 0) -> None:
    """Draws a seeded workload instance (fp_oracle_gen.cpp, the same draws as
    the product generator) and writes it as the .fphg file the reference
    harness reads -- without loading the product library."""
    L = _oracle()
    f = L.fpo_generate_fphg
    f.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, C.c_int, C.c_ulonglong,
                  C.c_char_p]
    f.restype = C.c_int
    if f(nov, noe, size_lo, size_hi, size_alpha, pin_beta, src_rule, sort_pins, seed, str(path).encode()) != 0:
        raise RuntimeError(f"oracle generator failed for {path}")


def fphg_header(path) -> tuple:
    """(nov, noe, pins) of an .fphg file."""
    raw = Path(path).read_bytes()[:24]
    nov, noe = np.frombuffer(raw, np.int32, 2, 8)
    return int(nov), int(noe), int(np.frombuffer(raw, np.int64, 1, 16)[0])


def run_reference_file(path, K: int, metric: str, passes: int, threads: int = 1, timeout: float = 3600) -> dict:
    """The reference's partition() / partition_par() on an .fphg instance file,
    no capture: its printed metrics and 'Refinement took' seconds."""
    metric = metric.upper()
    exe = REF_DIR / REF_BIN[metric]
    if not exe.exists():
        raise FileNotFoundError(f"{exe} not built (reference sources unavailable)")
    env = dict(os.environ)
    env.setdefault("OMP_NUM_THREADS", str(max(threads, 1)))
    with tempfile.TemporaryDirectory(prefix="fpref") as td:
        res = subprocess.run([str(exe), str(path), str(K), str(passes), str(threads), "-"], capture_output=True,
                             text=True, timeout=timeout, env=env, cwd=td)
    if res.returncode != 0:
        raise ReferenceRunError(res.returncode, f"reference run failed ({res.returncode}):\n"
                                                f"{res.stdout[-2000:]}\n{res.stderr[-2000:]}")
    out = {"stdout": res.stdout}
    after = {}
    for key in OUTPUT_ORDER:
        ma = re.search(rf"^After Refinement {_PRINT_NAMES[key]} : (-?\d+)$", res.stdout, re.M)
        if ma:
            after[key] = int(ma.group(1))
    out["metrics_final"] = after
    mt = re.search(r"^Refinement took : ([0-9.eE+-]+) seconds", res.stdout, re.M)
    out["refine_seconds"] = float(mt.group(1)) if mt else None
    return out


class FphgInstance:
    """An .fphg instance as numpy arrays (the attributes run_oracle reads),
    loaded without the product library."""

    def __init__(self, path):
        raw = Path(path).read_bytes()
        if raw[:5] != b"FPHG1":
            raise ValueError("not an FPHG1 file")
        self.nov, self.noe, self.pins = fphg_header(path)
        off = 24
        for name, n, dt in (("vptr", self.nov + 1, np.uint32), ("vnets", self.pins, np.uint32),
                            ("nptr", self.noe + 1, np.uint32), ("npins", self.pins, np.uint32),
                            ("src", self.noe, np.int32)):
            setattr(self, name, np.frombuffer(raw, dt, n, off).copy())
            off += 4 * n
        self.weights = None
        self.ordering = None
