"""GB300 refinement engine for FastPartitioner hypergraph partitions.

The package is a thin host-side mirror of FastPartitioner's per-metric
``partition_gpu()`` entry points over the C ABI in ``include/fastpart.h``.  The
refinement passes and the metric evaluation run as CUDA kernels for sm_103a in
``libfastpart.so``; there is no CPU fallback.  If the library is missing or no
GPU is visible, the calls that need the device raise ``FastPartError``.

Typical use::

    import fastpartitioner_gb300 as fp
    hg = fp.generate(fp.GenSpec.column_net(16384, 16384, 2, 16, seed=0))
    with fp.Engine() as eng:
        inst = eng.instance(hg, K=8, metric="TV")
        inst.initial_partition()
        before = inst.metrics()
        inst.refine(5)
        after = inst.metrics()
"""
from __future__ import annotations

import ctypes as C
import dataclasses
from pathlib import Path
from typing import Optional, Sequence

import numpy as np

_PKG = Path(__file__).resolve().parent
_LIB_PATH = _PKG / "libfastpart.so"

FP_OK = 0
ERRORS = {
    -1: "invalid argument or malformed hypergraph",
    -2: "CUDA runtime error",
    -3: "out of memory",
    -4: "device-side wait timed out",
    -5: "input on which the reference behaviour is undefined",
    -6: "call out of order",
    -7: "file error",
}

# Metric ids of the C ABI; the reference's directory / print names map onto them.
METRICS = {"CN": 0, "TV": 1, "TM": 2, "MSM": 3, "MSV": 4, "MSRV": 5,
           "MGM": 3, "MGV": 4, "MGAV": 5}
METRIC_NAMES = ["CN", "TV", "TM", "MSM", "MSV", "MSRV"]
# Order of fp_metrics() values: the order the reference prints them.
OUTPUT_ORDER = ["TV", "CN", "TM", "MSM", "MSV", "MSRV"]

# status codes of include/fastpart.h
OK = 0
ERR_INVALID = -1
ERR_CUDA = -2
ERR_NOMEM = -3
ERR_DEVICE_TIMEOUT = -4
ERR_UNSUPPORTED = -5
ERR_STATE = -6
ERR_IO = -7


class FastPartError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        super().__init__(f"{what}: {ERRORS.get(status, 'unknown status')} ({status})")


def metric_id(metric) -> int:
    if isinstance(metric, (int, np.integer)):
        if not 0 <= int(metric) <= 5:
            raise ValueError(f"unknown metric {metric}")
        return int(metric)
    try:
        return METRICS[str(metric).upper()]
    except KeyError:
        raise ValueError(f"unknown metric {metric!r}") from None


# ---------------------------------------------------------------- C types

class _Hypergraph(C.Structure):
    _fields_ = [("nov", C.c_int32), ("noe", C.c_int32), ("pins", C.c_int64),
                ("vptr", C.c_void_p), ("vnets", C.c_void_p), ("nptr", C.c_void_p),
                ("npins", C.c_void_p), ("src", C.c_void_p), ("weights", C.c_void_p),
                ("ordering", C.c_void_p)]


class _GenParams(C.Structure):
    _fields_ = [("nov", C.c_int32), ("noe", C.c_int32), ("size_lo", C.c_int32),
                ("size_hi", C.c_int32), ("size_alpha", C.c_double), ("pin_beta", C.c_double),
                ("src_rule", C.c_int32), ("sort_pins", C.c_int32), ("weight_rule", C.c_int32),
                ("seed", C.c_uint64)]


_lib_handle = None


def library_path() -> Path:
    return _LIB_PATH


class FpState(C.Structure):
    """fp_state of include/fastpart.h: the reference's refinement arrays."""
    _fields_ = [(n, C.c_void_p) for n in ("part_vec", "ep_starts", "ep_ends", "ep_parts", "ep_cnt", "part_sizes",
                                          "marker", "send", "recv", "conn", "msgs")]


def lib():
    """The loaded engine library (raises FastPartError-free OSError if absent)."""
    global _lib_handle
    if _lib_handle is None:
        if not _LIB_PATH.exists():
            raise OSError(f"{_LIB_PATH} is not built; run fastpartitioner_gb300.build.build()")
        L = C.CDLL(str(_LIB_PATH))
        vp, i32, i64, dbl = C.c_void_p, C.c_int32, C.c_int64, C.c_double
        pp = C.POINTER(C.c_void_p)
        sig = {
            "fp_validate": ([C.POINTER(_Hypergraph)], C.c_int),
            "fp_bfs_order": ([C.POINTER(_Hypergraph), C.c_int32, C.c_void_p, C.c_void_p], C.c_int),
            "fp_stream_partition": ([C.POINTER(_Hypergraph), i32, i32, dbl, C.POINTER(FpState)], C.c_int),
            "fp_check_state": ([C.POINTER(_Hypergraph), i32, i32, dbl, C.POINTER(FpState)], C.c_int),
            "fp_ctx_create": ([i32, pp], C.c_int),
            "fp_ctx_destroy": ([vp], C.c_int),
            "fp_ctx_set_stream": ([vp, vp], C.c_int),
            "fp_ctx_set_arena": ([vp, i64], C.c_int),
            "fp_ctx_set_sm_limit": ([vp, i32], C.c_int),
            "fp_instance_create": ([vp, C.POINTER(_Hypergraph), i32, i32, dbl, pp], C.c_int),
            "fp_instance_destroy": ([vp], C.c_int),
            "fp_instance_device_bytes": ([vp, C.POINTER(i64)], C.c_int),
            "fp_instance_footprint": ([i32, i32, i64, i32, i32, C.POINTER(i64)], C.c_int),
            "fp_initial_partition": ([vp], C.c_int),
            "fp_set_stream_mode": ([vp, i32, C.POINTER(i32)], C.c_int),
            "fp_set_stream_walk": ([vp, i32], C.c_int),
            "fp_refine": ([vp, i32], C.c_int),
            "fp_reset_state": ([vp], C.c_int),
            "fp_set_engine": ([vp, i32], C.c_int),
            "fp_debug_barrier_fault": ([vp, i32, i32], C.c_int),
            "fp_set_decision_log": ([vp, i32], C.c_int),
            "fp_get_decisions": ([vp, vp, vp, vp, vp], C.c_int),
            "fp_set_classes": ([vp, i64, i64], C.c_int),
            "fp_set_window": ([vp, i32, i32], C.c_int),
            "fp_metrics": ([vp, vp], C.c_int),
            "fp_get_partition": ([vp, vp], C.c_int),
            "fp_get_lists": ([vp, vp, vp, vp], C.c_int),
            "fp_set_state": ([vp, C.POINTER(FpState)], C.c_int),
            "fp_get_state": ([vp, C.POINTER(FpState)], C.c_int),
            "fp_get_part_sizes": ([vp, vp], C.c_int),
            "fp_get_moves": ([vp, vp, i32], C.c_int),
            "fp_last_launches": ([vp, vp], C.c_int),
            "fp_get_stats": ([vp, vp, i32], C.c_int),
            "fp_strerror": ([C.c_int], C.c_char_p),
            "fp_generate": ([C.POINTER(_GenParams), pp], C.c_int),
            "fp_graph_from_nets": ([i32, i32, vp, vp, vp, pp], C.c_int),
            "fp_graph_from_vertices": ([i32, i32, vp, vp, vp, pp], C.c_int),
            "fp_read_patohlike": ([C.c_char_p, i32, i32, pp], C.c_int),
            "fp_thin_nets": ([C.POINTER(_Hypergraph), i32, i32, pp], C.c_int),
            "fp_create_inverse": ([vp, i32, i32, i64, vp, vp, vp, vp], C.c_int),
            "fp_thin_nets_device": ([vp, C.POINTER(_Hypergraph), i32, i32, pp], C.c_int),
            "fp_bfs_order_device": ([vp, C.POINTER(_Hypergraph), i32, vp, vp], C.c_int),
            "fp_write_patohlike": ([vp, C.c_char_p], C.c_int),
            "fp_graph_view": ([vp, C.POINTER(_Hypergraph)], C.c_int),
            "fp_graph_destroy": ([vp], C.c_int),
            "fp_metrics_noalloc": ([i32, i32, i32, i64, vp, vp, vp, vp, vp, vp, vp], C.c_int),
            "fp_partition_gpu": ([i32, vp, vp, vp, i32, i32, i64, vp, vp, i32, vp, C.c_char_p,
                                  i32, i32, vp, vp, vp, vp], C.c_int),
        }
        for name, (args, res) in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib_handle = L
    return _lib_handle


def _check(status: int, what: str):
    if status != FP_OK:
        raise FastPartError(status, what)


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data


# ---------------------------------------------------------------- hypergraphs

@dataclasses.dataclass
class Hypergraph:
    """A hypergraph as the engine consumes it.

    vptr/vnets: nets of each vertex in scan order (the reference's row_ptr /
    col_ind); nptr/npins: pins of each net (row_ptr_inv / col_ind_inv); src: the
    source vertex of each net; weights: vertex weights or None (unit);
    ordering: visiting order or None (vertex ids)."""
    nov: int
    noe: int
    vptr: np.ndarray
    vnets: np.ndarray
    nptr: np.ndarray
    npins: np.ndarray
    src: np.ndarray
    weights: Optional[np.ndarray] = None
    ordering: Optional[np.ndarray] = None

    def __post_init__(self):
        self.vptr = np.ascontiguousarray(self.vptr, dtype=np.uint32)
        self.vnets = np.ascontiguousarray(self.vnets, dtype=np.uint32)
        self.nptr = np.ascontiguousarray(self.nptr, dtype=np.uint32)
        self.npins = np.ascontiguousarray(self.npins, dtype=np.uint32)
        self.src = np.ascontiguousarray(self.src, dtype=np.int32)
        if self.weights is not None:
            self.weights = np.ascontiguousarray(self.weights, dtype=np.int32)
        if self.ordering is not None:
            self.ordering = np.ascontiguousarray(self.ordering, dtype=np.int32)

    @property
    def pins(self) -> int:
        return int(self.vnets.size)

    def validate(self) -> int:
        """fp_validate status (0 when the engine accepts the hypergraph)."""
        v = self.view()
        return int(lib().fp_validate(C.byref(v)))

    def bfs_order(self, start: int) -> np.ndarray:
        """The reference's BFS visiting order (-o 1; fp_bfs_order): three BFS
        runs, from `start`, from the farthest vertex, and from the farthest
        again, listing vertices in discovery order.  The reference drivers
        start from rand() % nov (TV/tv.cpp:120).  Raises FastPartError if a
        vertex is not reached.  Host code, no GPU."""
        out = np.empty(self.nov, np.int32)
        far = np.empty(2, np.int32)
        v = self.view()
        _check(lib().fp_bfs_order(C.byref(v), int(start), _ptr(out), _ptr(far)), "fp_bfs_order")
        return out

    def thin(self, mean_factor: int, min_pins: int) -> "Hypergraph":
        """CN thinning (fp_thin_nets, the CN driver's -m 1 -n min_pins -z
        mean_factor): the hypergraph of the nets with fewer than mean_factor x
        mean and fewer than min_pins pins.  Host code."""
        g = C.c_void_p()
        v = self.view()
        _check(lib().fp_thin_nets(C.byref(v), int(mean_factor), int(min_pins), C.byref(g)), "fp_thin_nets")
        return _take_graph(g)

    def view(self) -> _Hypergraph:
        return _Hypergraph(self.nov, self.noe, self.pins, _ptr(self.vptr), _ptr(self.vnets),
                           _ptr(self.nptr), _ptr(self.npins), _ptr(self.src),
                           _ptr(self.weights), _ptr(self.ordering))

    @staticmethod
    def from_nets(nov: int, nptr, npins, src=None) -> "Hypergraph":
        """Builds vertex -> nets as the transpose of net -> pins (nets ascending
        per vertex), the orientation of the TV and CN drivers."""
        nptr = np.ascontiguousarray(nptr, dtype=np.uint32)
        npins = np.ascontiguousarray(npins, dtype=np.uint32)
        noe = nptr.size - 1
        s = None if src is None else np.ascontiguousarray(src, dtype=np.int32)
        g = C.c_void_p()
        _check(lib().fp_graph_from_nets(nov, noe, _ptr(nptr), _ptr(npins), _ptr(s), C.byref(g)),
               "fp_graph_from_nets")
        return _take_graph(g)

    @staticmethod
    def from_vertices(nov: int, noe: int, vptr, vnets, src=None) -> "Hypergraph":
        """Builds net -> pins from vertex -> nets (the reference's createInverse,
        shared/utils.cpp:32-56): the row_ptr / col_ind that partition() gets."""
        vptr = np.ascontiguousarray(vptr, dtype=np.uint32)
        vnets = np.ascontiguousarray(vnets, dtype=np.uint32)
        s = None if src is None else np.ascontiguousarray(src, dtype=np.int32)
        g = C.c_void_p()
        _check(lib().fp_graph_from_vertices(nov, noe, _ptr(vptr), _ptr(vnets), _ptr(s), C.byref(g)),
               "fp_graph_from_vertices")
        return _take_graph(g)

    def save_fphg(self, path) -> None:
        """Binary instance file read by the oracle's reference driver."""
        with open(path, "wb") as f:
            f.write(b"FPHG1\0\0\0")
            f.write(np.array([self.nov, self.noe], dtype=np.int32).tobytes())
            f.write(np.array([self.pins], dtype=np.int64).tobytes())
            for a in (self.vptr, self.vnets, self.nptr, self.npins):
                f.write(a.astype(np.uint32).tobytes())
            f.write(self.src.astype(np.int32).tobytes())

    @staticmethod
    def load_fphg(path) -> "Hypergraph":
        raw = Path(path).read_bytes()
        if raw[:5] != b"FPHG1":
            raise ValueError("not an FPHG1 file")
        nov, noe = np.frombuffer(raw, np.int32, 2, 8)
        pins = int(np.frombuffer(raw, np.int64, 1, 16)[0])
        off = 24
        arrs = []
        for n, dt in ((nov + 1, np.uint32), (pins, np.uint32), (noe + 1, np.uint32), (pins, np.uint32),
                      (noe, np.int32)):
            arrs.append(np.frombuffer(raw, dt, int(n), off).copy())
            off += 4 * int(n)
        return Hypergraph(int(nov), int(noe), *arrs)


def _take_graph(g: C.c_void_p) -> Hypergraph:
    v = _Hypergraph()
    try:
        _check(lib().fp_graph_view(g, C.byref(v)), "fp_graph_view")
        pins = v.pins

        def arr(p, n, dt):
            if n == 0:
                return np.zeros(0, dt)
            return np.ctypeslib.as_array(C.cast(p, C.POINTER(np.ctypeslib.as_ctypes_type(dt))), (n,)).copy()
        hg = Hypergraph(v.nov, v.noe, arr(v.vptr, v.nov + 1, np.uint32), arr(v.vnets, pins, np.uint32),
                        arr(v.nptr, v.noe + 1, np.uint32), arr(v.npins, pins, np.uint32),
                        arr(v.src, v.noe, np.int32),
                        arr(v.weights, v.nov, np.int32) if v.weights else None)
    finally:
        lib().fp_graph_destroy(g)
    return hg


@dataclasses.dataclass
class GenSpec:
    """Seeded synthetic hypergraph (see csrc/fp_gen.cpp)."""
    nov: int
    noe: int
    size_lo: int
    size_hi: int
    size_alpha: float = 0.0     # > 0: Zipf(alpha) sizes clipped to [lo, hi]
    pin_beta: float = 0.0       # > 0: Zipf(beta) pin popularity
    src_rule: int = 0           # 0 lowest-id pin, 1 first drawn pin
    sort_pins: int = 1
    weight_rule: int = 0        # 0 unit, 1 degree
    seed: int = 0

    @staticmethod
    def column_net(nov, noe, lo, hi, seed=0) -> "GenSpec":
        """Column-net sparse pattern: uniform sizes in [lo, hi], uniform pins,
        source = lowest-id pin, unit weights."""
        return GenSpec(nov, noe, lo, hi, 0.0, 0.0, 0, 1, 0, seed)

    @staticmethod
    def zipf(nov, noe, alpha, lo, hi, beta=0.0, weight_rule=0, seed=0) -> "GenSpec":
        """Zipf(alpha) net sizes clipped to [lo, hi]; pins by Zipf(beta)
        popularity (uniform if beta == 0); source = first drawn pin."""
        return GenSpec(nov, noe, lo, hi, alpha, beta, 1, 0, weight_rule, seed)


def generate(spec: GenSpec) -> Hypergraph:
    p = _GenParams(spec.nov, spec.noe, spec.size_lo, spec.size_hi, spec.size_alpha, spec.pin_beta,
                   spec.src_rule, spec.sort_pins, spec.weight_rule, spec.seed)
    g = C.c_void_p()
    _check(lib().fp_generate(C.byref(p), C.byref(g)), "fp_generate")
    return _take_graph(g)


def read_patohlike(path, transpose: bool = True, write_cache: bool = False) -> Hypergraph:
    """Reads a PaToH-like .hg file (and its .plbin cache, as the reference does).
    transpose=True: file lines are nets (TV, CN drivers); False: file lines are
    vertices (TM, MSM, MGV, MSRV drivers)."""
    g = C.c_void_p()
    _check(lib().fp_read_patohlike(str(path).encode(), int(transpose), int(write_cache), C.byref(g)),
           "fp_read_patohlike")
    return _take_graph(g)


def write_patohlike(hg: Hypergraph, path) -> None:
    """Writes hg's net -> pins CSR as a 0-based PaToH-like text file."""
    lines = [f"0 {hg.nov} {hg.noe} {hg.pins}"]
    for e in range(hg.noe):
        lines.append(" ".join(map(str, hg.npins[hg.nptr[e]:hg.nptr[e + 1]])))
    Path(path).write_text("\n".join(lines) + "\n")


# ---------------------------------------------------------------- engine

class Engine:
    """One GPU and one stream (fp_ctx)."""

    def __init__(self, device: int = 0):
        self._ctx = C.c_void_p()
        _check(lib().fp_ctx_create(device, C.byref(self._ctx)), "fp_ctx_create")

    def set_stream(self, stream_handle: Optional[int]) -> None:
        """Runs subsequent work on the given cudaStream_t (e.g. a torch stream's
        ``cuda_stream``); None selects the engine's own stream."""
        _check(lib().fp_ctx_set_stream(self._ctx, stream_handle), "fp_ctx_set_stream")

    def set_arena(self, nbytes: int) -> None:
        """fp_ctx_set_arena: instances of this engine take their device buffers
        from one allocation of `nbytes` (one instance at a time); 0 releases it."""
        _check(lib().fp_ctx_set_arena(self._ctx, int(nbytes)), "fp_ctx_set_arena")

    def set_sm_limit(self, sms: int) -> None:
        """fp_ctx_set_sm_limit: size this engine's grids for `sms` SMs (0: all)."""
        _check(lib().fp_ctx_set_sm_limit(self._ctx, int(sms)), "fp_ctx_set_sm_limit")

    def instance(self, hg: Hypergraph, K: int, metric, eps_factor: float = 1.05) -> "Instance":
        return Instance(self, hg, K, metric_id(metric), eps_factor)

    def create_inverse(self, nov: int, noe: int, row_ptr, col_ind):
        """fp_create_inverse on this engine's GPU: the net -> pins CSR
        (row_ptr_inv, col_ind_inv) of a vertex -> nets CSR, pins ascending per
        net (the reference's createInverse)."""
        row_ptr = np.ascontiguousarray(row_ptr, dtype=np.uint32)
        col_ind = np.ascontiguousarray(col_ind, dtype=np.uint32)
        pins = int(row_ptr[-1]) if len(row_ptr) else 0
        rp = np.empty(noe + 1, np.uint32)
        ci = np.empty(max(pins, 1), np.uint32)
        _check(lib().fp_create_inverse(self._ctx, int(nov), int(noe), pins, _ptr(row_ptr), _ptr(col_ind), _ptr(rp),
                                       _ptr(ci)), "fp_create_inverse")
        return rp, ci[:pins]

    def thin(self, hg: Hypergraph, mean_factor: int, min_pins: int) -> Hypergraph:
        """fp_thin_nets_device: Hypergraph.thin on this engine's GPU."""
        g = C.c_void_p()
        v = hg.view()
        _check(lib().fp_thin_nets_device(self._ctx, C.byref(v), int(mean_factor), int(min_pins), C.byref(g)),
               "fp_thin_nets_device")
        return _take_graph(g)

    def bfs_order(self, hg: Hypergraph, start: int, far: Optional[np.ndarray] = None) -> np.ndarray:
        """fp_bfs_order_device: Hypergraph.bfs_order on this engine's GPU; the
        two farthest vertices into `far` (2 int32) if given."""
        out = np.empty(hg.nov, np.int32)
        f = np.empty(2, np.int32) if far is None else far
        v = hg.view()
        _check(lib().fp_bfs_order_device(self._ctx, C.byref(v), int(start), _ptr(out), _ptr(f)),
               "fp_bfs_order_device")
        return out

    def close(self):
        if self._ctx:
            lib().fp_ctx_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Instance:
    """A hypergraph resident on the device with its refinement state."""

    def __init__(self, engine: Engine, hg: Hypergraph, K: int, metric: int, eps_factor: float):
        self.engine = engine
        self.hg = hg
        self.K = K
        self.metric = metric
        self._h = C.c_void_p()
        view = hg.view()
        _check(lib().fp_instance_create(engine._ctx, C.byref(view), K, metric, eps_factor,
                                        C.byref(self._h)), "fp_instance_create")

    def initial_partition(self) -> None:
        _check(lib().fp_initial_partition(self._h), "fp_initial_partition")

    def set_stream(self, where: str) -> None:
        """fp_set_stream_mode: 'auto' (the default: TV / MSV / MSRV stream on
        the device when the instance qualifies), 'host', or 'device' (TV, MSV,
        MSRV and CN on the device whenever the instance qualifies)."""
        modes = {"auto": 0, "host": 1, "device": 2}
        if where not in modes:
            raise ValueError(f"stream must be one of {sorted(modes)}")
        _check(lib().fp_set_stream_mode(self._h, modes[where], None), "fp_set_stream_mode")

    def set_stream_walk(self, on: bool) -> None:
        """fp_set_stream_walk: the device stream walks changed decisions
        inside its windows (tuning only)."""
        _check(lib().fp_set_stream_walk(self._h, int(bool(on))), "fp_set_stream_walk")

    def streamed_on_device(self) -> bool:
        """True if the last initial_partition ran on the device."""
        out = C.c_int32()
        _check(lib().fp_set_stream_mode(self._h, -1, C.byref(out)), "fp_set_stream_mode")
        return bool(out.value)

    def refine(self, passes: int) -> None:
        _check(lib().fp_refine(self._h, passes), "fp_refine")

    def set_engine(self, engine: str) -> None:
        """'auto' (speculative grid-wide engine where available) or 'sequential'
        (single-CTA walk); both give identical results."""
        _check(lib().fp_set_engine(self._h, {"auto": 0, "sequential": 1}[engine]), "fp_set_engine")

    def set_window(self, min_len: int, grow: int) -> None:
        """fp_set_window: window length after an early end (tuning only)."""
        _check(lib().fp_set_window(self._h, int(min_len), int(grow)), "fp_set_window")

    def reset_state(self) -> None:
        """Uploads the host-side stream result again (host -> device)."""
        _check(lib().fp_reset_state(self._h), "fp_reset_state")

    def state_bytes(self) -> int:
        """Bytes fp_reset_state copies host -> device."""
        K, m = self.K, self.metric
        b = 4 * (self.hg.nov + self.hg.noe + 2 * self.hg.pins) + 4 * 5 * K
        if m in (2, 3):
            words = (K + 31) // 32
            b += 4 * K * K + 4 * 4 * K * words   # conn, zero masks, conn == 1 masks
        return b

    def set_classes(self, light_work: int, super_work: int) -> None:
        """Bounds of the warp / CTA / whole-grid evaluation classes; a tuning
        knob, results are unchanged.  TV, MSV, MSRV, TM, MSM: vertex work (the
        sum over its nets of min(net size, K)); CN: net pins."""
        _check(lib().fp_set_classes(self._h, light_work, super_work), "fp_set_classes")

    def metrics(self) -> dict:
        out = np.zeros(6, np.int64)
        _check(lib().fp_metrics(self._h, _ptr(out)), "fp_metrics")
        return dict(zip(OUTPUT_ORDER, map(int, out)))

    def partition(self) -> np.ndarray:
        pv = np.empty(self.hg.nov, np.int32)
        _check(lib().fp_get_partition(self._h, _ptr(pv)), "fp_get_partition")
        return pv

    def lists(self):
        """(ep_len, ep_part, ep_cnt): the ordered per-net part lists."""
        ln = np.empty(self.hg.noe, np.int32)
        pt = np.empty(self.hg.pins, np.int32)
        ct = np.empty(self.hg.pins, np.int32)
        _check(lib().fp_get_lists(self._h, _ptr(ln), _ptr(pt), _ptr(ct)), "fp_get_lists")
        return ln, pt, ct

    STATE_FIELDS = ("part_vec", "ep_starts", "ep_ends", "ep_parts", "ep_cnt", "part_sizes", "marker", "send",
                    "recv", "conn", "msgs")

    def set_state(self, part_vec, ep_starts, ep_ends, ep_parts, ep_cnt, **optional) -> None:
        """Uploads a refinement state in the reference's layout (fp_set_state):
        ep_ends[e] is the number of parts listed for net e (lambda(e)), as the
        reference keeps it; optional: part_sizes, marker, send, recv, conn
        (K*K), msgs."""
        st, keep = _state_struct(part_vec, ep_starts, ep_ends, ep_parts, ep_cnt, **optional)
        _check(lib().fp_set_state(self._h, C.byref(st)), "fp_set_state")

    def get_state(self) -> dict:
        """Every array of fp_state, copied from the device (conn is K*K)."""
        nov, noe, P, K = self.hg.nov, self.hg.noe, self.hg.pins, self.K
        sizes = dict(part_vec=nov, ep_starts=noe, ep_ends=noe, ep_parts=P, ep_cnt=P, part_sizes=K, marker=K,
                     send=K, recv=K, conn=K * K, msgs=K)
        out = {k: np.empty(n, np.int32) for k, n in sizes.items()}
        st = FpState(**{k: v.ctypes.data for k, v in out.items()})
        _check(lib().fp_get_state(self._h, C.byref(st)), "fp_get_state")
        return out

    def part_sizes(self) -> np.ndarray:
        s = np.empty(self.K, np.int32)
        _check(lib().fp_get_part_sizes(self._h, _ptr(s)), "fp_get_part_sizes")
        return s

    def moves(self, n: int) -> np.ndarray:
        m = np.zeros(n, np.int64)
        _check(lib().fp_get_moves(self._h, _ptr(m), n), "fp_get_moves")
        return m

    def set_decision_log(self, on: bool = True) -> None:
        """fp_set_decision_log: record the decisions of each refine call's last pass."""
        _check(lib().fp_set_decision_log(self._h, int(bool(on))), "fp_set_decision_log")

    def decisions(self) -> dict:
        """fp_get_decisions: the last refine's last-pass records as int32 arrays
        dest, gain, loss, moved (one entry per vertex; per net for CN)."""
        n = self.hg.noe if metric_id(self.metric) == 0 else self.hg.nov
        out = {k: np.empty(n, np.int32) for k in ("dest", "gain", "loss", "moved")}
        _check(lib().fp_get_decisions(self._h, *(_ptr(out[k]) for k in ("dest", "gain", "loss", "moved"))),
               "fp_get_decisions")
        return out

    def debug_barrier_fault(self, leave_at: int, poll_limit: int = 0) -> None:
        """fp_debug_barrier_fault: the next refine launches' last CTA leaves at
        its leave_at-th grid barrier without arriving, and the others give up
        after poll_limit polls (0: the default limit); (0, 0) turns it off."""
        _check(lib().fp_debug_barrier_fault(self._h, int(leave_at), int(poll_limit)), "fp_debug_barrier_fault")

    def stats(self) -> dict:
        """Round statistics of the last refine on the grid-wide engine."""
        x = np.zeros(48, np.int64)
        _check(lib().fp_get_stats(self._h, _ptr(x), 48), "fp_get_stats")
        names = ["windows", "heavy_rounds", "window_moves", "cut_none", "cut_stale", "cut_size", "cut_volume",
                 "cut_maxpart", "cut_conflict", "walked"]
        d = {n: int(x[i]) for i, n in enumerate(names)}
        d.update(eval_ms=x[16] / 1e6, validate_ms=x[17] / 1e6, commit_ms=x[18] / 1e6, heavy_ms=x[19] / 1e6,
                 round_state_ms=x[20] / 1e6, warp_max_cycles=int(x[21]), cta_max_cycles=int(x[23]),
                 light_cycles=int(x[25]), light_evals=int(x[26]), cut_owncount=int(x[27]),
                 cut_setafter=int(x[28]), cta_tally_cycles=int(x[29]), cta_decide_cycles=int(x[30]),
                 cta_rest_cycles=int(x[31]), local_eval_ms=x[32] / 1e6, grid_vertex_ms=x[33] / 1e6,
                 grid_tally_ms=x[34] / 1e6, local_validate_ms=x[35] / 1e6, cta_evals=int(x[40]),
                 light_tally_cycles=int(x[41]), light_decide_cycles=int(x[42]), light_rest_cycles=int(x[43]),
                 window_fixes=int(x[44]), val_prefix_cta_ns=int(x[45]), val_light_cta_ns=int(x[46]),
                 val_rest_cta_ns=int(x[47]))
        return d

    def last_launches(self) -> int:
        x = np.zeros(1, np.int64)
        _check(lib().fp_last_launches(self._h, _ptr(x)), "fp_last_launches")
        return int(x[0])

    def device_bytes(self) -> int:
        """Bytes of the instance's device allocations (fp_instance_device_bytes)."""
        out = C.c_int64()
        _check(lib().fp_instance_device_bytes(self._h, C.byref(out)), "fp_instance_device_bytes")
        return int(out.value)

    def close(self):
        if self._h:
            lib().fp_instance_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


NOALLOC_MAX_K = 1024   # FP_NOALLOC_MAX_K


def footprint(nov: int, noe: int, pins: int, K: int, metric) -> int:
    """Device bytes an instance of these sizes allocates (fp_instance_footprint);
    no device needed."""
    out = C.c_int64()
    _check(lib().fp_instance_footprint(int(nov), int(noe), int(pins), int(K), metric_id(metric), C.byref(out)),
           "fp_instance_footprint")
    return int(out.value)


def _state_struct(part_vec, ep_starts, ep_ends, ep_parts, ep_cnt, **optional):
    """An FpState over int32 copies of the arrays (returned with it: they must
    stay alive while the struct is used)."""
    arrs = dict(part_vec=part_vec, ep_starts=ep_starts, ep_ends=ep_ends, ep_parts=ep_parts, ep_cnt=ep_cnt)
    for k, v in optional.items():
        if k not in Instance.STATE_FIELDS:
            raise TypeError(f"unknown state array {k}")
        if v is not None:
            arrs[k] = v
    keep = {k: np.ascontiguousarray(v, dtype=np.int32) for k, v in arrs.items()}
    return FpState(**{k: v.ctypes.data for k, v in keep.items()}), keep


def check_state(hg: Hypergraph, K: int, metric, part_vec, ep_starts, ep_ends, ep_parts, ep_cnt,
                eps: float = 1.05, **optional) -> None:
    """fp_check_state: raises FastPartError unless the arrays are a valid
    refinement state of hg in the reference's layout (ep_ends = lambda(e)) --
    the check set_state applies, on the host alone."""
    st, keep = _state_struct(part_vec, ep_starts, ep_ends, ep_parts, ep_cnt, **optional)
    v = hg.view()
    _check(lib().fp_check_state(C.byref(v), int(K), metric_id(metric), float(eps), C.byref(st)), "fp_check_state")


def stream_partition(hg: Hypergraph, K: int, metric, eps: float = 1.05) -> dict:
    """The metric's streaming initial partition on the host (fp_stream_partition),
    in the fp_state layout (ep_ends[e] = lambda(e), the reference's count of
    listed parts): part_vec, ep_starts, ep_ends, ep_parts, ep_cnt,
    part_sizes, marker, send, recv, conn (K*K), msgs.  No GPU needed; an
    instance takes it with set_state."""
    nov, noe, P = hg.nov, hg.noe, hg.pins
    sizes = dict(part_vec=nov, ep_starts=noe, ep_ends=noe, ep_parts=P, ep_cnt=P, part_sizes=K, marker=K,
                 send=K, recv=K, conn=K * K, msgs=K)
    out = {k: np.empty(n, np.int32) for k, n in sizes.items()}
    st = FpState(**{k: v.ctypes.data for k, v in out.items()})
    v = hg.view()
    _check(lib().fp_stream_partition(C.byref(v), int(K), metric_id(metric), float(eps), C.byref(st)),
           "fp_stream_partition")
    return out


def metrics_noalloc(K, nov, noe, pins, nptr, src, part_vec, ep_len, ep_part, out, stream=None) -> None:
    """fp_metrics_noalloc: the six metrics of a refinement state held in the
    caller's device memory, written to `out` (6 int64, device) on `stream`,
    with nothing allocated by the library.  Array arguments are device
    addresses (ints, e.g. tensor.data_ptr()); `stream` a raw CUDA stream handle
    or None for the default stream.  The call returns before the GPU is done."""
    _check(lib().fp_metrics_noalloc(K, nov, noe, pins, nptr, src, part_vec, ep_len, ep_part, out, stream),
           "fp_metrics_noalloc")


def partition_gpu(metric, row_ptr, col_ind, net_appearence, nov, noe, pins, edge_wgths, src_nodes, K,
                  ordering, f_name="", REFI_OPT=1, REFI_ITER=1, row_ptr_inv=None, col_ind_inv=None):
    """Mirror of the reference's partition_gpu(): same arguments, same stdout
    lines.  Returns (part_vec, metrics_before, metrics_after) as numpy arrays /
    dicts in the reference's print order."""
    a = lambda x, dt: None if x is None else np.ascontiguousarray(x, dtype=dt)
    row_ptr, col_ind = a(row_ptr, np.uint32), a(col_ind, np.uint32)
    net_app, ew = a(net_appearence, np.uint32), a(edge_wgths, np.int32)
    srcs, order = a(src_nodes, np.int32), a(ordering, np.int32)
    rpi, cii = a(row_ptr_inv, np.uint32), a(col_ind_inv, np.uint32)
    pv = np.empty(nov, np.int32)
    mo = np.zeros(12, np.int64)
    _check(lib().fp_partition_gpu(metric_id(metric), _ptr(row_ptr), _ptr(col_ind), _ptr(net_app), nov, noe,
                                  pins, _ptr(ew), _ptr(srcs), K, _ptr(order), str(f_name).encode(), REFI_OPT,
                                  REFI_ITER, _ptr(rpi), _ptr(cii), _ptr(pv), _ptr(mo)), "fp_partition_gpu")
    return pv, dict(zip(OUTPUT_ORDER, map(int, mo[:6]))), dict(zip(OUTPUT_ORDER, map(int, mo[6:])))
