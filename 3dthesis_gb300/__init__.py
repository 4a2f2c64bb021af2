"""GB300 (sm_103a) implementation of 3DThesis's hot path, driven through its C ABI.

The package is a thin ctypes layer over ``libthesis_gb300.so`` (declared in
``include/thesis_gb300.h``).  Its ``Simulation`` class mirrors the reference's
operator interface for the path:

=======================  ==================================================================
``Simulation(deck)``     Init::GetFileNames + Init::ReadSimParams + Grid(sim)
``integrate(t, is_sol)`` Calc::Integrate_Serial -> the node fields xb ... expmod
``calc_T(t, pts)``       Grid::Calc_T (set = false) at many points
``snapshot(i)``          one snapshot of Run::Snapshots_NoTracking
``solidify()``           Run::Solidify (Tracking None / Volume / Surface)
``field(name)``          Grid getters (T, tSol, G, V, Gx, Gy, Gz, dTdt, eqFrac, ...)
``simulate()``           Run::Simulate plus the CSV outputs of the reference CLI
=======================  ==================================================================

There is no CPU fallback: if the library is missing or no GPU is present the calls
raise ``ThesisError``.
"""
from __future__ import annotations

import ctypes
import os
from typing import Dict, Optional, Sequence

import numpy as np

from . import decks  # noqa: F401  (re-exported workload definitions)

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libthesis_gb300.so")
CLI_PATH = os.path.join(_HERE, "thesis_gb300")

FP64 = 0
FP32_KAHAN = 1
_PRECISIONS = {"fp64": FP64, "fp32": FP32_KAHAN, "fp32_kahan": FP32_KAHAN, FP64: FP64, FP32_KAHAN: FP32_KAHAN}

NODE_FIELDS = ("xb", "yb", "zb", "phix", "phiy", "phiz", "dtau", "expmod")
FIELDS = ("T", "tSol", "G", "V", "Gx", "Gy", "Gz", "dTdt", "eqFrac", "numMelt", "depth", "output_flag")
EXPORTED = ("th_ctx_create_from_deck", "th_ctx_destroy", "th_last_error", "th_get_info", "th_snapshot_time",
            "th_nodes", "th_calc_T", "th_calc_T_device", "th_snapshot", "th_solidify", "th_field",
            "th_simulate", "th_pairs", "th_set_tile_shape", "th_last_kernel_ms", "th_sync",
            "th_calc_T_noalloc", "th_run_stats", "th_run_reset", "th_autotune",
            "th_batch_create", "th_batch_destroy", "th_batch_last_error", "th_batch_points", "th_batch_snapshot",
            "th_batch_snapshot_device", "th_batch_set_tile_shape", "th_batch_autotune", "th_batch_pairs",
            "th_adj_create", "th_adj_destroy", "th_adj_last_error", "th_adj_num_params", "th_adj_params",
            "th_adj_host_nodes", "th_adj_forward", "th_adj_backward", "th_calc_T_times_device",
            "th_device_rates", "th_rrdf", "th_rdf", "th_deck_info", "th_output_rrdf", "th_T_hist")


class ThesisError(RuntimeError):
    """A th_* call returned a non-zero status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"[status {status}] {message}")
        self.status = status


class Info(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
                ("pnum", ctypes.c_int64), ("n_beams", ctypes.c_int32), ("n_snapshots", ctypes.c_int32),
                ("mode", ctypes.c_int32), ("tracking", ctypes.c_int32), ("dt", ctypes.c_double),
                ("end_time", ctypes.c_double), ("T0", ctypes.c_double), ("TL", ctypes.c_double),
                ("xmin", ctypes.c_double), ("xmax", ctypes.c_double), ("ymin", ctypes.c_double),
                ("ymax", ctypes.c_double), ("zmin", ctypes.c_double), ("zmax", ctypes.c_double),
                ("precision", ctypes.c_int32), ("out_flags", ctypes.c_int32)]


_lib: Optional[ctypes.CDLL] = None


def load_library(path: str = LIB_PATH) -> ctypes.CDLL:
    """Loads the C-ABI library (built in-tree by ``__graft_entry__.build()``)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ThesisError(-1, f"{path} is missing: build it with __graft_entry__.build()")
    L = ctypes.CDLL(path)
    vp, c_int, c_i64, c_d = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_double
    L.th_ctx_create_from_deck.argtypes = [ctypes.c_char_p, c_int, ctypes.POINTER(vp)]
    L.th_ctx_destroy.argtypes = [vp]
    L.th_ctx_destroy.restype = None
    L.th_last_error.argtypes = [vp]
    L.th_last_error.restype = ctypes.c_char_p
    L.th_get_info.argtypes = [vp, ctypes.POINTER(Info)]
    L.th_snapshot_time.argtypes = [vp, c_int]
    L.th_snapshot_time.restype = c_d
    L.th_nodes.argtypes = [vp, c_d, c_int, vp, c_int, ctypes.POINTER(c_int)]
    L.th_calc_T.argtypes = [vp, c_d, vp, c_i64, vp]
    L.th_calc_T_device.argtypes = [vp, c_d, vp, c_i64, vp, vp]
    L.th_sync.argtypes = [vp, vp]
    L.th_calc_T_times_device.argtypes = [vp, vp, c_int, vp, c_i64, vp, vp]
    L.th_calc_T_noalloc.argtypes = [vp, c_d, vp, c_i64, vp, vp]
    L.th_run_stats.argtypes = [vp, vp, c_int]
    L.th_run_reset.argtypes = [vp]
    L.th_snapshot.argtypes = [vp, c_int, vp]
    L.th_solidify.argtypes = [vp, c_i64, ctypes.POINTER(c_i64)]
    L.th_field.argtypes = [vp, ctypes.c_char_p, vp]
    L.th_simulate.argtypes = [vp]
    L.th_pairs.argtypes = [vp, ctypes.POINTER(c_i64)]
    L.th_set_tile_shape.argtypes = [vp, c_int, c_int]
    L.th_last_kernel_ms.argtypes = [vp, ctypes.POINTER(ctypes.c_float)]
    L.th_autotune.argtypes = [vp, c_int, ctypes.POINTER(c_int), ctypes.POINTER(c_int)]
    L.th_batch_create.argtypes = [ctypes.POINTER(ctypes.c_char_p), c_int, c_int, ctypes.POINTER(vp)]
    L.th_batch_destroy.argtypes = [vp]
    L.th_batch_destroy.restype = None
    L.th_batch_last_error.argtypes = [vp]
    L.th_batch_last_error.restype = ctypes.c_char_p
    L.th_batch_points.argtypes = [vp, vp]
    L.th_batch_snapshot.argtypes = [vp, c_int, vp]
    L.th_batch_snapshot_device.argtypes = [vp, c_int, vp, vp]
    L.th_batch_set_tile_shape.argtypes = [vp, c_int, c_int]
    L.th_batch_autotune.argtypes = [vp, c_int, ctypes.POINTER(c_int), ctypes.POINTER(c_int)]
    L.th_batch_pairs.argtypes = [vp, ctypes.POINTER(c_i64)]
    L.th_adj_create.argtypes = [ctypes.c_char_p, c_int, vp, c_int, vp, c_int, ctypes.POINTER(vp)]
    L.th_adj_destroy.argtypes = [vp]
    L.th_adj_destroy.restype = None
    L.th_adj_last_error.argtypes = [vp]
    L.th_adj_last_error.restype = ctypes.c_char_p
    L.th_adj_num_params.argtypes = [vp]
    L.th_adj_params.argtypes = [vp, vp]
    L.th_adj_host_nodes.argtypes = [vp, vp, c_int, vp, c_int, vp, ctypes.POINTER(c_int)]
    L.th_adj_forward.argtypes = [vp, vp, vp]
    L.th_adj_backward.argtypes = [vp, vp, vp]
    L.th_device_rates.argtypes = [vp]
    L.th_rrdf.argtypes = [vp, vp, vp, vp, c_i64, ctypes.POINTER(c_i64)]
    L.th_rdf.argtypes = [vp, vp, vp, c_i64, ctypes.POINTER(c_i64)]
    L.th_output_rrdf.argtypes = [vp, ctypes.c_char_p, c_int]
    L.th_T_hist.argtypes = [vp, vp, vp, c_i64, ctypes.POINTER(c_i64)]
    L.th_deck_info.argtypes = [ctypes.c_char_p, ctypes.POINTER(Info)]
    _lib = L
    return L


def device_rates() -> Dict[str, float]:
    """Measured issue rates of the current CUDA device: SM count, maximum SM clock (MHz),
    MUFU ex2 results and FP32 FMA lane-operations per SM per clock."""
    L = load_library()
    out = np.zeros(4)
    st = L.th_device_rates(out.ctypes.data_as(ctypes.c_void_p))
    if st != 0:
        raise ThesisError(st, L.th_last_error(None).decode())
    return {"sm_count": int(out[0]), "sm_max_mhz": float(out[1]), "ex2_per_sm_clk": float(out[2]),
            "fma_per_sm_clk": float(out[3])}


def deck_info(param_input: str) -> Dict[str, float]:
    """A deck's grid, mode and timing summary from host parsing alone (no context, no GPU):
    th_deck_info."""
    L = load_library()
    info = Info()
    st = L.th_deck_info(os.fspath(param_input).encode(), ctypes.byref(info))
    if st != 0:
        raise ThesisError(st, L.th_last_error(None).decode())
    return {f: getattr(info, f) for f, _ in Info._fields_}


def deck_weight(param_input: str) -> float:
    """Work estimate of a deck for splitting decks across GPUs: points times snapshots
    (Snapshots mode) or times timesteps (Solidification mode)."""
    d = deck_info(param_input)
    if d["mode"] == 0:
        return float(d["pnum"]) * max(1, d["n_snapshots"])
    return float(d["pnum"]) * max(1.0, d["end_time"] / d["dt"]) if d["dt"] > 0 else float(d["pnum"])


def shard_decks(paths, rank: int, world: int, weights=None) -> list:
    """The indices of the decks rank `rank` of `world` runs, in ascending order: decks are
    dealt heaviest first to the least-loaded rank (ties to the lower rank, equal weights in
    input order), so every rank computes the same partition from the same list and the
    ranks exchange nothing.  Weights default to deck_weight."""
    if not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    w = [deck_weight(p) for p in paths] if weights is None else [float(x) for x in weights]
    load = [0.0] * world
    mine = []
    for i in sorted(range(len(w)), key=lambda i: (-w[i], i)):
        r = min(range(world), key=lambda q: (load[q], q))
        load[r] += w[i]
        if r == rank:
            mine.append(i)
    return sorted(mine)


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class Simulation:
    """One deck on one GPU (the context is bound to the current CUDA device)."""

    def __init__(self, param_input: str, precision="fp32"):
        self._lib = load_library()
        self._ctx = ctypes.c_void_p()
        prec = _PRECISIONS[precision]
        st = self._lib.th_ctx_create_from_deck(os.fspath(param_input).encode(), prec, ctypes.byref(self._ctx))
        if st != 0:
            raise ThesisError(st, self._lib.th_last_error(None).decode())
        self.precision = prec
        inf = Info()
        self._check(self._lib.th_get_info(self._ctx, ctypes.byref(inf)))
        self.info: Dict[str, object] = {f: getattr(inf, f) for f, _ in Info._fields_}

    # ------------------------------------------------------------------ plumbing
    def _check(self, st: int):
        if st != 0:
            raise ThesisError(st, self._lib.th_last_error(self._ctx).decode())

    def close(self):
        if self._ctx:
            self._lib.th_ctx_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> int:
        return self._ctx.value

    @property
    def pnum(self) -> int:
        return int(self.info["pnum"])

    @property
    def snapshot_times(self):
        return [self._lib.th_snapshot_time(self._ctx, i) for i in range(int(self.info["n_snapshots"]))]

    # ------------------------------------------------------------------ hot path
    def integrate(self, t: float, is_sol: bool = False) -> Dict[str, np.ndarray]:
        """Quadrature nodes at t, as the reference's Nodes fields."""
        cap = 4096
        while True:
            buf = np.zeros((8, cap))
            n = ctypes.c_int32()
            self._check(self._lib.th_nodes(self._ctx, float(t), int(bool(is_sol)), _ptr(buf), cap, ctypes.byref(n)))
            if n.value <= cap:
                return {f: buf[i, :n.value].copy() for i, f in enumerate(NODE_FIELDS)}
            cap = n.value

    def calc_T(self, t: float, pts: Optional[np.ndarray] = None) -> np.ndarray:
        """T at flat point ids (k fastest); all points when pts is None."""
        if pts is None:
            out = np.empty(self.pnum)
            self._check(self._lib.th_calc_T(self._ctx, float(t), None, self.pnum, _ptr(out)))
            return out
        p = np.ascontiguousarray(pts, dtype=np.int64)
        out = np.empty(p.size)
        self._check(self._lib.th_calc_T(self._ctx, float(t), _ptr(p), p.size, _ptr(out)))
        return out

    def calc_T_device(self, t: float, d_pts: int, n: int, d_T: int, stream: int = 0):
        """Device-pointer form (integers are raw CUDA addresses, e.g. tensor.data_ptr())."""
        self._check(self._lib.th_calc_T_device(self._ctx, float(t), ctypes.c_void_p(d_pts or None), int(n),
                                               ctypes.c_void_p(d_T), ctypes.c_void_p(stream or None)))

    def calc_T_noalloc(self, t: float, d_pts: int, n: int, d_T: int, stream: int = 0):
        """Like calc_T_device, but the node list uses the library's static device array
        instead of memory the context allocates; never allocates device memory."""
        self._check(self._lib.th_calc_T_noalloc(self._ctx, float(t), ctypes.c_void_p(d_pts or None), int(n),
                                                ctypes.c_void_p(d_T), ctypes.c_void_p(stream or None)))

    def calc_T_times_device(self, times, d_pts: int, n: int, d_T: int, stream: int = 0):
        """T at every time of ``times`` into device memory d_T (len(times) x n doubles)."""
        t = np.ascontiguousarray(times, dtype=np.float64)
        self._check(self._lib.th_calc_T_times_device(self._ctx, _ptr(t), t.size, ctypes.c_void_p(d_pts or None),
                                                     int(n), ctypes.c_void_p(d_T), ctypes.c_void_p(stream or None)))

    def sync(self, stream: int = 0):
        self._check(self._lib.th_sync(self._ctx, ctypes.c_void_p(stream or None)))

    def snapshot(self, idx: int, out: Optional[np.ndarray] = None, copy: bool = True) -> Optional[np.ndarray]:
        if copy and out is None:
            out = np.empty(self.pnum)
        self._check(self._lib.th_snapshot(self._ctx, int(idx), _ptr(out) if copy else None))
        return out

    def solidify(self, max_steps: int = 0) -> int:
        steps = ctypes.c_int64()
        self._check(self._lib.th_solidify(self._ctx, int(max_steps), ctypes.byref(steps)))
        return steps.value

    def reset(self):
        """Discards the solidification state; the next solidify() starts at t = 0."""
        self._check(self._lib.th_run_reset(self._ctx))

    def run_stats(self) -> Dict[str, float]:
        """Device time (ms) and counters of the solidification loop so far."""
        out = np.zeros(34)
        self._check(self._lib.th_run_stats(self._ctx, _ptr(out), 34))
        keys = ("ms_nodes", "ms_track", "ms_solidify", "windows", "records", "max_items", "steps", "slot_cap",
                "ms_device", "pairs_solidify", "pairs_total", "loop_ms_work", "loop_ms_barrier", "loop_items",
                "loop_item_clocks", "loop_wait_clocks", "loop_depth_sum", "loop_steps", "loop_evals",
                "loop_eval_clocks", "loop_ms_start0", "loop_ms_start1", "loop_ms_start2", "loop_ms_start3",
                "loop_ms_end0", "loop_ms_end1", "loop_ms_end2", "loop_ms_end3", "loop_eval_nodes",
                "records_redone_fp64", "guarded_decisions", "ms_rrdf", "rrdf_rows", "records_fixed_fp64")
        return dict(zip(keys, out.tolist()))

    def rdf(self):
        """After solidify() on a deck with Output RDF 1: (counts (pnum, 3) int32 - per point its
        numbers of melting times, solidification times and cooling rates -, vals - point by
        point its melting times, then solidification times, then cooling rates)
        (Grid::get_RDF_tm / _tl / _cr, src/Grid.h:360-362)."""
        n = ctypes.c_int64()
        counts = np.zeros((self.pnum, 3), dtype=np.int32)
        self._check(self._lib.th_rdf(self._ctx, _ptr(counts), None, 0, ctypes.byref(n)))
        vals = np.zeros(n.value)
        self._check(self._lib.th_rdf(self._ctx, None, _ptr(vals), n.value, ctypes.byref(n)))
        return counts, vals

    def rrdf(self):
        """After solidify() on a Stork deck: the doubly reduced data, (idx (n, 3) uint32,
        ts (n, 2), Ts (n, 16)) - per row the cell index, the previous and current step time
        and the 8 vertex temperatures at each (Grid::get_RRDF_*, src/Grid.h:368-370)."""
        n = ctypes.c_int64()
        self._check(self._lib.th_rrdf(self._ctx, None, None, None, 0, ctypes.byref(n)))
        idx = np.zeros((n.value, 3), dtype=np.uint32)
        ts, Ts = np.zeros((n.value, 2)), np.zeros((n.value, 16))
        self._check(self._lib.th_rrdf(self._ctx, _ptr(idx), _ptr(ts), _ptr(Ts), n.value, ctypes.byref(n)))
        return idx, ts, Ts

    def T_hist(self):
        """With Output T_hist 1 (Tracking None), after simulate() or solidify(): the
        evaluation times (n,) and every point's temperature at each, (n, pnum)
        (Grid::get_t_hist / get_T_hist, src/Grid.h:357-358)."""
        n = ctypes.c_int64()
        self._check(self._lib.th_T_hist(self._ctx, None, None, 0, ctypes.byref(n)))
        t, T = np.zeros(n.value), np.zeros((n.value, self.pnum))
        self._check(self._lib.th_T_hist(self._ctx, _ptr(t), _ptr(T), n.value, ctypes.byref(n)))
        return t, T

    def output_rrdf(self, name: str = "RRDF", binary: bool = False):
        """After solidify() on a Stork deck: writes the doubly reduced data to
        <deck dir>/Data/<deck name>.<name>.csv or .bin (Grid::Output_RRDF_csv / _bin,
        src/Grid.cpp:203-273)."""
        self._check(self._lib.th_output_rrdf(self._ctx, name.encode(), 1 if binary else 0))

    def field(self, name: str) -> np.ndarray:
        out = np.empty(self.pnum)
        self._check(self._lib.th_field(self._ctx, name.encode(), _ptr(out)))
        return out

    def simulate(self):
        self._check(self._lib.th_simulate(self._ctx))

    @property
    def pairs(self) -> int:
        v = ctypes.c_int64()
        self._check(self._lib.th_pairs(self._ctx, ctypes.byref(v)))
        return v.value

    def set_tile_shape(self, kp: int, kch: int):
        self._check(self._lib.th_set_tile_shape(self._ctx, int(kp), int(kch)))

    @property
    def last_kernel_ms(self) -> float:
        v = ctypes.c_float()
        self._check(self._lib.th_last_kernel_ms(self._ctx, ctypes.byref(v)))
        return v.value

    def autotune(self, idx: int = 0):
        """Times every tile shape on snapshot idx, keeps the fastest and returns it."""
        kp, kch = ctypes.c_int32(), ctypes.c_int32()
        self._check(self._lib.th_autotune(self._ctx, int(idx), ctypes.byref(kp), ctypes.byref(kch)))
        return kp.value, kch.value


class Batch:
    """Many Snapshots decks evaluated together (a process-parameter sweep) on the current
    CUDA device.  A batch snapshot returns one flat array; deck d's grid is
    ``T[offsets[d]:offsets[d + 1]]`` in the deck's own point order."""

    def __init__(self, param_inputs: Sequence[str], precision="fp32"):
        self._lib = load_library()
        self._b = ctypes.c_void_p()
        names = [os.fspath(p).encode() for p in param_inputs]
        arr = (ctypes.c_char_p * len(names))(*names)
        st = self._lib.th_batch_create(arr, len(names), _PRECISIONS[precision], ctypes.byref(self._b))
        if st != 0:
            raise ThesisError(st, self._lib.th_batch_last_error(None).decode())
        self.n = len(names)
        self.offsets = np.zeros(self.n + 1, dtype=np.int64)
        self._check(self._lib.th_batch_points(self._b, _ptr(self.offsets)))

    def _check(self, st: int):
        if st != 0:
            raise ThesisError(st, self._lib.th_batch_last_error(self._b).decode())

    def close(self):
        if self._b:
            self._lib.th_batch_destroy(self._b)
            self._b = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def pnum(self) -> int:
        return int(self.offsets[-1])

    def snapshot(self, idx: int, out: Optional[np.ndarray] = None) -> np.ndarray:
        if out is None:
            out = np.empty(self.pnum)
        self._check(self._lib.th_batch_snapshot(self._b, int(idx), _ptr(out)))
        return out

    def snapshot_device(self, idx: int, d_T: int, stream: int = 0):
        self._check(self._lib.th_batch_snapshot_device(self._b, int(idx), ctypes.c_void_p(d_T),
                                                       ctypes.c_void_p(stream or None)))

    def set_tile_shape(self, kp: int, kch: int):
        self._check(self._lib.th_batch_set_tile_shape(self._b, int(kp), int(kch)))

    def autotune(self, idx: int = 0):
        kp, kch = ctypes.c_int32(), ctypes.c_int32()
        self._check(self._lib.th_batch_autotune(self._b, int(idx), ctypes.byref(kp), ctypes.byref(kch)))
        return kp.value, kch.value

    @property
    def pairs(self) -> int:
        v = ctypes.c_int64()
        self._check(self._lib.th_batch_pairs(self._b, ctypes.byref(v)))
        return v.value


PARAM_NAMES = ("P", "eta", "Width_X", "Width_Y", "Depth_Z", "alpha")


class Adjoint:
    """Probe temperatures of a single-beam deck as a differentiable function of
    theta = (P, efficiency, Width_X, Width_Y, Depth_Z, alpha, x1, y1, x2, y2, ...) - the path
    vertices after the origin, in metres - and their gradient (``backward``)."""

    def __init__(self, param_input: str, probes: np.ndarray, times: Sequence[float], precision="fp32"):
        self._lib = load_library()
        self._a = ctypes.c_void_p()
        self.probes = np.ascontiguousarray(probes, dtype=np.int64)
        self.times = np.ascontiguousarray(times, dtype=np.float64)
        st = self._lib.th_adj_create(os.fspath(param_input).encode(), _PRECISIONS[precision], _ptr(self.probes),
                                     self.probes.size, _ptr(self.times), self.times.size, ctypes.byref(self._a))
        if st != 0:
            raise ThesisError(st, self._lib.th_adj_last_error(None).decode())
        self.num_params = int(self._lib.th_adj_num_params(self._a))

    def _check(self, st: int):
        if st != 0:
            raise ThesisError(st, self._lib.th_adj_last_error(self._a).decode())

    def close(self):
        if self._a:
            self._lib.th_adj_destroy(self._a)
            self._a = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> np.ndarray:
        th = np.empty(self.num_params)
        self._check(self._lib.th_adj_params(self._a, _ptr(th)))
        return th

    def host_nodes(self, theta: np.ndarray, time_idx: int, tangents: bool = False):
        """(values[8, n], tangents[8, n, num_params] or None) of the node list at times[time_idx]."""
        theta = np.ascontiguousarray(theta, dtype=np.float64)
        n = ctypes.c_int32()
        self._check(self._lib.th_adj_host_nodes(self._a, _ptr(theta), int(time_idx), None, 0, None, ctypes.byref(n)))
        cap = max(1, n.value)
        vals = np.zeros((8, cap))
        tan = np.zeros((8, cap, self.num_params)) if tangents else None
        self._check(self._lib.th_adj_host_nodes(self._a, _ptr(theta), int(time_idx), _ptr(vals), cap,
                                                _ptr(tan) if tangents else None, ctypes.byref(n)))
        return vals[:, :n.value], (tan[:, :n.value] if tangents else None)

    def forward(self, theta: np.ndarray) -> np.ndarray:
        theta = np.ascontiguousarray(theta, dtype=np.float64)
        out = np.empty((self.times.size, self.probes.size))
        self._check(self._lib.th_adj_forward(self._a, _ptr(theta), _ptr(out)))
        return out

    def backward(self, dL_dT: np.ndarray) -> np.ndarray:
        g = np.ascontiguousarray(dL_dT, dtype=np.float64).reshape(self.times.size, self.probes.size)
        out = np.empty(self.num_params)
        self._check(self._lib.th_adj_backward(self._a, _ptr(g), _ptr(out)))
        return out


def probe_temperatures(adj: "Adjoint", theta):
    """torch.autograd entry: T[times, probes] = f(theta) with the gradient from the adjoint
    kernel.  theta is a float64 torch tensor of adj.num_params entries."""
    import torch

    class _ProbeT(torch.autograd.Function):
        @staticmethod
        def forward(ctx, th):
            T = adj.forward(th.detach().cpu().numpy())
            return torch.from_numpy(T).to(th.device)

        @staticmethod
        def backward(ctx, grad_T):
            g = adj.backward(grad_T.detach().cpu().numpy())
            return torch.from_numpy(g).to(grad_T.device)

    return _ProbeT.apply(theta)
