"""ctypes wrapper of the CPU oracle (oracle/liboracle.so) - test infrastructure."""
import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "oracle", "liboracle.so")
NODE_FIELDS = ("xb", "yb", "zb", "phix", "phiy", "phiz", "dtau", "expmod")
_lib = None


def load():
    global _lib
    if _lib is None:
        src = os.path.join(ROOT, "oracle", "thesis_oracle.cpp")
        if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
            subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
        L = ctypes.CDLL(LIB)
        vp = ctypes.c_void_p
        L.or_load.restype = vp
        L.or_load.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int]
        L.or_free.argtypes = [vp]
        L.or_info.argtypes = [vp, vp]
        L.or_snapshot_time.argtypes = [vp, ctypes.c_int]
        L.or_snapshot_time.restype = ctypes.c_double
        L.or_nodes.argtypes = [vp, ctypes.c_double, ctypes.c_int, vp, ctypes.c_int]
        L.or_calc_T.argtypes = [vp, ctypes.c_double, vp, ctypes.c_int64, vp, ctypes.c_int]
        L.or_snapshot.argtypes = [vp, ctypes.c_int, vp, ctypes.c_int]
        L.or_solidify.argtypes = [vp, ctypes.c_int, ctypes.c_int64]
        L.or_solidify.restype = ctypes.c_int64
        L.or_solidify_budget.argtypes = [vp, ctypes.c_int, ctypes.c_int64, ctypes.c_double]
        L.or_solidify_budget.restype = ctypes.c_int64
        L.or_field.argtypes = [vp, ctypes.c_char_p, vp]
        L.or_solid_fields.argtypes = [vp, ctypes.c_int64, ctypes.c_double, vp]
        L.or_solid_fields_many.argtypes = [vp, vp, vp, ctypes.c_int64, vp, ctypes.c_int]
        L.or_schedule.argtypes = [vp, ctypes.c_double, ctypes.c_int]
        L.or_schedule.restype = ctypes.c_uint64
        L.or_schedule_many.argtypes = [vp, vp, ctypes.c_int64, ctypes.c_int, vp, ctypes.c_int]
        L.or_rdf.argtypes = [vp, vp, vp, vp, ctypes.c_int64]
        L.or_rdf.restype = ctypes.c_int64
        L.or_rrdf.argtypes = [vp, vp, vp, vp, ctypes.c_int64]
        L.or_rrdf.restype = ctypes.c_int64
        L.or_pairs.argtypes = [vp]
        L.or_pairs.restype = ctypes.c_int64
        _lib = L
    return Oracle


class Oracle:
    def __init__(self, param_input):
        load()
        err = ctypes.create_string_buffer(512)
        self.h = _lib.or_load(os.fspath(param_input).encode(), err, 512)
        if not self.h:
            raise RuntimeError(err.value.decode())
        info = np.zeros(16)
        _lib.or_info(self.h, info.ctypes.data_as(ctypes.c_void_p))
        self.nx, self.ny, self.nz, self.pnum = (int(v) for v in info[:4])
        self.n_snapshots = int(info[5])
        self.end_time = info[9]
        self.T0, self.TL = info[10], info[11]

    def __del__(self):
        if getattr(self, "h", None):
            _lib.or_free(self.h)
            self.h = None

    def snapshot_time(self, i):
        return _lib.or_snapshot_time(self.h, i)

    def nodes(self, t, is_sol=False):
        cap = 4096
        while True:
            buf = np.zeros((8, cap))
            n = _lib.or_nodes(self.h, float(t), int(is_sol), buf.ctypes.data_as(ctypes.c_void_p), cap)
            if n <= cap:
                return {f: buf[i, :n].copy() for i, f in enumerate(NODE_FIELDS)}
            cap = n

    def calc_T(self, t, pts, threads=0):
        p = np.ascontiguousarray(pts, dtype=np.int64)
        out = np.empty(p.size)
        _lib.or_calc_T(self.h, float(t), p.ctypes.data_as(ctypes.c_void_p), p.size,
                       out.ctypes.data_as(ctypes.c_void_p), threads)
        return out

    def snapshot(self, i, threads=0):
        out = np.empty(self.pnum)
        _lib.or_snapshot(self.h, i, out.ctypes.data_as(ctypes.c_void_p), threads)
        return out

    def solidify(self, threads=0, max_steps=0, budget_s=0.0):
        """Steps taken; stops at the finish test, after max_steps (> 0) or after the first
        step ending more than budget_s (> 0) seconds after the start."""
        return _lib.or_solidify_budget(self.h, threads, max_steps, float(budget_s))

    def field(self, name):
        out = np.empty(self.pnum)
        rc = _lib.or_field(self.h, name.encode(), out.ctypes.data_as(ctypes.c_void_p))
        if rc:
            raise KeyError(name)
        return out

    SOLID = ("G", "Gx", "Gy", "Gz", "dTdt", "V", "eqFrac", "dTdt_raw", "dTdt_mag", "G_mag")

    def solid_fields(self, p, tsol):
        out = np.zeros(10)
        _lib.or_solid_fields(self.h, int(p), float(tsol), out.ctypes.data_as(ctypes.c_void_p))
        return dict(zip(self.SOLID, out))

    def solid_fields_many(self, pts, tsol, threads=0):
        """The fields of Grid::Solidify at each point's given solidification time: a dict of
        arrays (G ... eqFrac, then dTdt_raw = a lap + dT_t before its truncation, and the
        magnitudes dTdt_mag, G_mag of the terms the cooling rate and the gradient sum)."""
        p = np.ascontiguousarray(pts, dtype=np.int64)
        t = np.ascontiguousarray(tsol, dtype=np.float64)
        out = np.zeros((p.size, 10))
        _lib.or_solid_fields_many(self.h, p.ctypes.data_as(ctypes.c_void_p), t.ctypes.data_as(ctypes.c_void_p),
                                  p.size, out.ctypes.data_as(ctypes.c_void_p), threads)
        return {f: out[:, i].copy() for i, f in enumerate(self.SOLID)}

    def schedule(self, t, is_sol=False, threads=0):
        """Signature of the quadrature walk's discrete choices at each time in t."""
        tt = np.ascontiguousarray(np.atleast_1d(t), dtype=np.float64)
        out = np.zeros(tt.size, dtype=np.uint64)
        _lib.or_schedule_many(self.h, tt.ctypes.data_as(ctypes.c_void_p), tt.size, int(is_sol),
                              out.ctypes.data_as(ctypes.c_void_p), threads)
        return out

    def rdf(self):
        """After a run with Output RDF 1: (counts (pnum, 3) int32 - per point the numbers of
        melting times, solidification times and cooling rates -, vals - all values, per point
        its melting times, then solidification times, then cooling rates -, dT - per
        solidification time its secant's T - T_last)."""
        n = _lib.or_rdf(self.h, None, None, None, 0)
        counts = np.zeros((self.pnum, 3), dtype=np.int32)
        vals = np.zeros(max(n, 0))
        dT = np.zeros(max(n, 0))
        _lib.or_rdf(self.h, counts.ctypes.data_as(ctypes.c_void_p), vals.ctypes.data_as(ctypes.c_void_p),
                    dT.ctypes.data_as(ctypes.c_void_p), n)
        return counts, vals, dT[:int(counts[:, 1].sum())]

    def rrdf(self):
        """After a Stork run: (idx (n, 3) uint32, ts (n, 2), Ts (n, 16)), the rows in the
        reference's single-thread order."""
        n = _lib.or_rrdf(self.h, None, None, None, 0)
        idx = np.zeros((n, 3), dtype=np.uint32)
        ts, Ts = np.zeros((n, 2)), np.zeros((n, 16))
        _lib.or_rrdf(self.h, idx.ctypes.data_as(ctypes.c_void_p), ts.ctypes.data_as(ctypes.c_void_p),
                     Ts.ctypes.data_as(ctypes.c_void_p), n)
        return idx, ts, Ts

    @property
    def pairs(self):
        return _lib.or_pairs(self.h)
