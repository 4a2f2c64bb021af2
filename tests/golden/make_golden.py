"""Generate the golden fixtures in this directory from the UNMODIFIED reference.

Run from the repository root, on a machine holding the 3DThesis sources:

    make -C oracle ref REF=/path/to/3DThesis     # builds oracle/_ref/libthesis_ref.so
    python tests/golden/make_golden.py

Each deck is written to a scratch directory and loaded by the reference library in its
own process (the reference keeps function-static state).  The fixtures hold:

* ``nodes_<deck>.npz``  - quadrature node lists (8 fields) at the deck's snapshot times,
  plus ``is_sol`` lists at the same times (Calc::Integrate_Serial).
* ``temp_snapshot_raster.npz`` - T at 4096 seeded points of the 200x100x40 raster grid at
  its three snapshot times (Grid::Calc_T with set = false).
* ``run_<deck>.npz`` - a full Run::Simulate on a small solidification deck: the packed
  molten-point mask, per-field checksums over all output points, and every output
  field at a seeded subset of 1500 output points.
  The ``*_rdf`` runs (Output RDF 1) also hold every melting time, solidification time and
  cooling rate of every point (Grid::get_RDF_*) and the reference's ``RDF.Final`` file.
* ``csv_<deck>.npz`` - the reference's own output files (Grid::Output) of a whole run of
  a small Snapshots deck and a small Solidification deck, byte for byte: ``names`` and
  ``file<i>`` (the file's bytes).

* ``rrdf_<deck>.npz`` - a whole Stork run (Tracking Stork): the row count, the number of
  steps with rows and a SHA-256 digest of the doubly reduced data (cell indices, step
  times, vertex temperatures; the reference run with one thread, so rows come in cell
  order within a step); the first deck's fixture also holds the reference's own
  ``<name>.RRDF.csv`` (Grid::Output_RRDF_csv) byte for byte.

``python tests/golden/make_golden.py csv`` (or ``comp``, ``rdf``, ``rrdf``) regenerates only
the csv (or the path-compression, the RDF, the Stork) fixtures.
"""
from __future__ import annotations

import importlib
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
decks = importlib.import_module("3dthesis_gb300.decks")
REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libthesis_ref.so")

_CHILD = r"""
import ctypes, sys, numpy as np
L = ctypes.CDLL(sys.argv[1]); L.ref_load.restype = ctypes.c_void_p
L.ref_snapshot_time.restype = ctypes.c_double
job = dict(np.load(sys.argv[3], allow_pickle=True))
h = ctypes.c_void_p(L.ref_load(sys.argv[2].encode()))
info = np.zeros(8); L.ref_info(h, info.ctypes.data_as(ctypes.c_void_p))
out = {"info": info}
cap = 60000
def nodes(t, sol):
    buf = np.zeros(8 * cap)
    n = L.ref_nodes(h, ctypes.c_double(t), sol, buf.ctypes.data_as(ctypes.c_void_p), cap)
    return buf.reshape(8, cap)[:, :n].copy()
if "times" in job:
    for i, t in enumerate(job["times"]):
        out[f"t{i}"] = np.float64(t)
        out[f"nodes{i}"] = nodes(float(t), 0)
        out[f"sol_nodes{i}"] = nodes(float(t), 1)
if "pts" in job:
    pts = job["pts"].astype(np.int64)
    for i in range(int(info[5])):
        t = L.ref_snapshot_time(h, i); T = np.zeros(len(pts))
        L.ref_calc_T(h, ctypes.c_double(t), pts.ctypes.data_as(ctypes.c_void_p), ctypes.c_int64(len(pts)),
                     T.ctypes.data_as(ctypes.c_void_p))
        out[f"t{i}"] = np.float64(t); out[f"T{i}"] = T
if "csv" in job:
    import os
    L.ref_simulate(h)
    if str(job["csv"]) == "Solidification":
        L.ref_output(h, b"Solidification.Final")
    names = sorted(os.listdir("Data"))
    out["names"] = np.array(names)
    for i, nm in enumerate(names):
        with open(os.path.join("Data", nm), "rb") as f:
            out[f"file{i}"] = np.frombuffer(f.read(), dtype=np.uint8)
if "rrdf" in job:
    import os
    L.ref_rrdf.restype = ctypes.c_int64
    L.ref_simulate(h)
    n = L.ref_rrdf(h, None, None, None, ctypes.c_int64(0))
    idx = np.zeros((n, 3), dtype=np.uint32); ts = np.zeros((n, 2)); Ts = np.zeros((n, 16))
    L.ref_rrdf(h, idx.ctypes.data_as(ctypes.c_void_p), ts.ctypes.data_as(ctypes.c_void_p),
               Ts.ctypes.data_as(ctypes.c_void_p), ctypes.c_int64(n))
    out.update(idx=idx, ts=ts, Ts=Ts)
    L.ref_output_rrdf(h, b"RRDF")
    names = sorted(os.listdir("Data"))
    out["names"] = np.array(names)
    for i, nm in enumerate(names):
        with open(os.path.join("Data", nm), "rb") as f:
            out[f"file{i}"] = np.frombuffer(f.read(), dtype=np.uint8)
    L.ref_output_rrdf_bin(h, b"RRDF")                # the binary form, kept apart from the CSV
    with open(os.path.join("Data", [nm for nm in os.listdir("Data") if nm.endswith(".bin")][0]), "rb") as f:
        out["bin_file"] = np.frombuffer(f.read(), dtype=np.uint8)
if "custom" in job:
    import os
    L.ref_simulate(h)
    if str(job["custom"]) == "Solidification":
        L.ref_output(h, b"Solidification.Final")
        for f in ("T", "tSol", "G", "V", "dTdt"):
            a = np.zeros(int(info[3])); L.ref_field(h, f.encode(), a.ctypes.data_as(ctypes.c_void_p)); out[f] = a
    names = sorted(os.listdir("Data"))
    out["names"] = np.array(names)
    for i, nm in enumerate(names):
        with open(os.path.join("Data", nm), "rb") as f:
            out[f"file{i}"] = np.frombuffer(f.read(), dtype=np.uint8)
if "thist" in job:
    import os
    L.ref_simulate(h)
    L.ref_output_T_hist(h, b"T.hist")
    nm = [f for f in os.listdir("Data") if f.endswith("T.hist.csv")][0]
    out["thist_name"] = np.asarray(nm)
    with open(os.path.join("Data", nm), "rb") as f:
        out["thist_file"] = np.frombuffer(f.read(), dtype=np.uint8)
if "fields" in job:
    L.ref_simulate(h)
    if "rdf" in job:
        import os
        L.ref_rdf.restype = ctypes.c_int64
        n = L.ref_rdf(h, None, None, ctypes.c_int64(0))
        counts = np.zeros(3 * int(info[3]), dtype=np.int32); vals = np.zeros(n)
        L.ref_rdf(h, counts.ctypes.data_as(ctypes.c_void_p), vals.ctypes.data_as(ctypes.c_void_p), ctypes.c_int64(n))
        out.update(rdf_counts=counts, rdf_vals=vals)
        L.ref_output_rdf(h, b"RDF.Final")
        with open(os.path.join("Data", os.listdir("Data")[0]), "rb") as f:
            out["rdf_file"] = np.frombuffer(f.read(), dtype=np.uint8)
    for f in job["fields"]:
        a = np.zeros(int(info[3])); L.ref_field(h, str(f).encode(), a.ctypes.data_as(ctypes.c_void_p)); out[str(f)] = a
np.savez(sys.argv[4], **out)
"""


def run_ref(deck, job: dict, scratch: str) -> dict:
    d = os.path.join(scratch, deck.name)
    deck.write(d)
    jf, of = os.path.join(scratch, "job.npz"), os.path.join(scratch, "out.npz")
    np.savez(jf, **job)
    subprocess.run([sys.executable, "-c", _CHILD, REF_LIB, d, jf, of], check=True,
                   stdout=subprocess.DEVNULL)
    return dict(np.load(of))


def node_fixture(deck, times, scratch):
    r = run_ref(deck, {"times": np.asarray(times, dtype=np.float64)}, scratch)
    np.savez_compressed(os.path.join(HERE, f"nodes_{deck.name}.npz"), **r)
    return r


def run_fixture(deck, scratch, tag):
    fields = ["T", "output_flag"] + [f for f in ("tSol", "G", "V", "Gx", "Gy", "Gz", "dTdt", "eqFrac",
                                                 "numMelt", "depth") if deck.outputs.get(f)]
    job = {"fields": np.asarray(fields)}
    if deck.outputs.get("RDF"):
        job["rdf"] = np.asarray(1)
    r = run_ref(deck, job, scratch)
    flag = r["output_flag"] > 0
    idx = np.flatnonzero(flag)
    rng = np.random.default_rng(1234)
    sub = np.sort(rng.choice(idx, min(1500, idx.size), replace=False)) if idx.size else idx
    out = {"info": r["info"], "mask": np.packbits(flag), "n_points": np.int64(flag.size), "sample": sub}
    if "rdf_counts" in r:                          # the reduced data: every value, and the file
        out.update(rdf_counts=r["rdf_counts"], rdf_vals=r["rdf_vals"], rdf_file=r["rdf_file"])
    for f in fields:
        if f == "output_flag":
            continue
        v = r[f][flag]
        out[f"{f}_sum"] = np.float64(np.sum(v))
        out[f"{f}_abssum"] = np.float64(np.sum(np.abs(v)))
        out[f"{f}_max"] = np.float64(np.max(v)) if v.size else np.float64(0)
        out[f"{f}_sample"] = r[f][sub]
    np.savez_compressed(os.path.join(HERE, f"run_{tag}.npz"), **out)
    return out


RASTER_END = 0.0380224859550507   # end of the 10 x 2 mm raster (s)
NODE_TIMES = {
    "snapshot_raster": [0.25 * RASTER_END, 0.5 * RASTER_END, RASTER_END, 0.012345678, 0.03, RASTER_END + 2e-3],
    "small_spots": [0.3e-3, 0.9e-3, 1.7e-3, 2.52e-3, 3.1e-3],
    "small_multibeam": [1e-4, 5e-4, 1.5e-3, 2.5e-3],
    "small_bcs": [0.4e-3, 1.2e-3, 3.0e-3],
    # path compression (Settings: Path Compression 1, src/Calc.cpp:48-58,213-501)
    "comp_spots": [0.3e-3, 0.9e-3, 1.7e-3, 2.52e-3, 3.1e-3, 4.0e-3],
    "comp_lines": [0.4e-3, 1.1e-3, 1.9e-3, 2.6e-3],
    "comp_zigzag": [0.2e-3, 0.7e-3, 1.3e-3, 2.2e-3, 3.0e-3],
}
RUNS = {"small_surface": ("small_surface", "Surface"), "small_volume": ("small_surface", "Volume"),
        "small_none": ("small_surface", "None"), "small_multibeam": ("small_multibeam",),
        "small_surface_comp": ("small_surface", "Surface"), "small_surface_rdf": ("small_surface", "Surface"),
        "small_volume_rdf": ("small_surface", "Volume")}


CSV_DECKS = ("csv_snapshot", "small_multibeam")
# Stork runs (Tracking Stork, src/Run.cpp:711-1079): the doubly reduced data; the first deck's
# fixture also holds the reference's RRDF file
RRDF_DECKS = ("small_stork", "surface_stork", "stork_bigpool")


def rrdf_deck(name):
    """The deck each rrdf_<name>.npz fixture was made from."""
    if name == "surface_stork":
        d = decks.small_surface("Stork")
        d.name = "surface_stork"
        return d
    if name == "stork_bigpool":                # a 150 um beam on a 5 um grid: ~2,400 cell columns a step
        d = decks.small_surface("Stork")
        d.name = "stork_bigpool"
        d.beams = [decks.BeamSpec(width_x=150e-6, width_y=150e-6, power=400.0)]
        d.paths = [decks.serpentine_path(1, 0.2, 0.08, 0.8)]
        d.axes = (decks.AxisSpec(-0.1e-3, -0.1e-3 + 89 * 5e-6, num=90),
                  decks.AxisSpec(-34.5 * 5e-6, 34.5 * 5e-6, num=70), decks.AxisSpec(-11 * 5e-6, 0.0, num=12))
        return d
    return decks.small_stork()


def rrdf_digest(idx, ts, Ts):
    """SHA-256 of the rows: the index, time and temperature arrays' little-endian bytes."""
    import hashlib
    h = hashlib.sha256()
    for a, dt in ((idx, "<u4"), (ts, "<f8"), (Ts, "<f8")):
        h.update(np.ascontiguousarray(a, dtype=dt).tobytes())
    return h.hexdigest()


def rrdf_fixture(deck, scratch, with_file):
    r = run_ref(deck, {"rrdf": np.asarray(1)}, scratch)
    out = {"rows": np.int64(r["idx"].shape[0]), "digest": np.asarray(rrdf_digest(r["idx"], r["ts"], r["Ts"])),
           "steps": np.int64(np.unique(r["ts"][:, 1]).size)}
    if with_file:
        out["names"] = r["names"]
        out.update({k: v for k, v in r.items() if k.startswith("file") or k == "bin_file"})
    np.savez_compressed(os.path.join(HERE, f"rrdf_{deck.name}.npz"), **out)
    return out


def csv_deck(name):
    """The deck each csv_<name>.npz fixture was made from."""
    if name == "csv_snapshot":
        d = decks.small_snapshot()
        d.name = "csv_snapshot"
        d.axes = (decks.AxisSpec(0.0, 0.58e-3, num=30), decks.AxisSpec(-0.05e-3, 0.33e-3, num=20),
                  decks.AxisSpec(-0.08e-3, 0.0, num=5))
        return d
    return getattr(decks, name)()


CUSTOM_DECKS = ("custom_snapshot", "custom_notrack")


def custom_deck(name):
    """The deck each custom_<name>.npz fixture (Domain: Custom File) was made from: seeded
    points over the scanned area instead of a grid (the Domain's grid stays in the file and
    only bounds the domain)."""
    rng = np.random.default_rng(11)
    if name == "custom_snapshot":
        d = decks.small_snapshot()
        lo, hi = (0.0, -0.05, -0.09), (0.59, 0.34, 0.0)
        n = 300
    else:                                          # Surface tracking in the file: the run goes without
        d = decks.small_surface("Surface")
        lo, hi = (-0.05, -0.1, -0.11), (0.44, 0.29, 0.0)
        n = 200
        d.outputs = {"T": 1, "tSol": 1, "G": 1, "V": 1, "dTdt": 1}
    pts = rng.uniform(lo, hi, size=(n, 3))
    pts[: n // 4, 2] = 0.0                         # a quarter on the top surface
    d.points = [tuple(float(v) for v in p) for p in pts]
    d.name = name
    return d


def custom_fixture(deck, scratch):
    job = {"custom": np.asarray(deck.mode), "pts": np.arange(len(deck.points), dtype=np.int64)}
    if deck.mode != "Snapshots":
        del job["pts"]
    r = run_ref(deck, job, scratch)
    np.savez_compressed(os.path.join(HERE, f"{deck.name}.npz"), **r)
    return r


THIST_DECKS = ("thist_snapshot", "thist_notrack")


def thist_deck(name):
    """The deck each thist_<name>.npz fixture (Output T_hist 1) was made from."""
    if name == "thist_snapshot":                   # three snapshots of a 30x20x5 grid
        d = csv_deck("csv_snapshot")
        d.outputs = {"T": 1, "T_hist": 1}
    else:                                          # every step of a 16x14x5 grid without tracking
        d = decks.small_stork()
        d.tracking = "None"
        d.axes = (decks.AxisSpec(-0.05e-3, 0.1e-3, num=16), decks.AxisSpec(-0.1e-3, 0.03e-3, num=14),
                  decks.AxisSpec(-0.04e-3, 0.0, num=5))
        d.outputs = {"T": 1, "tSol": 1, "T_hist": 1}
    d.name = name
    return d


def thist_fixture(deck, scratch):
    r = run_ref(deck, {"thist": np.asarray(1)}, scratch)
    out = {"file_name": r["thist_name"], "file_bytes": r["thist_file"]}
    np.savez_compressed(os.path.join(HERE, f"{deck.name}.npz"), **out)
    return out


def csv_fixture(deck, scratch):
    r = run_ref(deck, {"csv": np.asarray(deck.mode)}, scratch)
    out = {k: v for k, v in r.items() if k == "names" or k.startswith("file")}
    np.savez_compressed(os.path.join(HERE, f"csv_{deck.name}.npz"), **out)
    return out


def node_deck(name):
    """The deck each nodes_<name>.npz fixture was made from."""
    if name.startswith("comp_"):
        d = {"comp_spots": decks.small_spots, "comp_lines": decks.small_snapshot,
             "comp_zigzag": decks.small_zigzag}[name]()
        d.name = name
        d.settings_extra = {"Path": {"Compression": "1"}}
        return d
    if name == "small_bcs":
        d = decks.small_snapshot()
        d.name = "small_bcs"
        d.bcs = {"X_min": -0.02e-3, "X_max": 0.6e-3, "Y_min": -0.05e-3, "Z_min": -0.2e-3, "Reflections": 2}
        return d
    return getattr(decks, name)()


def run_deck(tag):
    """The deck each run_<tag>.npz fixture was made from."""
    fn, *args = RUNS[tag]
    d = getattr(decks, fn)(*args)
    if tag.endswith("_comp"):                  # path compression on
        d.name = tag
        d.settings_extra = {"Path": {"Compression": "1"}}
    if tag.endswith("_rdf"):                   # the reduced data format (Output RDF 1)
        d.name = tag
        d.outputs = dict(d.outputs, RDF=1, numMelt=1)
    return d


def main():
    if not os.path.exists(REF_LIB):
        sys.exit(f"missing {REF_LIB}: build it with `make -C oracle ref`")
    if sys.argv[1:] == ["comp"]:               # only the path-compression fixtures
        with tempfile.TemporaryDirectory() as scratch:
            for name in [n for n in NODE_TIMES if n.startswith("comp_")]:
                node_fixture(node_deck(name), NODE_TIMES[name], scratch)
            for tag in [t for t in RUNS if t.endswith("_comp")]:
                run_fixture(run_deck(tag), scratch, tag)
        print("compression fixtures written to", HERE)
        return
    if sys.argv[1:] == ["rdf"]:
        with tempfile.TemporaryDirectory() as scratch:
            for tag in [t for t in RUNS if t.endswith("_rdf")]:
                run_fixture(run_deck(tag), scratch, tag)
        print("rdf fixtures written to", HERE)
        return
    if sys.argv[1:] == ["rrdf"]:
        with tempfile.TemporaryDirectory() as scratch:
            for i, name in enumerate(RRDF_DECKS):
                rrdf_fixture(rrdf_deck(name), scratch, i == 0)
        print("rrdf fixtures written to", HERE)
        return
    if sys.argv[1:] == ["custom"]:
        with tempfile.TemporaryDirectory() as scratch:
            for name in CUSTOM_DECKS:
                custom_fixture(custom_deck(name), scratch)
        print("custom fixtures written to", HERE)
        return
    if sys.argv[1:] == ["thist"]:
        with tempfile.TemporaryDirectory() as scratch:
            for name in THIST_DECKS:
                thist_fixture(thist_deck(name), scratch)
        print("thist fixtures written to", HERE)
        return
    if sys.argv[1:] == ["csv"]:
        with tempfile.TemporaryDirectory() as scratch:
            for name in CSV_DECKS:
                csv_fixture(csv_deck(name), scratch)
        print("csv fixtures written to", HERE)
        return
    with tempfile.TemporaryDirectory() as scratch:
        for name, times in NODE_TIMES.items():
            node_fixture(node_deck(name), times, scratch)
        rng = np.random.default_rng(7)
        pts = np.sort(rng.choice(800000, 4096, replace=False)).astype(np.int64)
        r = run_ref(decks.snapshot_raster(), {"pts": pts}, scratch)
        np.savez_compressed(os.path.join(HERE, "temp_snapshot_raster.npz"), pts=pts, **r)
        for tag in RUNS:
            run_fixture(run_deck(tag), scratch, tag)
        for name in CSV_DECKS:
            csv_fixture(csv_deck(name), scratch)
        for i, name in enumerate(RRDF_DECKS):
            rrdf_fixture(rrdf_deck(name), scratch, i == 0)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
