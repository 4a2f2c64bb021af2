"""Test infrastructure: times the CPU oracle (the C++ restatement that the bench's CPU legs
run) against the unmodified reference compiled from its own sources (oracle/_ref, built by
`make -C oracle ref REF=<3DThesis tree>`), on the same whole solidification run with the
same number of OpenMP threads.  Run where the reference sources are present:

    python oracle/compare_speed.py [threads]

Prints one JSON line per implementation: the wall time of Run::Simulate (the reference) or
of the oracle's run, and the steps of the run.
"""
import importlib
import json
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

_CHILD = r"""
import ctypes, sys, time
L = ctypes.CDLL(sys.argv[1]); L.ref_load.restype = ctypes.c_void_p
h = ctypes.c_void_p(L.ref_load(sys.argv[2].encode()))
t0 = time.perf_counter(); L.ref_simulate(h); print(time.perf_counter() - t0)
"""


def main():
    threads = int(sys.argv[1]) if len(sys.argv) > 1 else (os.cpu_count() or 1)
    decks = importlib.import_module("3dthesis_gb300.decks")
    import oracle_lib
    ref_lib = os.path.join(ROOT, "oracle", "_ref", "libthesis_ref.so")
    with tempfile.TemporaryDirectory() as tmp:
        deck = decks.surface_serpentine()
        deck.max_threads = threads                     # the reference's MaxThreads setting
        path = deck.write(os.path.join(tmp, "surface"))
        o = oracle_lib.Oracle(path)
        t0 = time.perf_counter()
        steps = o.solidify(threads=threads)
        port = time.perf_counter() - t0
        print(json.dumps({"impl": "oracle port", "deck": deck.name, "threads": threads, "steps": int(steps),
                          "seconds": round(port, 2), "pairs": int(o.pairs)}))
        if os.path.exists(ref_lib):
            r = subprocess.run([sys.executable, "-c", _CHILD, ref_lib, os.path.dirname(path)], check=True,
                               capture_output=True, text=True)
            ref = float(r.stdout.strip().splitlines()[-1])
            print(json.dumps({"impl": "reference (own sources, -O3)", "deck": deck.name, "threads": threads,
                              "seconds": round(ref, 2), "port_speedup": round(ref / port, 3)}))


if __name__ == "__main__":
    main()
