"""C-ABI library: loads, exports every declared symbol, and rejects bad decks on the host."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = []
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            text = open(os.path.join(ROOT, "include", h)).read()
            names += re.findall(r"^\w[\w\s\*]*?\b(th_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(built_library):
    lib = ctypes.CDLL(built_library)
    names = declared_symbols()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_layer_binds_every_symbol(thesis, built_library):
    assert set(declared_symbols()) <= set(thesis.EXPORTED)


def _create(thesis, path):
    L = thesis.load_library()
    ctx = ctypes.c_void_p()
    st = L.th_ctx_create_from_deck(path.encode(), 1, ctypes.byref(ctx))
    return st, L.th_last_error(None).decode(), ctx


def test_missing_deck_is_an_error(thesis, built_library, tmp_path):
    st, msg, ctx = _create(thesis, str(tmp_path / "nope" / "ParamInput.txt"))
    assert st == 1 and "cannot open" in msg and not ctx.value


@pytest.mark.parametrize("edit,needle", [
    (lambda d: setattr(d, "mode", "Bogus"), "exactly one"),
    (lambda d: setattr(d, "tracking", "Geometry"), "tracking"),
    (lambda d: setattr(d.beams[0], "width_x", 0.0), "widths"),
    (lambda d: d.outputs.update(T_hist=1), "T_hist output needs Tracking None"),
])
def test_bad_decks_are_rejected_before_any_launch(thesis, built_library, decks, tmp_path, edit, needle):
    d = decks.small_surface("Surface")
    edit(d)
    path = d.write(str(tmp_path / "deck"))
    if d.mode == "Bogus":
        with open(os.path.join(os.path.dirname(path), "Mode.txt"), "w") as f:
            f.write("Bogus\n{\n}\n")
    st, msg, ctx = _create(thesis, path)
    assert st != 0 and needle.lower() in msg.lower() and not ctx.value


def test_custom_point_files_are_read_as_the_reference_reads_them(thesis, built_library, tmp_path):
    """Domain: Custom File (Init::FileRead_Points, src/Init.cpp:816-857): the first line is
    skipped, each point is three numbers in mm, and a custom deck goes without tracking.  The
    point counts are the reference's (tests/golden/custom_*.npz); a file whose first line
    already holds a point loses that point, as the reference's does."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import make_golden
    import numpy as np
    for name in make_golden.CUSTOM_DECKS:
        d = make_golden.custom_deck(name)
        g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", f"{name}.npz"))
        info = thesis.deck_info(d.write(str(tmp_path / name)))
        assert info["pnum"] == int(g["info"][3]) == len(d.points)
        assert info["tracking"] == 0
    snap = make_golden.custom_deck("custom_snapshot")          # Snapshots with a tracking mode:
    snap.tracking = "Volume"                                    # without tracking for custom points
    assert thesis.deck_info(snap.write(str(tmp_path / "snapvol")))["tracking"] == 0
    grid = make_golden.csv_deck("csv_snapshot")                 # and still refused on a grid
    grid.tracking = "Volume"
    with pytest.raises(thesis.ThesisError):
        thesis.deck_info(grid.write(str(tmp_path / "gridvol")))
    path = d.write(str(tmp_path / "noheader"))
    pts = os.path.join(os.path.dirname(path), "Points.txt")
    with open(pts) as f:
        lines = f.read().splitlines()
    with open(pts, "w") as f:
        f.write("\n".join(lines[1:]) + "\n")
    assert thesis.deck_info(path)["pnum"] == len(d.points) - 1


def test_T_hist_decks_without_tracking_parse(thesis, built_library, tmp_path):
    """Output T_hist 1 is taken without tracking (Snapshots and NoTracking solidification:
    every point shares the evaluation times); the host-only parse accepts both decks."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import make_golden
    import numpy as np
    for name in make_golden.THIST_DECKS:
        d = make_golden.thist_deck(name)
        info = thesis.deck_info(d.write(str(tmp_path / name)))
        assert info["pnum"] == np.prod([ax.num for ax in d.axes])
