"""Input decks in 3DThesis's own keyword-file format.

A deck is a directory holding ``ParamInput.txt`` plus the Mode / Material /
Beam / Path / Domain / Output / Settings files it names, laid out exactly as the
reference CLI reads them (``src/Init.cpp:233-303``).  Path files are in mm with a
header line and an implicit spot segment at the origin (``src/Init.cpp:560-625``).

The named workloads are the synthetic benchmark cases:

* ``snapshot_raster``   - 10 x 2 mm raster, 200x100x40 grid, snapshots at 25/50/100 %.
* ``surface_serpentine`` - 50 x 5 mm serpentine, 500x500x100 grid, Surface tracking.
* ``volume_multibeam``  - 4 seeded, rotated serpentines, 400x400x80 grid, Volume tracking.
* ``snapshot_sweep``    - 256 seeded single-beam snapshot instances (uneven sizes).

Small variants (``small_*``) keep the same structure at sizes the CPU oracle
finishes in seconds; the tests use them.
"""
from __future__ import annotations

import math
import os
import random
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Tuple

# segment = (mode, x_mm, y_mm, z_mm, pmod, param)  mode 0 = line (param = speed m/s),
# mode 1 = spot (param = dwell time s)
Seg = Tuple[int, float, float, float, float, float]


@dataclass
class BeamSpec:
    width_x: float = 50e-6
    width_y: float = 50e-6
    depth_z: float = 1e-6
    power: float = 200.0
    efficiency: float = 0.35


@dataclass
class MaterialSpec:
    T0: float = 300.0
    TL: float = 1600.0
    k: float = 26.6
    c: float = 600.0
    rho: float = 7900.0
    cet: Optional[Tuple[float, float, float]] = None  # (N0, n, a)


@dataclass
class AxisSpec:
    vmin: float
    vmax: float
    num: Optional[int] = None
    res: Optional[float] = None


@dataclass
class Deck:
    name: str
    mode: str                       # "Snapshots" | "Solidification"
    beams: List[BeamSpec]
    paths: List[List[Seg]]
    material: MaterialSpec = field(default_factory=MaterialSpec)
    axes: Optional[Tuple[AxisSpec, AxisSpec, AxisSpec]] = None
    scan_fracs: Optional[Sequence[float]] = None
    times: Optional[Sequence[float]] = None
    tracking: str = "None"
    timestep: Optional[float] = None
    output_frequency: Optional[int] = None
    check_radius: Optional[float] = None
    outputs: Dict[str, int] = field(default_factory=dict)
    max_threads: int = 1
    bcs: Optional[Dict[str, float]] = None
    settings_extra: Dict[str, Dict[str, str]] = field(default_factory=dict)
    # custom points in place of a grid (Domain: Custom File), mm, written to Points.txt under
    # a header line (the reference skips the file's first line)
    points: Optional[Sequence[Tuple[float, float, float]]] = None

    # ------------------------------------------------------------------ write
    def write(self, directory: str) -> str:
        """Write every file of the deck into ``directory``; returns the path of
        ``ParamInput.txt``."""
        os.makedirs(directory, exist_ok=True)
        multi = len(self.beams) > 1
        beam_name = "Beam.*.txt" if multi else "Beam.txt"
        path_name = "Path.*.txt" if multi else "Path.txt"
        files = {
            "ParamInput.txt": _block("Simulation", [("Name", self.name), ("Mode", "Mode.txt"),
                                                    ("Material", "Material.txt"),
                                                    ("Beam", beam_name), ("Path", path_name)])
            + _block("Options", [("Domain", "Domain.txt"), ("Output", "Output.txt"),
                                 ("Settings", "Settings.txt")]),
            "Mode.txt": self._mode_text(),
            "Material.txt": self._material_text(),
            "Domain.txt": self._domain_text(),
            "Output.txt": self._output_text(),
            "Settings.txt": self._settings_text(),
        }
        if self.points is not None:
            files["Points.txt"] = "x y z\n" + "".join(f"{_f(x)} {_f(y)} {_f(z)}\n" for x, y, z in self.points)
        for i, (b, p) in enumerate(zip(self.beams, self.paths)):
            bname = f"Beam.{i + 1}.txt" if multi else "Beam.txt"
            pname = f"Path.{i + 1}.txt" if multi else "Path.txt"
            files[bname] = _block("Shape", [("Width_X", _f(b.width_x)), ("Width_Y", _f(b.width_y)),
                                            ("Depth_Z", _f(b.depth_z))]) \
                + _block("Intensity", [("Power", _f(b.power)), ("Efficiency", _f(b.efficiency))])
            files[pname] = _path_text(p)
        for fname, text in files.items():
            with open(os.path.join(directory, fname), "w") as fh:
                fh.write(text)
        return os.path.join(directory, "ParamInput.txt")

    def _mode_text(self) -> str:
        if self.mode == "Snapshots":
            items = []
            if self.times is not None:
                items.append(("Times", ",".join(_f(t) for t in self.times)))
            if self.scan_fracs is not None:
                items.append(("ScanFracs", ",".join(_f(s) for s in self.scan_fracs)))
            items.append(("Tracking", self.tracking))
            return _block("Snapshots", items)
        items = [("Tracking", self.tracking)]
        if self.timestep is not None:
            items.append(("Timestep", _f(self.timestep)))
        if self.output_frequency is not None:
            items.append(("OutputFrequency", str(int(self.output_frequency))))
        if self.check_radius is not None:
            items.append(("CheckRadius", _f(self.check_radius)))
        return _block("Solidification", items)

    def _material_text(self) -> str:
        m = self.material
        text = _block("Constants", [("T_0", _f(m.T0)), ("T_L", _f(m.TL)), ("k", _f(m.k)),
                                    ("c", _f(m.c)), ("p", _f(m.rho))])
        if m.cet is not None:
            text += _block("CET", [("N0", _f(m.cet[0])), ("n", _f(m.cet[1])), ("a", _f(m.cet[2]))])
        return text

    def _domain_text(self) -> str:
        text = ""
        if self.axes is not None:
            for name, ax in zip("XYZ", self.axes):
                items = [("Min", _f(ax.vmin)), ("Max", _f(ax.vmax))]
                if ax.num is not None:
                    items.append(("Num", str(int(ax.num))))
                if ax.res is not None:
                    items.append(("Res", _f(ax.res)))
                text += _block(name, items)
        if self.bcs:
            text += _block("BoundaryConditions", [(k, _f(v)) for k, v in self.bcs.items()])
        if self.points is not None:
            text += _block("Custom", [("File", "Points.txt")])
        return text

    def _output_text(self) -> str:
        grid = [("x", 1), ("y", 1), ("z", 1)]
        temp = [("T", self.outputs.get("T", 1)), ("T_hist", self.outputs.get("T_hist", 0))]
        sol_keys = ["tSol", "G", "Gx", "Gy", "Gz", "V", "dTdt", "eqFrac", "depth", "numMelt"]
        sol = [(k, self.outputs.get(k, 0)) for k in sol_keys] + [("RDF", self.outputs.get("RDF", 0)),
                                                                  ("MP_Stats", 0)]
        return (_block("Grid", [(k, str(v)) for k, v in grid])
                + _block("Temperature", [(k, str(v)) for k, v in temp])
                + _block("Solidification", [(k, str(v)) for k, v in sol]))

    def _settings_text(self) -> str:
        text = _block("Compute", [("MaxThreads", str(int(self.max_threads)))])
        for blk, items in self.settings_extra.items():
            text += _block(blk, list(items.items()))
        return text


def _f(v: float) -> str:
    return repr(float(v))


def _block(name: str, items: Sequence[Tuple[str, str]]) -> str:
    body = "".join(f"\t{k}\t{v}\n" for k, v in items)
    return f"{name}\n{{\n{body}}}\n"


def _path_text(segs: Sequence[Seg]) -> str:
    lines = ["Mode\tX(mm)\tY(mm)\tZ(mm)\tPmod\tTime(s)"]
    for m, x, y, z, q, prm in segs:
        lines.append(f"{int(m)}\t{_f(x)}\t{_f(y)}\t{_f(z)}\t{_f(q)}\t{_f(prm)}")
    return "\n".join(lines) + "\n"


# ---------------------------------------------------------------------- paths
def raster_path(tracks: int, length_mm: float, hatch_mm: float, speed: float,
                lead_in: bool = True) -> List[Seg]:
    """Unidirectional raster along +x: a power-off move to the start of each track
    (the first one from the implicit origin, zero length) then the lit track."""
    segs: List[Seg] = []
    for n in range(tracks):
        y = round(n * hatch_mm, 12)
        if lead_in or n > 0:
            segs.append((0, 0.0, y, 0.0, 0.0, speed))
        segs.append((0, length_mm, y, 0.0, 1.0, speed))
    return segs


def serpentine_path(tracks: int, length_mm: float, hatch_mm: float, speed: float,
                    x0: float = 0.0, y0: float = 0.0, angle: float = 0.0,
                    cx: float = 0.0, cy: float = 0.0) -> List[Seg]:
    """Boustrophedon raster with power-off hatch moves, optionally rotated by
    ``angle`` about (cx, cy) (all mm)."""
    pts: List[Tuple[float, float, float]] = []   # (x, y, pmod)
    pts.append((x0, y0, 0.0))                    # power-off move from the origin
    for n in range(tracks):
        y = y0 + n * hatch_mm
        xa, xb = (x0, x0 + length_mm) if n % 2 == 0 else (x0 + length_mm, x0)
        if n > 0:
            pts.append((xa, y, 0.0))
        pts.append((xb, y, 1.0))
    ca, sa = math.cos(angle), math.sin(angle)
    segs: List[Seg] = []
    for x, y, q in pts:
        if angle != 0.0:
            dx, dy = x - cx, y - cy
            x, y = cx + ca * dx - sa * dy, cy + sa * dx + ca * dy
        segs.append((0, round(x, 12), round(y, 12), 0.0, q, speed))
    return segs


def spot_raster_path(nx: int, ny: int, pitch_mm: float, dwell: float) -> List[Seg]:
    """Point raster of spot-mode segments (mode 1) with power-off jumps."""
    segs: List[Seg] = []
    for j in range(ny):
        for i in range(nx):
            x, y = i * pitch_mm, j * pitch_mm
            segs.append((1, x, y, 0.0, 0.0, 1e-5))
            segs.append((1, x, y, 0.0, 1.0, dwell))
    return segs


# ------------------------------------------------------------------ workloads
def snapshot_raster() -> Deck:
    """10 tracks x 2 mm along x, hatch 0.1 mm, 1.0 m/s; 200x100x40 grid at 10 um;
    snapshots at 25/50/100 % of the scan."""
    return Deck(
        name="snapshot_raster", mode="Snapshots", beams=[BeamSpec()],
        paths=[raster_path(10, 2.0, 0.1, 1.0)],
        axes=(AxisSpec(0.0, 1.99e-3, num=200), AxisSpec(-0.05e-3, 0.94e-3, num=100),
              AxisSpec(-0.39e-3, 0.0, num=40)),
        scan_fracs=[25, 50, 100], tracking="None")


def surface_serpentine(tracks: int = 50, length_mm: float = 5.0,
                       grid: Tuple[int, int, int] = (500, 500, 100)) -> Deck:
    """Serpentine of 50 x 5 mm tracks, hatch 80 um, 0.8 m/s; Surface tracking on a
    500x500x100 grid at 10 um, dt = 1e-5 s; outputs tSol, G, V, dTdt."""
    nx, ny, nz = grid
    return Deck(
        name="surface_serpentine", mode="Solidification", beams=[BeamSpec()],
        paths=[serpentine_path(tracks, length_mm, 0.08, 0.8)],
        axes=(AxisSpec(0.0, (nx - 1) * 1e-5, num=nx), AxisSpec(-0.5e-3, -0.5e-3 + (ny - 1) * 1e-5, num=ny),
              AxisSpec(-(nz - 1) * 1e-5, 0.0, num=nz)),
        tracking="Surface", timestep=1e-5,
        outputs={"T": 0, "tSol": 1, "G": 1, "V": 1, "dTdt": 1})


def volume_multibeam(seed: int = 0, grid: Tuple[int, int, int] = (400, 400, 80),
                     tracks: int = 20, length_mm: float = 3.0) -> Deck:
    """Four beams, each a seeded serpentine of 20 x 3 mm tracks rotated by U[0, pi)
    about the grid centre, v ~ U(0.5, 1.5) m/s, P ~ U(150, 400) W, widths
    ~ U(40, 100) um; Volume tracking on 400x400x80 at 10 um, dt = 5e-6 s."""
    rng = random.Random(seed)
    nx, ny, nz = grid
    cx, cy = (nx - 1) * 1e-2 / 2, (ny - 1) * 1e-2 / 2
    beams, paths = [], []
    hatch = 0.1
    for _ in range(4):
        v = rng.uniform(0.5, 1.5)
        beams.append(BeamSpec(width_x=rng.uniform(40e-6, 100e-6), width_y=rng.uniform(40e-6, 100e-6),
                              depth_z=1e-6, power=rng.uniform(150, 400), efficiency=0.35))
        ang = rng.uniform(0.0, math.pi)
        x0 = cx - length_mm / 2
        y0 = cy - (tracks - 1) * hatch / 2
        paths.append(serpentine_path(tracks, length_mm, hatch, v, x0=x0, y0=y0, angle=ang, cx=cx, cy=cy))
    return Deck(
        name="volume_multibeam", mode="Solidification", beams=beams, paths=paths,
        axes=(AxisSpec(0.0, (nx - 1) * 1e-5, num=nx), AxisSpec(0.0, (ny - 1) * 1e-5, num=ny),
              AxisSpec(-(nz - 1) * 1e-5, 0.0, num=nz)),
        tracking="Volume", timestep=5e-6,
        outputs={"T": 0, "tSol": 1, "G": 1, "V": 1, "dTdt": 1})


def snapshot_sweep(n: int = 256, seed: int = 0) -> List[Deck]:
    """256 independent single-beam snapshot instances: P ~ U(100, 400) W,
    v ~ U(0.5, 2) m/s, width ~ U(40, 120) um, U{1..30} tracks of 2 mm (hatch
    0.1 mm), grids nx, ny ~ U{50..400}, nz ~ U{10..60} at 10 um, snapshot at 100 %."""
    rng = random.Random(seed)
    decks = []
    for k in range(n):
        p = rng.uniform(100, 400)
        v = rng.uniform(0.5, 2.0)
        w = rng.uniform(40e-6, 120e-6)
        tr = rng.randint(1, 30)
        nx, ny, nz = rng.randint(50, 400), rng.randint(50, 400), rng.randint(10, 60)
        decks.append(Deck(
            name=f"sweep{k:03d}", mode="Snapshots",
            beams=[BeamSpec(width_x=w, width_y=w, depth_z=1e-6, power=p, efficiency=0.35)],
            paths=[raster_path(tr, 2.0, 0.1, v)],
            axes=(AxisSpec(0.0, (nx - 1) * 1e-5, num=nx), AxisSpec(-0.2e-3, -0.2e-3 + (ny - 1) * 1e-5, num=ny),
                  AxisSpec(-(nz - 1) * 1e-5, 0.0, num=nz)),
            scan_fracs=[100], tracking="None"))
    return decks


# ------------------------------------------------------- small (test) decks
def small_snapshot() -> Deck:
    d = snapshot_raster()
    d.name = "small_snapshot"
    d.paths = [raster_path(3, 0.6, 0.1, 1.0)]
    d.axes = (AxisSpec(0.0, 0.59e-3, num=60), AxisSpec(-0.05e-3, 0.34e-3, num=40), AxisSpec(-0.09e-3, 0.0, num=10))
    d.scan_fracs = [25, 50, 100]
    return d


def small_surface(tracking: str = "Surface", dt: float = 1e-5) -> Deck:
    d = surface_serpentine(tracks=3, length_mm=0.4, grid=(50, 40, 12))
    d.name = f"small_{tracking.lower()}"
    d.axes = (AxisSpec(-0.05e-3, 0.44e-3, num=50), AxisSpec(-0.1e-3, 0.29e-3, num=40), AxisSpec(-0.11e-3, 0.0, num=12))
    d.tracking = tracking
    d.timestep = dt
    d.outputs = {"T": 1, "tSol": 1, "G": 1, "V": 1, "dTdt": 1, "Gx": 1, "Gy": 1, "Gz": 1,
                 "eqFrac": 1, "numMelt": 1, "depth": 1 if tracking == "Surface" else 0}
    d.material = MaterialSpec(cet=(3e13, 3.0, 1.25e6))
    return d


def small_stork() -> Deck:
    """Two 0.1 mm tracks on a 20x22x7 grid at 10 um, Stork tracking, dt = 2e-5 s: the pool
    reaches the bottom layer, so the walk's bottom rule is exercised."""
    d = small_surface("Stork", dt=2e-5)
    d.paths = [serpentine_path(2, 0.1, 0.08, 0.8)]
    d.axes = (AxisSpec(-0.05e-3, 0.14e-3, num=20), AxisSpec(-0.1e-3, 0.11e-3, num=22), AxisSpec(-0.06e-3, 0.0, num=7))
    return d


def small_multibeam(seed: int = 1) -> Deck:
    d = volume_multibeam(seed=seed, grid=(40, 40, 10), tracks=3, length_mm=0.25)
    d.name = "small_multibeam"
    d.timestep = 1e-5
    d.outputs = {"T": 1, "tSol": 1, "G": 1, "V": 1, "dTdt": 1, "numMelt": 1}
    return d


def small_spots() -> Deck:
    """Spot-mode raster (mode-1 segments) on the snapshot path: exercises the
    spot branch of the beam position and step-size rules."""
    return Deck(
        name="small_spots", mode="Snapshots", beams=[BeamSpec(width_x=40e-6, width_y=60e-6, power=300)],
        paths=[spot_raster_path(4, 3, 0.1, 2e-4)],
        axes=(AxisSpec(-0.1e-3, 0.4e-3, num=26), AxisSpec(-0.1e-3, 0.3e-3, num=21), AxisSpec(-0.05e-3, 0.0, num=6)),
        scan_fracs=[30, 70, 100], tracking="None")


def small_zigzag() -> Deck:
    """A fine serpentine of 20 short 60 um tracks with 30 um hatch moves (a thin-wall-like
    path): successive segments lie within the heat's diffusion distance of each other."""
    return Deck(
        name="small_zigzag", mode="Snapshots", beams=[BeamSpec()],
        paths=[serpentine_path(20, 0.06, 0.03, 0.5)],
        axes=(AxisSpec(-0.1e-3, 0.19e-3, num=30), AxisSpec(-0.1e-3, 0.69e-3, num=40), AxisSpec(-0.05e-3, 0.0, num=6)),
        scan_fracs=[30, 70, 100], tracking="None")


def small_sweep(n: int = 10, seed: int = 3) -> List[Deck]:
    """Small uneven snapshot sweep: seeded power, speed, widths and track counts, grids
    from 8x8x3 to 40x30x10 points, snapshots at 50 % and 100 %; deck 1 scans spots and
    deck 2 carries two beams and deck 3 has reflecting boundaries, so node counts differ
    by deck."""
    rng = random.Random(seed)
    decks = []
    for k in range(n):
        nx, ny, nz = rng.randint(8, 40), rng.randint(8, 30), rng.randint(3, 10)
        w = rng.uniform(40e-6, 100e-6)
        beams = [BeamSpec(width_x=w, width_y=rng.uniform(40e-6, 100e-6), power=rng.uniform(100, 400))]
        paths = [raster_path(rng.randint(1, 4), 0.3, 0.05, rng.uniform(0.5, 2.0))]
        if k == 1:
            paths = [spot_raster_path(3, 2, 0.08, 1e-4)]
        if k == 2:
            beams.append(BeamSpec(width_x=60e-6, width_y=50e-6, power=200))
            paths.append(raster_path(2, 0.25, 0.06, 1.2))
        bcs = None
        if k == 3:
            bcs = {"X_min": -0.1e-3, "X_max": 0.45e-3, "Y_min": -0.08e-3, "Z_min": -0.2e-3, "Reflections": 2}
        decks.append(Deck(
            name=f"small_sweep{k:02d}", mode="Snapshots", beams=beams, paths=paths,
            axes=(AxisSpec(-0.05e-3, -0.05e-3 + (nx - 1) * 1e-5, num=nx),
                  AxisSpec(-0.05e-3, -0.05e-3 + (ny - 1) * 1e-5, num=ny),
                  AxisSpec(-(nz - 1) * 1e-5, 0.0, num=nz)),
            scan_fracs=[50, 100], tracking="None", bcs=bcs))
    return decks


def adjoint_calibration(grid: Tuple[int, int, int] = (300, 300, 60), tracks: int = 50,
                        length_mm: float = 5.0) -> Deck:
    """The Surface-serpentine path and material (50 x 5 mm tracks, hatch 80 um, 0.8 m/s,
    200 W) as a Snapshots deck on a 300x300x60 grid at 10 um; the calibration's probe points
    and times are chosen by the caller (``adjoint_probes``)."""
    nx, ny, nz = grid
    d = surface_serpentine(tracks=tracks, length_mm=length_mm)
    d.name = "adjoint_calibration"
    d.mode = "Snapshots"
    d.tracking = "None"
    d.timestep = None
    d.outputs = {"T": 1}
    d.axes = (AxisSpec(0.0, (nx - 1) * 1e-5, num=nx), AxisSpec(-0.5e-3, -0.5e-3 + (ny - 1) * 1e-5, num=ny),
              AxisSpec(-(nz - 1) * 1e-5, 0.0, num=nz))
    d.scan_fracs = [100]
    return d


def adjoint_probes(deck: Deck, n: int = 4096, seed: int = 0, times: Sequence[float] = (0.05, 0.15, 0.30)):
    """Seeded probe points (flat ids) in the top quarter of the grid, and the snapshot
    times (s) of the calibration loss."""
    rng = random.Random(seed)
    nx, ny, nz = (ax.num for ax in deck.axes)
    pts = []
    for _ in range(n):
        i, j, k = rng.randrange(nx), rng.randrange(ny), rng.randrange(max(0, nz - nz // 4), nz)
        pts.append((i * ny + j) * nz + k)
    return pts, list(times)


def small_adjoint() -> Deck:
    d = adjoint_calibration(grid=(40, 30, 10), tracks=3, length_mm=0.4)
    d.name = "small_adjoint"
    d.axes = (AxisSpec(-0.05e-3, 0.34e-3, num=40), AxisSpec(-0.1e-3, 0.19e-3, num=30), AxisSpec(-0.09e-3, 0.0, num=10))
    return d
