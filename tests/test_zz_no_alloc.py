"""th_calc_T_noalloc: the allocation-free evaluation entry point, through the C ABI.

It serves callers that cannot allocate device memory (their memory is owned by their own
pool or a budget fixed at start-up, or they call from a time loop where cudaMalloc /
cudaFree would synchronise the device).  Its node list lives in a static device array, so
it must give the same temperatures as th_calc_T_device, call after call, and refuse a node
list larger than that array.  This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL_FP32 = 0.01   # K, the FP32 + Kahan tolerance of the other GPU tests


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _reference(sim, torch, t, n, pts=None):
    out = torch.empty(n, dtype=torch.float64, device="cuda")
    s = torch.cuda.Stream()
    sim.calc_T_device(t, 0 if pts is None else pts.data_ptr(), n, out.data_ptr(), s.cuda_stream)
    sim.sync(s.cuda_stream)
    return out


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_noalloc_matches_device_entry_point_twice(built_library, thesis, deck_dir, torch_cuda, precision):
    torch = torch_cuda
    with thesis.Simulation(deck_dir("snapshot_raster"), precision) as sim:
        n = sim.pnum
        t = sim.snapshot_times[2]
        ref = _reference(sim, torch, t, n)
        rng = np.random.default_rng(3)
        pts = torch.from_numpy(np.sort(rng.choice(n, 5000, replace=False)).astype(np.int64)).cuda()
        ref_list = _reference(sim, torch, sim.snapshot_times[0], pts.numel(), pts)
        s = torch.cuda.Stream()
        for _ in range(2):                                  # two calls in a row
            out = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
            sim.calc_T_noalloc(t, 0, n, out.data_ptr(), s.cuda_stream)
            assert torch.max(torch.abs(out - ref)).item() <= TOL_FP32
            out_l = torch.full((pts.numel(),), float("nan"), dtype=torch.float64, device="cuda")
            sim.calc_T_noalloc(sim.snapshot_times[0], pts.data_ptr(), pts.numel(), out_l.data_ptr(), s.cuda_stream)
            assert torch.max(torch.abs(out_l - ref_list)).item() <= TOL_FP32


def test_noalloc_other_context_between_calls(built_library, thesis, deck_dir, torch_cuda):
    """The shared array holds the last call's list; a call for another deck in between
    must not leak into the next result."""
    torch = torch_cuda
    with thesis.Simulation(deck_dir("snapshot_raster"), "fp32") as a, \
            thesis.Simulation(deck_dir("small_spots"), "fp32") as b:
        ta, tb = a.snapshot_times[1], b.snapshot_times[2]
        ref_a, ref_b = _reference(a, torch, ta, a.pnum), _reference(b, torch, tb, b.pnum)
        out_a = torch.empty(a.pnum, dtype=torch.float64, device="cuda")
        out_b = torch.empty(b.pnum, dtype=torch.float64, device="cuda")
        a.calc_T_noalloc(ta, 0, a.pnum, out_a.data_ptr())
        b.calc_T_noalloc(tb, 0, b.pnum, out_b.data_ptr())
        a.calc_T_noalloc(ta, 0, a.pnum, out_a.data_ptr())
        assert torch.max(torch.abs(out_a - ref_a)).item() <= TOL_FP32
        assert torch.max(torch.abs(out_b - ref_b)).item() <= TOL_FP32


def test_noalloc_rejects_node_list_above_static_maximum(built_library, thesis, decks, tmp_path, torch_cuda):
    torch = torch_cuda
    d = decks.small_spots()
    d.paths = [decks.spot_raster_path(90, 100, 0.005, 2e-6)]     # 9000 lit spots: > 16384 nodes
    d.scan_fracs = [100]
    with thesis.Simulation(d.write(str(tmp_path / "many_spots")), "fp32") as sim:
        out = torch.empty(sim.pnum, dtype=torch.float64, device="cuda")
        with pytest.raises(thesis.ThesisError) as ei:
            sim.calc_T_noalloc(sim.snapshot_times[0], 0, sim.pnum, out.data_ptr())
        assert ei.value.status == 4 and "static maximum" in str(ei.value)
