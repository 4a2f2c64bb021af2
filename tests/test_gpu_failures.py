"""Failure paths of the device loop and of context creation, made to happen on purpose
without faulting the GPU: a lost work item (its step can never end, so the tracking loop's
bounded waits run out), record and work-queue overflows, and a failed device allocation in
context creation.  Each returns its status code through the C ABI, and a new context on the
same GPU then runs normally.  The knobs are environment variables read on the host
(THESIS_GB300_SPIN_LIMIT, _HOLD_ITEMS, _REC_CAP, _QUEUE_CAP, _FAIL_ALLOC; _REC_HIGH_WATER,
which ends launches early without a failure, is tested in test_gpu_fullsize)."""
import os
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402

pytestmark = pytest.mark.gpu
TIMEOUT, CAPACITY, CUDA = 6, 4, 3


@pytest.fixture(scope="module")
def surface(built_library, oracle, tmp_path_factory):
    deck = make_golden.run_deck("small_surface")
    path = deck.write(str(tmp_path_factory.mktemp("fail") / "small_surface"))
    return path, oracle(path).solidify(threads=4)


def _runs_normally(thesis, path, steps, prec):
    with thesis.Simulation(path, prec) as sim:
        assert sim.solidify() == steps


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_lost_item_times_out(surface, thesis, monkeypatch, prec):
    path, steps = surface
    monkeypatch.setenv("THESIS_GB300_SPIN_LIMIT", "4096")
    monkeypatch.setenv("THESIS_GB300_HOLD_ITEMS", "1")
    with thesis.Simulation(path, prec) as sim:
        with pytest.raises(thesis.ThesisError) as e:
            sim.solidify()
    assert e.value.status == TIMEOUT
    assert "wait exceeded its limit" in str(e.value)
    monkeypatch.delenv("THESIS_GB300_SPIN_LIMIT")
    monkeypatch.delenv("THESIS_GB300_HOLD_ITEMS")
    _runs_normally(thesis, path, steps, prec)


def test_record_overflow(surface, thesis, monkeypatch):
    path, steps = surface
    monkeypatch.setenv("THESIS_GB300_REC_CAP", "8")
    with thesis.Simulation(path, "fp32") as sim:
        with pytest.raises(thesis.ThesisError) as e:
            sim.solidify()
    assert e.value.status == CAPACITY
    assert "record" in str(e.value)
    monkeypatch.delenv("THESIS_GB300_REC_CAP")
    _runs_normally(thesis, path, steps, "fp32")


def test_work_queue_overflow(surface, thesis, monkeypatch):
    path, steps = surface
    monkeypatch.setenv("THESIS_GB300_QUEUE_CAP", "4")
    monkeypatch.setenv("THESIS_GB300_SPIN_LIMIT", "4096")     # the lost items' step then gives up soon
    with thesis.Simulation(path, "fp32") as sim:
        with pytest.raises(thesis.ThesisError) as e:
            sim.solidify()
    assert e.value.status == CAPACITY
    assert "work queue" in str(e.value)
    monkeypatch.delenv("THESIS_GB300_QUEUE_CAP")
    monkeypatch.delenv("THESIS_GB300_SPIN_LIMIT")
    _runs_normally(thesis, path, steps, "fp32")


@pytest.mark.parametrize("which", [1, 2, 3, 4])
def test_failed_allocation_in_context_creation(surface, thesis, monkeypatch, which):
    path, steps = surface
    monkeypatch.setenv("THESIS_GB300_FAIL_ALLOC", str(which))
    with pytest.raises(thesis.ThesisError) as e:
        thesis.Simulation(path, "fp32")
    assert e.value.status == CUDA
    assert "cudaMalloc" in str(e.value)
    monkeypatch.delenv("THESIS_GB300_FAIL_ALLOC")
    _runs_normally(thesis, path, steps, "fp32")
