"""Adjoint (calibration gradients) of probe temperatures.

CPU: the host walk in dual numbers reproduces the oracle's node lists bit for bit and its
tangents agree with central differences of the walk itself.  GPU: the forward equals the
oracle's temperatures at the probes (FP64 1e-7 K, FP32 0.01 K), and the adjoint gradient of
a squared-error loss matches central finite differences of the FP64 forward to 1e-4
relative, also through torch.autograd."""
import numpy as np
import pytest

TIMES = [4e-4, 9e-4, 1.6e-3]
FIELDS = ("xb", "yb", "zb", "phix", "phiy", "phiz", "dtau")


@pytest.fixture(scope="module")
def deck_path(tmp_path_factory, decks):
    return decks.small_adjoint().write(str(tmp_path_factory.mktemp("adj") / "small_adjoint"))


@pytest.fixture(scope="module")
def probes():
    rng = np.random.default_rng(11)
    return np.sort(rng.choice(40 * 30 * 10, 256, replace=False)).astype(np.int64)


def test_host_walk_matches_oracle_nodes(built_library, thesis, oracle, deck_path, probes):
    o = oracle(deck_path)
    with thesis.Adjoint(deck_path, probes, TIMES, "fp64") as adj:
        theta = adj.params()
        assert adj.num_params == 6 + 2 * 6         # a move to the start, 3 tracks, 2 hatch moves
        assert theta[0] == 200.0 and theta[1] == 0.35 and theta[2] == 50e-6
        for i, t in enumerate(TIMES):
            vals, _ = adj.host_nodes(theta, i)
            ref = o.nodes(t, False)
            assert vals.shape[1] == ref["xb"].size
            for j, f in enumerate(FIELDS):
                assert np.array_equal(vals[j], ref[f]), f
            np.testing.assert_allclose(np.log(vals[7]), ref["expmod"], rtol=0, atol=1e-12)


def test_host_tangents_match_central_differences(built_library, thesis, deck_path, probes):
    with thesis.Adjoint(deck_path, probes, TIMES, "fp64") as adj:
        theta = adj.params()
        vals, tan = adj.host_nodes(theta, 2, tangents=True)
        # per field and parameter, floored at 1e-6 of the field's largest tangent (parameters
        # that do not move a field leave only rounding noise in its differences)
        scale = np.maximum(np.max(np.abs(tan), axis=1, keepdims=True),
                           1e-6 * np.max(np.abs(tan), axis=(1, 2), keepdims=True)) + 1e-300
        for j in range(adj.num_params):
            step = 1e-7 * max(abs(theta[j]), 1e-4)
            tp, tm = theta.copy(), theta.copy()
            tp[j] += step
            tm[j] -= step
            vp, _ = adj.host_nodes(tp, 2)
            vm, _ = adj.host_nodes(tm, 2)
            if vp.shape != vals.shape or vm.shape != vals.shape:
                continue                                # a discrete change of the schedule
            fd = (vp - vm) / (2 * step)
            err = np.abs(fd - tan[:, :, j]) / scale[:, :, j]
            assert np.max(err) <= 1e-4, (j, np.max(err))


def test_bad_inputs(built_library, thesis, deck_path, decks, tmp_path):
    with pytest.raises(thesis.ThesisError):
        thesis.Adjoint(deck_path, np.array([10 ** 9]), TIMES)
    with pytest.raises(thesis.ThesisError):
        thesis.Adjoint(deck_path, np.array([1, 2]), [-1.0])
    multi = decks.small_multibeam()
    multi.mode, multi.scan_fracs, multi.tracking = "Snapshots", [100], "None"
    with pytest.raises(thesis.ThesisError) as e:
        thesis.Adjoint(multi.write(str(tmp_path / "mb")), np.array([1]), TIMES)
    assert e.value.status == 5


def _target(adj, theta):
    t = theta.copy()
    t[0] *= 1.1      # P
    t[2] *= 0.9      # Width_X
    t[5] *= 1.05     # alpha
    return adj.forward(t)


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-7), ("fp32", 0.01)])
def test_forward_matches_oracle(built_library, thesis, oracle, deck_path, probes, precision, tol):
    o = oracle(deck_path)
    with thesis.Adjoint(deck_path, probes, TIMES, precision) as adj:
        T = adj.forward(adj.params())
        for i, t in enumerate(TIMES):
            assert np.max(np.abs(T[i] - o.calc_T(t, probes))) <= tol


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_gradient_matches_central_differences(built_library, thesis, deck_path, probes, precision):
    with thesis.Adjoint(deck_path, probes, TIMES, "fp64") as ref, \
            thesis.Adjoint(deck_path, probes, TIMES, precision) as adj:
        theta = ref.params()
        target = _target(ref, theta)
        T = adj.forward(theta)
        grad = adj.backward(2.0 * (T - target))

        def loss(th):
            return float(np.sum((ref.forward(th) - target) ** 2))

        gmax = np.max(np.abs(grad))
        checked = 0
        for j in range(ref.num_params):
            step = 1e-6 * max(abs(theta[j]), 1e-4)
            tp, tm = theta.copy(), theta.copy()
            tp[j] += step
            tm[j] -= step
            same = all(ref.host_nodes(tp, i)[0].shape == ref.host_nodes(tm, i)[0].shape ==
                       ref.host_nodes(theta, i)[0].shape for i in range(len(TIMES)))
            if not same:
                continue
            fd = (loss(tp) - loss(tm)) / (2 * step)
            assert abs(grad[j] - fd) <= 1e-4 * abs(fd) + 1e-6 * gmax * max(abs(theta[j]), 1e-4) / max(abs(theta[j]), 1e-4), \
                (j, grad[j], fd)
            checked += 1
        assert checked >= ref.num_params - 2


@pytest.mark.gpu
def test_torch_autograd_function(built_library, thesis, deck_path, probes):
    torch = pytest.importorskip("torch")
    with thesis.Adjoint(deck_path, probes, TIMES, "fp32") as adj:
        theta0 = adj.params()
        target = torch.from_numpy(_target(adj, theta0))
        theta = torch.tensor(theta0, dtype=torch.float64, requires_grad=True)
        T = thesis.probe_temperatures(adj, theta)
        loss = ((T - target) ** 2).sum()
        loss.backward()
        direct = adj.backward(2.0 * (adj.forward(theta0) - target.numpy()))
        np.testing.assert_allclose(theta.grad.numpy(), direct, rtol=1e-12, atol=0)
        assert theta.grad[0] < 0          # more power lowers a loss whose target is hotter
