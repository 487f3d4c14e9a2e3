"""The adjoint (pydyn_gb300.adjoint): the transposes of a region-1 interval's tracer operators.

CPU: the fixture of the transposed reference operator (tests/golden/adjoint.npz, pydyn's own
interval applied to every basis vector of the `one` tree) is a transpose -- <A delta, y> equals
<delta, A^T y> within the reference itself -- and the cost's samples.  GPU: the device's
limits-off interval is bitwise pydyn's (A delta), the device adjoint of the same interval equals
the reference's transpose; the dot-product test <A x, y> = <x, A^T y>
to 1e-12 relative on glb6x4 and glb3x2 with physics; central finite differences of J against
the checkpointed gradient; the torch.autograd wrapper."""

from pathlib import Path

import numpy as np
import pytest
from conftest import assert_bitwise
from make_golden import load

from pydyn_gb300 import synth
from pydyn_gb300.adjoint import make_samples

FIX = load(Path(__file__).parent / "golden" / "adjoint.npz")["adjoint"]


def test_fixture_is_a_transpose():
    ins, outs, _ = FIX
    for k, y in enumerate(ins["y"]):
        lhs = float(np.dot(outs["A_delta"].ravel(), y.ravel()))
        rhs = float(np.dot(ins["delta"].ravel()[ins["index"]], outs["ATy"][k]))
        assert abs(lhs - rhs) <= 1e-12 * abs(lhs), (lhs, rhs)


def test_samples_are_seeded_and_inside():
    zoom = synth.tree("glb6x4", 25)
    s = make_samples(zoom, 168, 500, seed=3)
    assert s.shape == (500, 4)
    assert s[:, 0].min() >= 1 and s[:, 0].max() <= 168
    assert s[:, 1].max() < 60 and s[:, 2].max() < 45 and s[:, 3].max() < 25 and s.min() >= 0
    assert np.array_equal(s, make_samples(zoom, 168, 500, seed=3))


# ------------------------------------------------------------------ device
def _run(dev, config, lm, seed, lmax):
    from pydyn_gb300.adjoint import FluxGradient
    from pydyn_gb300.forward import Forward

    fw = Forward(dev, config, lm, seed, physics=True, lmax=lmax, limits=False)
    prob = FluxGradient(fw, 1, np.zeros((0, 4)), np.zeros(0))
    prob.set_flux(np.zeros((fw.zoom.g(1).im, fw.zoom.g(1).jm)))
    return fw, prob


@pytest.mark.gpu
def test_adjoint_is_the_reference_transpose(dev):
    ins, outs, meta = FIX
    fw, prob = _run(dev, meta["config"], meta["lm"], meta["seed"], meta["lmax"])
    got, atys = prob.interval_pair(ins["delta"], ins["y"])
    assert_bitwise(got, outs["A_delta"], "A delta: the limits-off interval, pydyn's bits")
    for k, aty in enumerate(atys):
        aty = aty.ravel()[ins["index"]]
        want = outs["ATy"][k]
        err = np.abs(aty - want).max() / np.abs(want).max()
        assert err <= 1e-12, f"y_{k}: A^T y differs from the reference's transpose by {err:.2e} (relative)"
    prob.close()
    fw.close()


@pytest.mark.gpu
@pytest.mark.parametrize("config,lm,seed", [("glb6x4", 25, 11), ("glb3x2", 34, 41)])
def test_dot_product(dev, config, lm, seed):
    fw, prob = _run(dev, config, lm, seed, lm)
    g = fw.zoom.g(1)
    rng = np.random.default_rng(9)
    shape = (4, g.im, g.jm, lm)
    scale = np.array([1.0, 0.3, 0.3, 0.3])[:, None, None, None]
    x = rng.random(shape) * scale
    y = (rng.random(shape) + 0.5) * scale
    ax, (aty,) = prob.interval_pair(x, [y])
    lhs, rhs = float(np.dot(ax.ravel(), y.ravel())), float(np.dot(x.ravel(), aty.ravel()))
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs), f"<Ax, y> = {lhs!r}, <x, A^T y> = {rhs!r}"
    prob.close()
    fw.close()


@pytest.mark.gpu
def test_gradient_against_central_differences(dev):
    from pydyn_gb300.adjoint import FluxGradient
    from pydyn_gb300.forward import Forward

    fw = Forward(dev, "glb6x4", 25, 11, physics=True, lmax=25, limits=False)
    hours = 4
    samples = make_samples(fw.zoom, hours, 60, seed=1)
    prob = FluxGradient(fw, hours, samples, np.zeros(len(samples)), every=2)
    flux = fw.physics.r[1]["flux"].host()
    prob.cost(flux)
    vals = np.concatenate([prob.rm_at[h][1] for h in range(1, hours + 1)])
    rows = np.concatenate([prob.rm_at[h][0] for h in range(1, hours + 1)])
    obs = np.empty(len(samples))
    obs[rows] = vals * (1.0 + 0.02 * np.random.default_rng(4).standard_normal(len(vals)))
    prob.obs = obs
    prob.cost(flux)
    grad = prob.gradient().host()
    picks = list(np.argsort(-np.abs(grad).ravel())[:4]) + list(np.random.default_rng(2).choice(grad.size, 2))
    for k in picks:
        i, j = np.unravel_index(k, grad.shape)
        h = 1e-6 * abs(flux[i, j])
        fp, fm = flux.copy(), flux.copy()
        fp[i, j] += h
        fm[i, j] -= h
        fd = (prob.cost(fp) - prob.cost(fm)) / (2.0 * h)
        tol = 1e-5 * abs(grad).max()
        assert abs(fd - grad[i, j]) <= tol, f"flux ({i}, {j}): FD {fd!r} vs adjoint {grad[i, j]!r}"
    prob.close()
    fw.close()


@pytest.mark.gpu
def test_torch_autograd_wrapper(dev):
    torch = pytest.importorskip("torch")
    from pydyn_gb300.adjoint import FluxGradient, ch4_flux_cost
    from pydyn_gb300.forward import Forward

    fw = Forward(dev, "one", 4, 23, physics=True, lmax=4, limits=False)
    samples = make_samples(fw.zoom, 3, 30, seed=2)
    prob = FluxGradient(fw, 3, samples, np.zeros(len(samples)), every=2)
    flux0 = fw.physics.r[1]["flux"].host()
    flux = torch.tensor(flux0, dtype=torch.float64, device="cuda", requires_grad=True)
    J = ch4_flux_cost(flux, prob)
    J.backward()
    assert float(J.detach()) == prob.cost(flux0)
    want = prob.gradient().host()
    np.testing.assert_array_equal(flux.grad.cpu().numpy(), want)
    prob.close()
    fw.close()
