"""The sm_103a kernels against the reference's outputs (golden fixtures) and against the oracle
on larger seeded inputs: bitwise, every array the kernel writes; the same errors."""

import zlib
from pathlib import Path

import numpy as np
import pytest
from cases import TRACERS, run_device, run_oracle
from conftest import assert_bitwise
from make_golden import load

CASES = load(Path(__file__).parent / "golden" / "kernels.npz")


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_device_matches_reference(dev, name):
    ins, outs, meta = CASES[name]
    got, err = run_device(dev, ins, meta)
    assert err == meta.get("error"), f"{name}: error {err} vs {meta.get('error')}"
    for k, v in outs.items():
        assert_bitwise(got[k], v, f"{name}.{k}")


def _state(rng, im, jm, lm, nt, cfl):
    """Seeded admissible inputs: masses ~1e9, tracers with slopes, per-line fluxes of Courant ~cfl
    (x periodic rows of one sign; y and z closed lines moving each line to a positive target)."""
    m = 1e9 * rng.uniform(0.8, 1.2, (im, jm, lm))
    rm = m[..., None] * rng.uniform(0.5, 1.5, (im, jm, lm, nt)) * 1e-6
    slopes = [0.3 * rm * rng.uniform(-1, 1, rm.shape) for _ in range(3)]
    scale = cfl * m.mean()
    am = scale * rng.choice([-1.0, 1.0], (1, jm, lm)) * rng.uniform(0.8, 1.0, (im + 1, jm, lm))
    am[im] = am[0]

    def closed(axis, amp):
        target = m * (1.0 + amp * rng.uniform(-1, 1, m.shape))
        target *= m.sum(axis=axis, keepdims=True) / target.sum(axis=axis, keepdims=True)
        f = np.cumsum(m - target, axis=axis)
        shape = list(m.shape)
        shape[axis] = 1
        return np.concatenate([np.zeros(shape), f], axis=axis)

    amp = min(0.6 * cfl, 0.9)
    bm = closed(1, amp)
    bm[:, jm] = 0.0
    cm = closed(2, amp)
    cm[..., lm] = 0.0
    return {"m": m, "rm": rm, "rxm": slopes[0], "rym": slopes[1], "rzm": slopes[2]}, (am, bm, cm)


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(120, 90, 34, 1), (60, 45, 25, 2), (90, 70, 34, 1)])
@pytest.mark.parametrize("cfl", [0.3, 1.6])
@pytest.mark.parametrize("op", ["x", "y", "z", "xred"])
def test_device_matches_oracle_at_size(dev, shape, cfl, op):
    im, jm, lm, nt = shape
    rng = np.random.default_rng(zlib.crc32(repr((shape, cfl, op)).encode()))
    st, fluxes = _state(rng, im, jm, lm, nt, cfl)
    flux = fluxes["xyz".index(op[0])]
    ins = {**st, "flux": flux}
    if op == "xred":  # production-like bands: whole-row, coarse and fine clusters at both poles
        bands = {120: (40, 8, 4, 2), 60: (60, 20, 10, 5), 90: (30, 9, 3, 2)}[im]
        clust = np.ones(jm, dtype=np.int32)
        for k, c in enumerate(bands):
            clust[k] = clust[jm - 1 - k] = c
        ins["clust"] = clust
    meta = {"op": op}
    want, werr = run_oracle(ins, meta)
    got, gerr = run_device(dev, ins, meta)
    assert gerr == werr
    for k in ("m", *TRACERS, "flux") if werr is None else ():
        assert_bitwise(got[k], want[k], f"{op}.{k}")
