"""Meteo_Setup_Mass's balancing on the device (pydyn_gb300.meteo) against pydyn
(tests/golden/balance.npz) and the oracle (oracle/balance.py).

The periodic Poisson solve is a float64 discrete Fourier transform of the device's own, not
FFTW's or NumPy's, so region 1's balanced fluxes are compared within a tolerance written below:
the difference from pydyn's, over the largest correction pydyn applied, at most 1e-10 (a sum of
im + jm products carries a few ulp; the corrections are 1e-6 of the fluxes).  Everything else --
the mass change, the Match of a child to its parent, the direct solve's products with the same
matrices -- is bitwise.  The checks' verdicts and the number of tries are pydyn's."""

from pathlib import Path

import numpy as np
import pytest
from conftest import assert_bitwise
from make_golden import balance_inputs, load

CASES = load(Path(__file__).parent / "golden" / "balance.npz")
TOL = 1e-10  # |device - pydyn| / max |pydyn's correction|


def _up(dev, d):
    from pydyn_gb300.device import DevArray

    return {k: DevArray.from_host(dev, np.ascontiguousarray(v)) for k, v in d.items() if isinstance(v, np.ndarray)}


def _close(got, want, before, name):
    scale = np.abs(want - before).max()
    err = np.abs(got - want).max() / scale
    assert err <= TOL, f"{name}: {err:.3e} of the largest correction ({scale:.3e})"


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["balance0", "balance1"])
def test_region1_balance_matches_pydyn(dev, name):
    from pydyn_gb300 import meteo as M

    ins, outs, meta = CASES[name]
    d = _up(dev, ins)
    info = M.setup_mass(d["pu"], d["pv"], d["pw"], d["sp1"], d["sp2"], d["levi_db"], d["area"], meta["dt"])
    assert (info["tries"], info["ok"]) == (meta["tries"], meta["ok"])
    _close(d["pu"].host(), outs["pu"], ins["pu"], "pu")
    _close(d["pv"].host(), outs["pv"], ins["pv"], "pv")
    for a in d.values():
        a.free()


@pytest.mark.gpu
def test_region1_balance_at_size_matches_the_oracle(dev):
    """glb3x2's grid, 34 levels: the oracle's NumPy path and the device, within the tolerance;
    the balanced fluxes pass the tight check."""
    from oracle import balance as OB

    from pydyn_gb300 import meteo as M

    rng = np.random.default_rng(501)
    ins = balance_inputs(rng, 120, 90, 34)
    pu, pv = ins["pu"].copy(), ins["pv"].copy()
    tries, ok, _, post = OB.setup_mass(pu, pv, ins["pw"], ins["sp1"], ins["sp2"], ins["levi_db"], ins["area"],
                                       ins["dt"])  # fmt: skip
    d = _up(dev, ins)
    info = M.setup_mass(d["pu"], d["pv"], d["pw"], d["sp1"], d["sp2"], d["levi_db"], d["area"], ins["dt"])
    assert (info["tries"], info["ok"]) == (tries, ok) and ok
    assert abs(info["post"][0] - post[0]) <= 1e-6 * post[0] + 1e-18
    _close(d["pu"].host(), pu, ins["pu"], "pu")
    _close(d["pv"].host(), pv, ins["pv"], "pv")
    for a in d.values():
        a.free()


@pytest.mark.gpu
def test_mass_change_and_check_match_the_oracle(dev):
    from oracle import balance as OB

    from pydyn_gb300 import meteo as M

    ins = balance_inputs(np.random.default_rng(502), 40, 30, 12)
    d = _up(dev, ins)
    dm = M.fill_mass_change(dev, d["sp1"], d["sp2"], d["levi_db"], d["area"], ins["dt"])
    assert_bitwise(dm.host(), OB.fill_mass_change(ins["sp1"], ins["sp2"], ins["levi_db"], ins["area"], ins["dt"]), "dm")
    ok, rms, mav = M.check_mass_balance(dev, d["pu"], d["pv"], d["sp1"], d["sp2"], ins["dt"], d["area"], 1e-7, 1e-6)
    wok, wrms, wmav = OB.check_mass_balance(ins["pu"], ins["pv"], ins["sp1"], ins["sp2"], ins["dt"], ins["area"],
                                            1e-7, 1e-6)  # fmt: skip
    assert ok == wok and mav == wmav and abs(rms - wrms) <= 1e-12 * wrms
    dm.free()
    for a in d.values():
        a.free()


@pytest.mark.gpu
def test_child_balance_with_pydyn_matrices_is_bitwise(dev):
    """The child's Match and direct solve with pydyn's own direct matrices: pydyn's bits."""
    from pydyn_gb300 import meteo as M

    ins, outs, meta = CASES["balchild0"]
    d = _up(dev, ins)
    rf = M.Refinement(*meta["rf"])
    poisson = M.PoissonDirect(dev, rf.ri, rf.rj, matrices=(ins["m_to_u"], ins["m_to_v"]))
    pu, pv, pw, info = M.setup_mass_child((d["pu"], d["pv"], d["pw"]), (d["ppu"], d["ppv"], d["ppw"]), d["sp1"],
                                          d["sp2"], d["levi_db"], d["area"], meta["dt"], rf, poisson)  # fmt: skip
    assert (info["tries"], info["ok"]) == (meta["tries"], meta["ok"])
    for k, v in (("pu", pu), ("pv", pv), ("pw", pw)):
        assert_bitwise(v.host(), outs[k], k)
    assert_bitwise(d["pu"].host(), ins["pu"], "raw pu left as it was")
    poisson.free()
    for a in (*d.values(), pu, pv, pw):
        a.free()


@pytest.mark.gpu
def test_child_direct_matrices_match_pydyn(dev):
    """The direct matrices made by the device's periodic solve, against pydyn's (NumPy FFT)."""
    from pydyn_gb300 import meteo as M

    ins, _, meta = CASES["balchild0"]
    poisson = M.PoissonDirect(dev, *meta["rf"][:2])
    for got, want in ((poisson.m_to_u, ins["m_to_u"]), (poisson.m_to_v, ins["m_to_v"])):
        assert np.abs(got - want).max() <= TOL * np.abs(want).max()
    poisson.free()


@pytest.mark.gpu
@pytest.mark.parametrize("kind", [0, 1, 2])
def test_match_sum_matches_the_oracle(dev, kind):
    from oracle import balance as OB

    from pydyn_gb300 import meteo as M

    rng = np.random.default_rng(510 + kind)
    rf = (3, 2, 4, 9, 3, 7)
    ni, nj, lm = rf[3] - rf[2] + 1, rf[5] - rf[4] + 1, 6
    shapes = {0: ((13, 10, lm), (ni * 3 + 1, nj * 2, lm)), 1: ((12, 11, lm), (ni * 3, nj * 2 + 1, lm)),
              2: ((12, 10, lm), (ni * 3, nj * 2, lm))}  # fmt: skip
    pshape, cshape = shapes[kind]
    pg, tg = rng.standard_normal(pshape), rng.standard_normal(cshape)
    want = tg.copy()
    (OB.match_u_sum, OB.match_v_sum, OB.match_cell_sum)[kind](pg, want, rf)
    d = _up(dev, {"pg": pg, "tg": tg})
    M.match(kind, d["pg"], d["tg"], M.Refinement(*rf))
    assert_bitwise(d["tg"].host(), want, "matched")
    for a in d.values():
        a.free()
