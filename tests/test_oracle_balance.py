"""The oracle's Meteo_Setup_Mass balancing (oracle/balance.py) against pydyn's own
(tests/golden/balance.npz, made by tests/golden/make_golden.py balance): region 1's periodic
Poisson correction through NumPy's FFT and a child's Match and direct solve, bitwise, with
pydyn's number of tries and verdict."""

from pathlib import Path

import pytest
from conftest import assert_bitwise
from make_golden import load

CASES = load(Path(__file__).parent / "golden" / "balance.npz")


@pytest.mark.parametrize("name", ["balance0", "balance1"])
def test_region1_balance_equals_pydyn(name):
    from oracle import balance as OB

    ins, outs, meta = CASES[name]
    pu, pv = ins["pu"].copy(), ins["pv"].copy()
    tries, ok, _, _ = OB.setup_mass(pu, pv, ins["pw"], ins["sp1"], ins["sp2"], ins["levi_db"], ins["area"],
                                    meta["dt"])  # fmt: skip
    assert (tries, ok) == (meta["tries"], meta["ok"])
    assert_bitwise(pu, outs["pu"], "pu")
    assert_bitwise(pv, outs["pv"], "pv")


def test_child_balance_equals_pydyn():
    from oracle import balance as OB

    ins, outs, meta = CASES["balchild0"]
    ri, rj = meta["rf"][:2]
    mu, mv = OB.direct_matrices(ri, rj)
    assert_bitwise(mu, ins["m_to_u"], "m_to_u")
    assert_bitwise(mv, ins["m_to_v"], "m_to_v")
    pu, pv, pw, tries, ok = OB.setup_mass_child((ins["pu"], ins["pv"], ins["pw"]), (ins["ppu"], ins["ppv"], ins["ppw"]),
                                                ins["sp1"], ins["sp2"], ins["levi_db"], ins["area"], meta["dt"],
                                                tuple(meta["rf"]), mu, mv)  # fmt: skip
    assert (tries, ok) == (meta["tries"], meta["ok"])
    for k, v in (("pu", pu), ("pv", pv), ("pw", pw)):
        assert_bitwise(v, outs[k], k)


def test_unbalanced_input_is_refused():
    from oracle import balance as OB

    ins, _, meta = CASES["balance0"]
    # fluxes 1e5 times too large: a convergence of ~1e5 Pa/s against the pressure's tendency, far
    # beyond the pre-check's 1e-4 per second of relative mismatch
    pu = ins["pu"] * 1e5
    with pytest.raises(ValueError, match="unbalanced"):
        OB.setup_mass(pu, ins["pv"].copy(), ins["pw"], ins["sp1"], ins["sp2"], ins["levi_db"], ins["area"], meta["dt"])
