"""The oracle against the reference's own outputs (tests/golden/kernels.npz, made from pydyn by
tests/golden/make_golden.py): every kernel case bitwise, every error case the same error."""

from pathlib import Path

import pytest
from cases import run_oracle
from conftest import assert_bitwise
from make_golden import load

CASES = load(Path(__file__).parent / "golden" / "kernels.npz")


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_reference(built, name):
    ins, outs, meta = CASES[name]
    got, err = run_oracle(ins, meta)
    assert err == meta.get("error"), f"{name}: error {err} vs {meta.get('error')}"
    for k, v in outs.items():
        assert_bitwise(got[k], v, f"{name}.{k}")
