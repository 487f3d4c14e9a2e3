"""The oracle's whole intervals against pydyn's own driver (tests/golden/steps.json): the
(ndyn, n) Check_CFL chooses and the sha1 over every state array after every interval."""

import json
from pathlib import Path

import pytest

GOLDEN = json.loads((Path(__file__).parent / "golden" / "steps.json").read_text())


@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_oracle_intervals_match_reference(built, name):
    from oracle.forward import OracleRun, digest

    run = GOLDEN[name]
    steps = run["steps"][: run.get("cpu_prefix", 8)]
    orc = OracleRun(run["config"], run["lm"], run["seed"], nt=run.get("nt", 1), umax=run.get("umax", 40.0),
                    physics=run.get("physics", False), lmax=run.get("lmax"))  # fmt: skip
    for k, (ndyn, n, want) in enumerate(steps):
        assert orc.interval() == (ndyn, n), f"interval {k}"
        assert digest(orc.st) == want, f"{name}: interval {k} differs from the reference"
