"""Whole intervals on the device against pydyn's own driver (tests/golden/steps.json, made by
tests/golden/make_golden.py steps): after every interval -- Check_CFL on a copy of m and sp,
then its steps -- the (ndyn, n) Check_CFL chose and a sha1 over every state array of every
region, halos included, must equal the reference's.  Eagerly enqueued and replayed as one
captured CUDA graph per interval."""

import json
from pathlib import Path

import pytest
from make_golden import STATE_FIELDS, digest

GOLDEN = json.loads((Path(__file__).parent / "golden" / "steps.json").read_text())


def _device_digest(fw):
    st = fw.st
    return digest({r: {name: st[r][name].host() for name in STATE_FIELDS} for r in fw.zoom.regions()})


@pytest.mark.gpu
@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_intervals_match_reference(dev, name, graph):
    from pydyn_gb300.forward import Forward

    run = GOLDEN[name]
    fw = Forward(dev, run["config"], run["lm"], run["seed"], nt=run.get("nt", 1), umax=run.get("umax", 40.0),
                 physics=run.get("physics", False), lmax=run.get("lmax"))  # fmt: skip
    for k, (ndyn, n, want) in enumerate(run["steps"]):
        got_ndyn, got_n = fw.interval(graph=graph)
        assert (got_ndyn, got_n) == (ndyn, n), f"interval {k}: Check_CFL chose {got_ndyn, got_n}, reference {ndyn, n}"
        assert _device_digest(fw) == want, f"{name}: interval {k} differs from the reference"
    fw.close()
