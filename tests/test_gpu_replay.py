"""The replay of a dump set with the state on the device (pydyn_gb300.replay) against pydyn's
replay of the same set (tests/golden/dumps.json: every event's kind, region, compared arrays and
verdict), a planted difference reported as the reference reports it, and the device comparison
(gb_compare) against the host restatement of the reference's report (oracle/compare.py)."""

import io
import json
import math
from pathlib import Path

import numpy as np
import pytest
from make_golden import DUMP_SETS, REPLAY_TAGS, write_dump_set

GOLD = json.loads((Path(__file__).parent / "golden" / "dumps.json").read_text())


def _same_report(got, want):
    assert set(got) == set(want), (got, want)
    for k, w in want.items():
        g = got[k]
        if isinstance(w, float) and math.isnan(w):
            assert isinstance(g, float) and math.isnan(g), (k, got, want)
        elif isinstance(w, tuple) and any(isinstance(x, float) and math.isnan(x) for x in w):
            assert all((math.isnan(a) and math.isnan(b)) or a == b for a, b in zip(g, w, strict=True)), (k, got, want)
        else:
            assert g == w, (k, got, want)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(DUMP_SETS))
def test_replay_on_device_matches_pydyns_replay(dev, tmp_path, name):
    from pydyn_gb300.replay import replay

    write_dump_set(name, tmp_path)
    res = replay(tmp_path, dev, tags=set(REPLAY_TAGS), out=io.StringIO())
    got = [[ev.seq, kind, ev.region, [r["name"] for r in reps], all(r["equal"] for r in reps)]
           for ev, kind, reps, _ in res]  # fmt: skip
    assert not res.failures, res.failures
    assert got == GOLD[name]["results"]
    assert all(row[4] for row in got)


@pytest.mark.gpu
def test_planted_difference_is_reported_as_the_reference_reports_it(dev, tmp_path):
    from oracle.compare import compare

    from pydyn_gb300.dump import load_events
    from pydyn_gb300.replay import replay

    d = tmp_path / "set"
    write_dump_set("two", d)
    target = sorted(d.glob("e*_aft_y_r2_p000_rm.bin"))[0]
    seq = int(target.name[1:6])
    before = load_events(d, tags={"aft_y"}, region=2)
    want_ok = next(e for e in before if e.seq == seq)["rm"].data.copy()
    raw = np.fromfile(target, dtype="<f8")
    k1, k2 = raw.size // 3, raw.size // 2
    raw[k1] = np.nextafter(raw[k1], np.inf)
    raw[k2] = -raw[k2] if raw[k2] != 0.0 else -0.0
    raw.tofile(target)
    planted = raw.reshape(want_ok.shape, order="F")
    res = replay(d, dev, tags={"y"}, out=io.StringIO())
    hits = [reps for ev, kind, reps, _ in res if kind == "y" and ev.region == 2 and ev.seq == seq - 1]
    assert len(hits) == 1  # the pair's bef_y, the event before the aft_y planted in
    reports = hits[0]
    rm = next(r for r in reports if r["name"] == "rm")
    _same_report(rm, compare(planted, want_ok, "rm"))
    assert all(r["equal"] for r in reports if r["name"] != "rm")


@pytest.mark.gpu
def test_engine_reuses_only_states_no_one_holds(dev):
    from pydyn_gb300 import synth
    from pydyn_gb300.replay import DeviceEngine

    engine = DeviceEngine(dev)
    zm = synth.tree("two", 4)
    a = engine.zeros(zm, 1)
    a[1]["m"].fill(5.0)
    b = engine.zeros(zm, 1)  # `a` is held: a new state
    assert b is not a and (a[1]["m"].host() == 5.0).all()
    a_id = id(a)
    del a
    c = engine.zeros(zm, 1)  # the first state is free again: reused, and zeroed
    assert id(c) == a_id and (c[1]["m"].host() == 0.0).all()
    assert engine.zeros(zm, 2) is not c  # another tracer count: another state
    del b, c
    engine.free()


@pytest.mark.gpu
def test_device_comparison_is_the_reference_report(dev):
    from oracle.compare import compare

    from pydyn_gb300.device import DevArray
    from pydyn_gb300.replay import DeviceEngine

    engine = DeviceEngine(dev)
    rng = np.random.default_rng(91)
    base = rng.standard_normal((7, 6, 5, 3)) * 10.0 ** rng.integers(-3, 4, (7, 6, 5, 3))
    cases = {"equal": lambda a: None}

    def ulps(a):
        a[1, 2, 3, 0] = np.nextafter(a[1, 2, 3, 0], np.inf)
        a[6, 5, 4, 2] = np.nextafter(np.nextafter(a[6, 5, 4, 2], -np.inf), -np.inf)

    def zeros(a):
        a[0, 0, 0, 0], a[2, 2, 2, 2] = -0.0, 0.0

    def nans(a):
        a[3, 1, 1, 1] = np.nan
        a[4, 4, 4, 1] = np.inf

    def big(a):
        a[5, 0, 2, 0] = -a[5, 0, 2, 0] * 1e300

    cases.update(ulps=ulps, zeros=zeros, nans=nans, big=big)
    for label, plant in cases.items():
        model = base.copy()
        model[2, 2, 2, 2] = -0.0
        ours = model.copy()
        plant(model)
        for layout in ("C", "F"):
            m = np.asarray(model, order=layout)
            dv = DevArray.from_host(dev, ours)
            got = engine.report(m, dv, label)
            _same_report(got, compare(model, ours, label))
            dv.free()
    engine.free()
