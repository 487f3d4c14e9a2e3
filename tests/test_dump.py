"""The dump reader (pydyn_gb300.dump) and the replay's host logic, on CPU.

The sets are written by the oracle (oracle/dumpset.py) into a temporary directory; their bytes,
the view pydyn's own reader takes of them (headers, bounds, values; merged ranks) and pydyn's
replay of them are pinned in tests/golden/dumps.json (made by tests/golden/make_golden.py
dumps).  Here: the writer makes exactly those bytes, this reader takes pydyn's reader's view,
the reader's errors, the tree rebuilt from the headers, and -- where the reference is
importable (PYDYN_REFERENCE) -- pydyn's reader and replay on the sets once more."""

import json
import os
import shutil
import sys
import types
from pathlib import Path

import numpy as np
import pytest
from make_golden import DUMP_SETS, REPLAY_TAGS, parse_digest, write_dump_set

GOLD = json.loads((Path(__file__).parent / "golden" / "dumps.json").read_text())


@pytest.fixture(scope="module")
def sets(tmp_path_factory, built):
    out = {}
    for name in DUMP_SETS:
        d = tmp_path_factory.mktemp(f"dump_{name}")
        (ndyn, n), sha = write_dump_set(name, d)
        out[name] = (d, ndyn, n, sha)
    return out


@pytest.mark.parametrize("name", sorted(DUMP_SETS))
def test_writer_makes_the_set_pydyn_checked(sets, name):
    d, ndyn, n, sha = sets[name]
    assert sha == GOLD[name]["sha1"]
    assert (ndyn, n) == (GOLD[name]["ndyn"], GOLD[name]["n"])


@pytest.mark.parametrize("name", sorted(DUMP_SETS))
def test_reader_takes_pydyns_view(sets, name):
    from pydyn_gb300.dump import load_events

    events = load_events(sets[name][0], merge=True)
    assert len(events) == GOLD[name]["events"]
    assert parse_digest(events) == GOLD[name]["parse"]


def test_reader_filters_and_sections(sets):
    from pydyn_gb300.dump import load_events

    d = sets["two"][0]
    evs = load_events(d, tags={"bef_x"}, region=2)
    assert evs and all(e.tag == "bef_x" and e.region == 2 for e in evs)
    ev = evs[0]
    g_im, g_jm, lm = ev.meta["im"], ev.meta["jm"], ev.meta["lm"]
    m = ev["m"]
    assert m.lower == (-1, -1, 1) and m.upper == (g_im + 2, g_jm + 2, lm)
    np.testing.assert_array_equal(ev.interior("m"), m.data[2 : g_im + 2, 2 : g_jm + 2, :])
    np.testing.assert_array_equal(m[3, 1:4], m.data[4, 2:6, :])  # an integer drops its axis
    am = ev["am"]
    np.testing.assert_array_equal(ev.interior("am"), am.data[0 : g_im + 1, 1 : g_jm + 1, 1 : lm + 1])
    assert "rm" in ev and "nothing" not in ev
    ev.release()
    assert ev.cached() == []


def test_reader_refuses_what_pydyn_dump_does_not_write(sets, tmp_path):
    from pydyn_gb300.dump import DumpError, Event

    src = sets["one"][0]
    meta = sorted(src.glob("*_bef_x_*.meta"))[0]
    text = meta.read_text()
    cut = tmp_path / meta.name
    cut.write_text("\n".join(line for line in text.splitlines() if not line.startswith("region")))
    with pytest.raises(DumpError, match="region"):
        Event(cut)
    bad = tmp_path / ("x" + meta.name)
    bad.write_text(text + "array broken = 1 2 3\n")
    with pytest.raises(DumpError, match="bad array"):
        Event(bad)
    bad.write_text(text + "array broken = 1 x\n")
    with pytest.raises(DumpError, match="not an array line"):
        Event(bad)
    short = tmp_path / meta.name.replace(".meta", "_m.bin")
    for p in src.glob(meta.stem + "_*.bin"):
        shutil.copy(p, tmp_path / p.name)
    short.write_bytes(short.read_bytes()[:-8])
    cut.write_text(text)
    ev = Event(cut)
    with pytest.raises(ValueError, match="values for bounds"):
        ev["m"]


def test_merge_refuses_ranks_that_disagree(sets, tmp_path):
    from pydyn_gb300.dump import RankMismatch, load_events

    d = tmp_path / "ranks"
    shutil.copytree(sets["two-ranks"][0], d)
    m1 = sorted(d.glob("e*_bef_z_r1_p001_m.bin"))[0]
    raw = np.fromfile(m1, dtype="<f8")
    raw[7] = np.nextafter(raw[7], np.inf)
    raw.tofile(m1)
    events = load_events(d, merge=True)
    ev = next(e for e in events if e.seq == int(m1.name[1:6]))
    with pytest.raises(RankMismatch, match="not replicated"):
        ev["m"]
    ev["rm"]  # the tracer arrays are split, not replicated: no check of one against another


def test_tree_from_the_headers(sets):
    from pydyn_gb300 import synth
    from pydyn_gb300.dump import load_events
    from pydyn_gb300.replay import build_tree

    for name, tree in (("two", "two"), ("one", "one")):
        events = load_events(sets[name][0])
        first = {}
        for e in events:
            first.setdefault(e.region, e)
        zm = build_tree(first)
        want = synth.tree(tree, first[1].meta["lm"])
        for attr in ("children", "ibeg", "iend", "jbeg", "jend", "splitorderzoom"):
            assert getattr(zm, attr) == getattr(want, attr), attr
        for r in zm.regions():
            assert (zm.owned(r) == want.owned(r)).all()
            assert (zm.g(r).redgrid is None) == (want.g(r).redgrid is None)


def test_tree_mismatch_is_refused(sets):
    from pydyn_gb300.dump import load_events
    from pydyn_gb300.replay import TreeMismatch, build_tree

    events = load_events(sets["two"][0])
    first = {}
    for e in events:
        first.setdefault(e.region, e)
    first[2].meta["ibeg"] += 1
    with pytest.raises(TreeMismatch):
        build_tree(first)


def test_scalar_report_is_the_reference_report():
    from oracle.compare import compare

    from pydyn_gb300.replay import scalar_report

    for a, b in ((3600.0, 3600.0), (3600.0, 1800.0), (0.0, -0.0), (1.0, np.nextafter(1.0, 2.0)), (2.0, np.nan)):
        want, got = compare(np.array([a]), np.array([b]), "x"), scalar_report("x", a, b)
        assert json.dumps(got, sort_keys=True) == json.dumps(want, sort_keys=True)


def _pydyn():
    ref = os.environ.get("PYDYN_REFERENCE")
    if not ref:
        pytest.skip("PYDYN_REFERENCE not set: the fixtures hold pydyn's view")
    sys.path.insert(0, ref)
    sys.modules.setdefault("netCDF4", types.SimpleNamespace(Dataset=None))
    import pydyn.dump
    import pydyn.replay

    return pydyn


@pytest.mark.parametrize("name", sorted(DUMP_SETS))
def test_pydyns_reader_and_replay_on_the_set(sets, name):
    import io

    pydyn = _pydyn()
    from make_golden import _gbmath

    d = sets[name][0]
    assert parse_digest(pydyn.dump.load_events(d, merge=True)) == GOLD[name]["parse"]
    pydyn.ops.use_libm(str(_gbmath()))
    res = pydyn.replay.replay(d, lapack="crout", tags=set(REPLAY_TAGS), out=io.StringIO())
    got = [[ev.seq, kind, ev.region, [r["name"] for r in reps], all(r["equal"] for r in reps)]
           for ev, kind, reps, _ in res]  # fmt: skip
    assert got == GOLD[name]["results"]
