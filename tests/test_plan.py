"""The step planner against pydyn's own driver: for every traced tree, the calls the planner
issues for Setup_MassFlow, a whole step (with the sources / chemistry hooks) and a Check_CFL
rehearsal equal, call for call and argument for argument, the calls pydyn's zoom.setup_massflow,
zoom.step and zoom.check_cfl_zoom made on a recording lib (tests/golden/traces.json, made by
tests/golden/make_golden.py traces).  Also the oracle's restatement of pydyn's driver against
the same traces, and the package's region tree against the oracle's, attribute by attribute."""

import json
from contextlib import contextmanager
from pathlib import Path

import numpy as np
import pytest

from pydyn_gb300 import plan as P
from pydyn_gb300 import tree as T

TRACES = json.loads((Path(__file__).parent / "golden" / "traces.json").read_text())
MASS_ONLY = ("_dynamum_region1", "_dynamvm_region1", "_dynamwm", "_dynamum_child", "_dynamvm_child")


def _arg(a):
    if isinstance(a, tuple):
        return [_arg(x) for x in a]
    if isinstance(a, dict) and "lmax" in a:
        return "<conv>"
    if isinstance(a, np.integer):
        return int(a)
    return a


class Recorder:
    """A lib that records calls in the fixture's form; `report` keywords are dropped (the
    planner's own way of reading the rehearsal's outcome once per step)."""

    def __init__(self):
        self.calls = []

    def __getattr__(self, name):
        rec = self

        def row(args, kw, tag):
            first = 1 if name in ("save", "restore", "scale") else 2
            out = [tag, *[_arg(a) for a in args[first:]]]
            kw = {k: v for k, v in kw.items() if k != "report"}
            if kw:
                out.append({k: _arg(v) for k, v in kw.items()})
            return out

        if name in ("outer_x_faces_zeroed", "outer_y_faces_zeroed"):

            @contextmanager
            def cm(*args, **kw):
                rec.calls.append(row(args, kw, "enter:" + name))
                yield
                rec.calls.append(["exit:" + name])

            return cm
        if name == "cfl_all_ok":
            return lambda st: True

        def call(*args, **kw):
            r = row(args, kw, name)
            if name in MASS_ONLY:
                r.append({"return": True})
            rec.calls.append(r)
            return True if name in MASS_ONLY else None

        return call


class Bare:
    def __init__(self, lib):
        self.lib = lib


def _trees(module, name):
    t = TRACES["plans"][name]
    lm = t["lm"]
    at, bt = np.linspace(2000.0, 0.0, lm + 1), np.linspace(1.0, 0.0, lm + 1)
    return module.Zoom([module.Region(**kw) for kw in t["regions"]], lm, at, bt)


def _hooks(lib):
    def hook(kind):
        return lambda zoom, st, region: lib.calls.append([kind, region, zoom.status[region]])

    return hook("sources"), hook("chemistry")


@pytest.mark.parametrize("name", sorted(TRACES["plans"]))
def test_plan_equals_pydyn_driver(name):
    want = TRACES["plans"][name]
    zoom = _trees(T, name)
    conv = {r: {"lmax": zoom.lm} for r in zoom.regions()}
    lib = Recorder()
    st = Bare(lib)
    P.setup_massflow(zoom, st, 3600)
    assert lib.calls == want["massflow"]
    lib.calls = []
    sources, chemistry = _hooks(lib)
    P.step(zoom, st, conv, 3600, sources=sources, chemistry=chemistry)
    assert lib.calls == want["step"]
    assert zoom.status == [0] + [len(zoom.splitorderzoom[r]) for r in zoom.regions()]
    lib.calls = []
    assert P.check_cfl(zoom, st, 3600, 1, 3600) == (3600, 1, 1)
    assert lib.calls == want["check_cfl"]


@pytest.mark.parametrize("name", sorted(TRACES["plans"]))
def test_oracle_driver_equals_pydyn_driver(name):
    from oracle import driver as D
    from oracle import tree as OT

    want = TRACES["plans"][name]
    zoom = _trees(OT, name)
    conv = {r: {"lmax": zoom.lm} for r in zoom.regions()}
    lib = Recorder()
    st = Bare(lib)
    D.setup_massflow(zoom, st, 3600)
    assert lib.calls == want["massflow"]
    lib.calls = []
    sources, chemistry = _hooks(lib)
    D.step(zoom, st, conv, 3600, sources=sources, chemistry=chemistry)
    assert lib.calls == want["step"]
    lib.calls = []
    assert D.check_cfl_zoom(zoom, st, 3600, 1, 3600) == (3600, 1, 1)
    assert lib.calls == want["check_cfl"]


def test_plan_is_made_once_per_tree():
    zoom = _trees(T, "two")
    assert P.step_plan(zoom) is P.step_plan(zoom)
    assert P.rehearsal_plan(zoom) is P.rehearsal_plan(zoom)


def test_shorter_step():
    """The Check_CFL time-step ladder (pydyn cfl.py:208-213): multiples of 2 tref_max dividing
    the read interval."""
    assert P.shorter_step(3600, 3600, 1) == 1800
    assert P.shorter_step(1800, 3600, 1) == 1200
    assert P.shorter_step(3600, 3600, 2) == 1800
    assert P.shorter_step(1200, 3600, 4) == 720
    with pytest.raises(ValueError):
        P.shorter_step(2, 3600, 1)


@pytest.mark.parametrize("config", ["one", "two", "three", "glb6x4", "glb3x2", "glb3x2+nam1x1", "glb3x2+nam72x44"])
def test_tree_equals_the_oracle_tree(config):
    """The package's table-derived tree against the oracle's restatement of pydyn's Zoom."""
    from oracle.forward import oracle_tree

    from pydyn_gb300 import synth

    ours = synth.tree(config, 6)
    theirs = oracle_tree(ours)
    for name in ("children", "ibeg", "iend", "jbeg", "jend", "lbeg", "lend", "isr", "ier", "jsr", "jer",
                 "splitorderzoom"):  # fmt: skip
        assert getattr(ours, name) == getattr(theirs, name), name
    for r in ours.regions():
        assert (ours.zoomed[r] == theirs.zoomed[r]).all()
        assert (ours.edge[r] == theirs.edge[r]).all()
        assert (ours.owned(r) == theirs.owned(r)).all()
        for axis in "xyzt":
            assert ours.ref(r, axis) == theirs.ref(r, axis)
    assert ours.split_orders("xyzzyx", 3) == theirs.split_orders("xyzzyx", 3)
