"""The device module held to pydyn's body contract, on the runs whose Check_CFL rejects steps
(config0-strong: glb6x4 at 160 m/s; two-reject: the two-region tree at 1000 m/s).

1. pydyn's own driver, call for call: tests/golden/traces.json holds every body call pydyn's
   zoom.check_cfl_zoom / setup_massflow / step made over its host bodies on these runs (made by
   tests/golden/make_golden.py traces), with each mass-only body's return.  The calls are issued
   on the device bodies in that order; every mass-only body must return what pydyn's returned,
   and after every interval the state's sha1 must be pydyn's (tests/golden/steps.json).
2. A driver that consumes the returns as pydyn's Check_CFL does (the oracle's restatement of
   pydyn's driver, oracle.driver) over the device bodies chooses pydyn's (ndyn, n) and ends
   every interval on pydyn's digest."""

import json
from pathlib import Path

import pytest
from make_golden import STATE_FIELDS, digest

HERE = Path(__file__).parent
TRACES = json.loads((HERE / "golden" / "traces.json").read_text())["runs"]
STEPS = json.loads((HERE / "golden" / "steps.json").read_text())


def _forward(dev, name):
    from pydyn_gb300.forward import Forward

    run = STEPS[name]
    return Forward(dev, run["config"], run["lm"], run["seed"], umax=run["umax"])


def _digest(fw):
    return digest({r: {k: fw.st[r][k].host() for k in STATE_FIELDS} for r in fw.zoom.regions()})


def _copy_m_sp(fw):
    for r in fw.zoom.regions():
        for k in ("m", "sp"):
            fw.cfl_st[r][k].assign(fw.st[r][k])


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(TRACES))
def test_pydyn_call_sequence_on_device(dev, name):
    fw = _forward(dev, name)
    zoom, lib = fw.zoom, fw.st.lib
    states = {"<main>": fw.st, "<cfl>": fw.cfl_st}
    cur, stack, k = fw.cfl_st, [], 0
    want = STEPS[name]["steps"]
    returns = 0
    for n_call, call in enumerate(TRACES[name]):
        head, args = call[0], list(call[1:])
        if head == "copy_m_sp":
            _copy_m_sp(fw)
            cur = fw.cfl_st
            continue
        if head == "interpolate":
            cur = states[args[0]]
            fw.put_weights(args[1])
            fw.interpolate(cur)
            continue
        if head == "interval":
            dev.sync()
            assert [args[0], args[1]] == want[k][:2]
            assert _digest(fw) == want[k][2], f"{name}: interval {k} differs from pydyn after its call sequence"
            k += 1
            continue
        if head.startswith("exit:"):
            stack.pop().__exit__(None, None, None)
            continue
        ret = args.pop()["return"] if args and isinstance(args[-1], dict) and "return" in args[-1] else None
        kw = args.pop() if args and isinstance(args[-1], dict) else {}
        args = [tuple(a) if isinstance(a, list) else a for a in args]
        if head == "convec_region":  # advection-only runs: convection over no level
            continue
        if head.startswith("enter:"):
            cm = getattr(lib, head[6:])(zoom, cur, *args, **kw)
            cm.__enter__()
            stack.append(cm)
            continue
        if head in ("save", "restore", "scale"):
            out = getattr(lib, head)(cur, *args, **kw)
        else:
            out = getattr(lib, head)(zoom, cur, *args, **kw)
        if ret is not None:
            returns += 1
            assert out is ret, f"{name}: call {n_call} {head}{tuple(args)} returned {out}, pydyn's {ret}"
    assert k == len(want) and not stack
    assert returns > 0
    fw.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(TRACES))
def test_pydyn_contract_driver_on_device(dev, name):
    from oracle import driver as D

    fw = _forward(dev, name)
    zoom = fw.zoom
    t = 0.0
    for k, (ndyn_want, n_want, sha) in enumerate(STEPS[name]["steps"]):
        _copy_m_sp(fw)
        t0 = t

        def interpolate(z, st, i, nd, t0=t0):
            fw.put_weights(t0 + (i - 0.5) * nd)
            fw.interpolate(st)

        ndyn, n, _ = D.check_cfl_zoom(zoom, fw.cfl_st, 3600, 1, 3600, interpolate)
        assert (ndyn, n) == (ndyn_want, n_want), f"{name}: interval {k}: Check_CFL chose {ndyn, n}"
        for s in range(n):
            fw.put_weights(t0 + s * ndyn + ndyn / 2.0)
            fw.interpolate(fw.st)
            D.setup_massflow(zoom, fw.st, ndyn)
            D.step(zoom, fw.st, None, ndyn, limits=True)
        dev.sync()
        assert _digest(fw) == sha, f"{name}: interval {k} differs from pydyn"
        t = t0 + 3600.0
    fw.close()
