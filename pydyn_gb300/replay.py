"""The replay of a pydyn_dump set with the state on the GB300.

Two parts, as in pydyn (replay.py, gpu/engine.py):

`DeviceEngine` has the members pydyn's replay calls on its engine -- zeros, copy_into, put, host,
compare, report, chemistry, sync (pydyn gpu/engine.py:17-74; replay.py:291-353) -- for a device
ZoomState whose bodies are pydyn_gb300.zoom.  A dump array goes to the device as its file holds
it (Fortran order) and a device kernel copies the section the state needs; a comparison is made
on the device (gb_compare) and only its report comes back, the state never.  The report is the
reference's (harness.compare's keys and values).  `zeros` reuses a state it made before for the
same tree and tracer count, zeroed on the device, when no caller holds it any more (the replay
of one event holds one state), and makes a new one otherwise.  The free run, which reads state
arrays on the host, is not served.

`replay()` is the reference's replay of a set from the model's own inputs (replay.py:
_Session.run, replay_operator, replay_m2phlb, replay_massflow, replay_cfl, physics), on this
engine and the device bodies, for a machine without pydyn: the tree from the headers (checked
against them), then every event -- a bef_<op> / aft_<op> pair of x y z v s c through the
planner's calls for that position of the split order, each region's m2phlb, the massflow and
cfl groups (the data pairs interpolated on the device) -- with the reports of every state array.
Not replayed: Meteo_Setup_Mass (`meteo` events: the device's Poisson solve is not bitwise),
the inputs read from the model's files (`--meteo` etc.) and the free run.

    python -m pydyn_gb300.replay <dump_dir> [--tags x,y,z,v,s,c,cfl,massflow,m2phlb] [--limit N]
                                            [--rank R] [-v]
"""

import ctypes
import sys
from collections import Counter
from datetime import datetime, timedelta

import numpy as np

from . import _native as N
from . import kernels as K
from . import plan as P
from .device import DevArray
from .dump import FArray, load_events
from .state import ZoomState
from .tree import RedGrid, Region, Zoom

STATE = ("m", "rm", "rxm", "rym", "rzm", "am", "bm", "cm")
INNER = {"s": "emis", "c": "chem"}  # the operators whose pair encloses input events
KINDS = ("x", "y", "z", "v", "s", "c", "cfl", "massflow", "m2phlb")


# ------------------------------------------------------------------ host arrays on the device
def _f_strides(shape):
    out = [1]
    for n in shape[:-1]:
        out.append(out[-1] * n)
    return tuple(out)


def on_device(dev, a, lower=None):
    """(view, owner): a host array (FArray, or NumPy with `lower` bounds) on the device.  Data in
    Fortran order go up as they lie and are viewed with Fortran strides; others in C order.
    `owner` is the allocation to free."""
    if isinstance(a, FArray):
        data, lower = a.data, a.lower
    else:
        data = np.asarray(a)
        lower = (0,) * data.ndim if lower is None else tuple(lower)
    if data.ndim > 1 and data.flags.f_contiguous and not data.flags.c_contiguous:
        buf = DevArray.from_host(dev, data.ravel(order="K"))
        return buf.reshape_axes(data.shape, _f_strides(data.shape), lower), buf
    buf = DevArray.from_host(dev, np.ascontiguousarray(data), lower)
    return buf, buf


def _section(a, like):
    """The section of DevArray `a` over the bounds of `like` (lower / upper)."""
    return a[tuple(slice(lo, hi) for lo, hi in zip(like.lower, like.upper, strict=True))]


def _bits_to_float(b):
    return float(np.array([b], dtype=np.int64).view(np.float64)[0])


# ------------------------------------------------------------------ the engine
class DeviceEngine:
    """pydyn's replay engine for a state on the device (see the module's docstring)."""

    name = "gb300"
    fingerprint = False
    asynchronous = True

    def __init__(self, dev):
        self.dev = dev
        self._out = DevArray.zeros(dev, (0, 4), dtype=np.int64)
        self._states = {}

    # -------------------------------------------------------------- states
    def zeros(self, zm, nt):
        """A zero state of the tree with nt tracers: one made before and no longer held by
        anyone (its only references the engine's list and this loop), zeroed on the device, or a
        new one.  A caller that keeps a state across events keeps it from being reused."""
        pool = self._states.setdefault((id(zm), nt), [])
        for st in pool:
            if sys.getrefcount(st) <= 3:  # the pool's list, the loop variable, the call's argument
                for f in st.fields.values():
                    for a in f.values():
                        a.fill(0.0)
                st.saved.clear()
                return st
        st = ZoomState.zeros(self.dev, zm, nt)
        pool.append(st)
        return st

    def copy_into(self, view, arr):
        """view[...] = the dump array `arr` over view's bounds (which the dump must cover)."""
        if not arr.covers(view):
            raise ValueError(f"dump bounds {arr} do not cover {view.lower}..{view.upper}")
        src, owner = on_device(self.dev, arr)
        view.assign(_section(src, view))
        owner.free()

    def put(self, view, values):
        view.upload(values)

    def host(self, x, tag="verify"):
        return x.host() if isinstance(x, DevArray) else x

    # -------------------------------------------------------------- comparisons
    def _report(self, model, ours, name, model_value):
        """harness.compare(model, ours)'s report from gb_compare on two device views of one
        extent; model_value(index) the model's value at a 0-based index."""
        if model.shape != ours.shape:
            raise ValueError(f"{name}: shape {model.shape} vs {ours.shape}")
        va, vb = model.view(), ours.view()
        N.check(self.dev.L.gb_compare(self.dev.h, ctypes.byref(va), ctypes.byref(vb), self._out.ptr), "gb_compare")
        n_diff, max_ulp, max_abs, max_rel, first = (int(x) for x in self._out.host())
        if n_diff == 0:
            return {"name": name, "equal": True, "n_diff": 0, "max_ulp": 0, "max_abs": 0.0, "max_rel": 0.0}
        idx = tuple(int(i) for i in np.unravel_index(first, ours.shape))
        mine = ours[tuple(lo + i for lo, i in zip(ours.lower, idx, strict=True))].host()
        return {"name": name, "equal": False, "n_diff": n_diff, "max_ulp": max_ulp, "max_abs": _bits_to_float(max_abs),
                "max_rel": _bits_to_float(max_rel), "first": idx,
                "first_values": (float(model_value(idx)), float(np.asarray(mine).reshape(())))}  # fmt: skip

    def compare(self, view, arr, name):
        """The state array `view` against the dump array `arr` over view's bounds."""
        if not arr.covers(view):
            shape = tuple(hi - lo + 1 for lo, hi in zip(view.lower, view.upper, strict=True))
            raise ValueError(f"{name}: the dump's {arr} does not cover {shape} at {view.lower}")
        src, owner = on_device(self.dev, arr)
        window = arr.data[arr.window(view)]
        try:
            return self._report(_section(src, view), view, name, lambda i: window[i])
        finally:
            owner.free()

    def report(self, model, ours, name):
        """compare(model, ours) of arrays that are not state views: `model` a host array, `ours`
        a DevArray (or a host array, put on the device)."""
        model = np.asarray(model, dtype=float)
        own = None
        if not isinstance(ours, DevArray):
            ours, own = on_device(self.dev, np.asarray(ours, dtype=float))
        src, owner = on_device(self.dev, model, ours.lower)
        try:
            return self._report(src, ours, name, lambda i: model[i])
        finally:
            owner.free()
            if own is not None:
                own.free()

    # -------------------------------------------------------------- the operators' inputs
    def chemistry(self, inputs, dt_sec):
        """chem.loss_rates and chem.decay on the device: (loss (ni, nj, lm, 4), decay (ni, nj, lm))
        DevArrays.  inputs: loss_rates' keywords, arrays as DevArrays or host arrays."""
        owned, d = [], {}
        for k, v in inputs.items():
            if isinstance(v, DevArray):
                d[k] = v
            elif isinstance(v, np.ndarray):
                d[k], o = on_device(self.dev, v)
                owned.append(o)
        temper = d["temper"]
        ni, nj, lm = temper.shape
        loss = DevArray.zeros(self.dev, (0, ni - 1), (0, nj - 1), (0, lm - 1), (0, 3))
        decay = DevArray.zeros(self.dev, (0, ni - 1), (0, nj - 1), (0, lm - 1))
        fields = {k: d[k] for k in K.CHEM_FIELDS if k in d}
        K.loss_rates(temper, d["phlb"], d["lat"], fields, float(dt_sec), loss=loss, decay=decay,
                     oh_scale=inputs.get("oh_scale", 1.0),
                     cl_scale=inputs.get("cl_scale", 1.0), o1d_scale=inputs.get("o1d_scale", 1.0),
                     soil_rate=inputs.get("soil_rate", 0.0))  # fmt: skip
        self.dev.sync()
        for o in owned:
            o.free()
        return loss, decay

    def calc_kzz(self, *args):
        raise NotImplementedError("DeviceEngine.calc_kzz: the inputs read from the model's files are not replayed here")

    def column_pressure(self, zm, m, dxyp):
        raise NotImplementedError("DeviceEngine.column_pressure: the free run is not replayed here")

    def pipeline(self, zm, st, depth):
        raise NotImplementedError("DeviceEngine.pipeline: the free run is not replayed here")

    def sync(self):
        self.dev.sync()

    def free(self):
        for pool in self._states.values():
            for st in pool:
                for f in st.fields.values():
                    for a in f.values():
                        a.free()
        self._states = {}
        self._out.free()


def _zero_based(a):
    return a.reshape_axes(a.shape, a.strides, (0,) * a.ndim)


# ------------------------------------------------------------------ the tree from the headers
class TreeMismatch(ValueError):
    """The tree built from the headers is not the model's (footprint, children, split order)."""


def _tuple(v):
    return (v,) if isinstance(v, int) else tuple(v)


def _redgrid(meta):
    """The reduced grid a header declares (nred, jred, clustsize), or None."""
    if not meta.get("grid_reduced") or not meta.get("nred"):
        return None
    n = meta["nred"]
    return RedGrid(meta["im"], meta["jm"], _tuple(meta["jred"])[:n], _tuple(meta["clustsize"])[:n])


def build_tree(first):
    """The region tree of one moment's events {region: event}: region 1 global, each child's
    corners from its footprint on its parent (whose corners are known first: parents are
    numbered before their children), then checked against the headers."""
    m1 = first[1].meta
    corners = {1: (-180.0, -90.0)}
    regions = []
    for r in sorted(first):
        m = first[r].meta
        kw = {k: m[k] for k in ("xref", "yref", "zref", "tref", "parent", "xcyc", "touch_sp", "touch_np")}
        if r == 1:
            regions.append(Region(m["grid_name"], m["im"], m["jm"], redgrid=_redgrid(m), **kw))
            continue
        p = first[m["parent"]].meta
        # a cell of refinement (xref, yref) is 360 / (im1 xref) by 180 / (jm1 yref) degrees
        west = corners[m["parent"]][0] + (m["ibeg"] - 1) * (360.0 / (m1["im"] * p["xref"]))
        south = corners[m["parent"]][1] + (m["jbeg"] - 1) * (180.0 / (m1["jm"] * p["yref"]))
        corners[r] = (west, south)
        regions.append(Region(m["grid_name"], m["im"], m["jm"], xbeg=west,
                              xend=west + m["im"] * (360.0 / (m1["im"] * m["xref"])), ybeg=south,
                              yend=south + m["jm"] * (180.0 / (m1["jm"] * m["yref"])), **kw))  # fmt: skip
    zm = Zoom(regions, m1["lm"], first[1]["at"].data, first[1]["bt"].data)
    check_tree(zm, first)
    return zm


def check_tree(zm, first):
    bad = []
    for r, ev in first.items():
        m = ev.meta
        if "splitorder" not in m:
            if list(first) == [1]:
                continue
            raise TreeMismatch(f"region {r}: no zoom header (splitorder, children, footprint) in {ev.path}")
        if zm.splitorderzoom[r] != m["splitorder"]:
            bad.append(f"region {r} splitorder: model {m['splitorder']!r}, here {zm.splitorderzoom[r]!r}")
        if sorted(zm.children[r]) != sorted(_tuple(m.get("children", ()))):
            bad.append(f"region {r} children: model {m.get('children')}, here {zm.children[r]}")
        if r > 1:
            bad += [f"region {r} {k}: model {m[k]}, here {getattr(zm, k)[r]}" for k in ("ibeg", "iend", "jbeg", "jend")
                    if getattr(zm, k)[r] != m[k]]  # fmt: skip
    if bad:
        raise TreeMismatch("the tree is not the model's:\n  " + "\n  ".join(bad))


def infer_status(zm, events):
    """Sets from before the zoom header carry no `status`: each pair's position in the split
    order is the next one holding its operator after the region's last (pydyn replay.py:826-842)."""
    pos = {}
    for ev in events:
        if not ev.tag.startswith(("bef_", "aft_")) or "status" in ev.meta:
            continue
        order, r = zm.splitorderzoom[ev.region], ev.region
        if ev.tag.startswith("aft_"):
            ev.meta["status"] = pos[r] % len(order)
            continue
        p = pos.get(r, -1) + 1
        while order[p % len(order)] != ev.tag[-1]:
            p += 1
        pos[r] = p
        ev.meta["status"] = p % len(order)


# ------------------------------------------------------------------ one event
def date(t):
    return datetime(*t)


def interpol_fractions(t, t1, t2):
    """go_date InterpolFractions: the weights of t1 and t2 at the instant t."""
    ds, ds1 = (t2 - t1).total_seconds(), (t - t1).total_seconds()
    a2 = 0.5 if abs(ds) < np.finfo(float).tiny else ds1 / ds
    return 1.0 - a2, a2


def span(events, k):
    """(aft event, inner input events) of the bef_ event events[k]."""
    ev = events[k]
    aft, inner_tag = "aft_" + ev.tag[4:], INNER.get(ev.tag[-1])
    inner = []
    for e in events[k + 1 :]:
        if e.region != ev.region:
            continue
        if e.tag == aft:
            return e, inner
        if e.tag == inner_tag:
            inner.append(e)
        elif e.tag == ev.tag:
            break
    raise ValueError(f"{ev}: no matching {aft} event")


class _DumpedConvection:
    """The convection inputs of a bef_v event on the device, as the `v` body takes a run's
    physics (convec_region(zoom, st, region, ndyn, inverse))."""

    def __init__(self, engine, ev):
        im, jm = ev.meta["im"], ev.meta["jm"]
        self.lmax = ev["entu"].upper[2]
        self.owned, self.d = [], {}
        cells = (slice(1, im), slice(1, jm), slice(1, self.lmax))
        for k in ("entu", "detu", "entd", "detd", "dkg"):
            if k in ev:
                a, o = on_device(engine.dev, ev[k])
                self.d[k] = a[cells]
            else:  # a build without diffusion dumps no dkg: no diffusion term
                a = o = DevArray.zeros(engine.dev, (1, im), (1, jm), (1, self.lmax))
                self.d[k] = a
            self.owned.append(o)
        for k in ("cloud_top", "cloud_lfs"):
            a, o = on_device(engine.dev, ev[k])
            self.d[k] = a[cells[:2]]
            self.owned.append(o)
        # the two integer maps must share their strides (a single-precision layout is not dumped)
        if self.d["cloud_top"].strides != self.d["cloud_lfs"].strides:
            raise ValueError(f"{ev}: cloud_top and cloud_lfs differ in layout")

    def convec_region(self, zoom, st, region, ndyn, inverse="crout"):
        from .physics import _interior, _owned_cols

        if inverse != "crout":
            raise NotImplementedError("convec_region: the device solves with the Crout inverse only")
        d = self.d
        cols = _owned_cols(zoom, st, region)
        if cols.shape[0] == 0:
            return
        K.convec(*_interior(st, region), d["entu"], d["detu"], d["entd"], d["detd"], d["dkg"], d["cloud_top"],
                 d["cloud_lfs"], cols, ndyn / (2.0 * zoom.g(region).tref), self.lmax)  # fmt: skip

    def free(self):
        for o in self.owned:
            o.free()


def _injections(engine, inner):
    """The emission of an s pair's `emis` events on the device: [(x (im, jm), level, tracer)],
    x = ((emis month2dt) (mol_mass / mol_mass_e)) efrac (emis.inject, pydyn emis.py:52-54)."""
    out = []
    for ev in inner:
        m = ev.meta
        src, owner = on_device(engine.dev, ev["emis"])
        x = DevArray.zeros(engine.dev, *((0, n - 1) for n in src.shape))
        x.scaled(_zero_based(src), float(m["month2dt"]))
        x.scaled(x, float(m["mol_mass"]) / float(m["mol_mass_e"]))
        x.scaled(x, float(m["efrac"]))
        owner.free()
        out.append((x, m["l_level"], m["i_tracer"]))
    return out


def _chem_inputs(engine, zm, ev):
    """loss_rates' inputs of a chem event, cut to the region's scope (ch4_loss_kernel's cells),
    on the device; and the arrays to free."""
    m = ev.meta
    lm = m["lm"]
    si, sj = zm.scope(ev.region)
    i0, i1, j0, j1 = si.start + 1, si.stop, sj.start + 1, sj.stop
    owned, out = [], {}

    def up(name, sec):
        a, o = on_device(engine.dev, ev[name])
        owned.append(o)
        return a[sec]

    out["temper"] = up("temper", (slice(i0, i1), slice(j0, j1), slice(1, lm)))
    out["phlb"] = up("phlb", (slice(i0, i1), slice(j0, j1), slice(1, lm + 1)))
    out["oh_3d"] = up("oh_3d", (slice(i0, i1), slice(j0, j1), slice(1, lm)))
    lat = np.ascontiguousarray(ev["lat"][j0:j1])
    out["lat"], o = on_device(engine.dev, lat)
    owned.append(o)
    for k in ("press", "oh", "cl", "od"):
        out[f"strat_{k}"] = up(f"strat_{k}", (slice(j0, j1),))
    if m["trop_cl_sink"]:
        out["pl_trop"] = up("pl_trop", (slice(i0, i1), slice(j0, j1)))
        out["cl_trop"] = up("cl_trop", (slice(i0, i1), slice(j0, j1)))
    if m["soil_sink"]:
        out["soil"] = up("soil", (slice(i0, i1), slice(j0, j1)))
        out["soil_rate"] = m["soil_rate"]
    out.update({k: m[k] for k in ("oh_scale", "cl_scale", "o1d_scale")})
    return out, owned


def replay_operator(zm, bef, aft, inner, engine, inverse="crout"):
    """One bef_<op> .. aft_<op> pair: the reports of every state array (and of the loss rates
    of a c)."""
    r, op, status = bef.region, bef.tag[-1], bef.meta["status"]
    order = zm.splitorderzoom[r]
    if order[status] != op:
        raise ValueError(f"{bef}: status {status} is {order[status]!r} in the split order, not {op!r}")
    st = engine.zeros(zm, bef["rm"].data.shape[3])
    for k in STATE:
        engine.copy_into(st[r][k], bef[k])
    zm.status[r] = status
    reports = []
    if op in "xyz":
        P.replay(P.operator_calls(zm, r, status), zm, st, limits=bool(bef.meta["limits"]))
    elif op == "v":
        conv = _DumpedConvection(engine, bef)
        try:
            st.lib.convec_region(zm, st, r, conv, bef.meta["nconv"], inverse)
            engine.sync()
        finally:
            conv.free()
    elif op == "s":
        inj = _injections(engine, inner)
        st.lib.sources_region(zm, st, r, inj)
        engine.sync()
        for x, _, _ in inj:
            x.free()
    else:
        (ev,) = inner
        if ev.meta.get("isotopes"):
            raise NotImplementedError("chem: the isotope path is not transcribed")
        inputs, owned = _chem_inputs(engine, zm, ev)
        loss, decay = engine.chemistry(inputs, ev.meta["dt_sec"])
        for o in owned:
            o.free()
        reports.append(engine.report(ev["loss"].data, loss, "loss"))
        tracers = ev.meta["ch4_tracers"]
        st.lib.chemistry_region(zm, st, r, decay, _tuple(tracers))
        engine.sync()
        loss.free()
        decay.free()
    return reports + [engine.compare(st[r][k], aft[k], k) for k in STATE]


def replay_m2phlb(zm, ev, dxyp, engine):
    """m2phlb1 (region 1) or m2phlb (a child) on the event's air mass: sp and phlb."""
    st = engine.zeros(zm, 1)
    r, g = ev.region, zm.g(ev.region)
    engine.copy_into(st[r]["m"], ev["m"])
    for q, arr in dxyp.items():
        engine.copy_into(st[q]["dxyp"], arr)
    (st.lib.m2phlb1 if r == 1 else st.lib.m2phlb)(zm, st, r)
    phlb = st[r]["phlb"][1 : g.im, 1 : g.jm, 1 : zm.lm + 1]
    return [engine.compare(st[r]["sp"], ev["sp"], "sp"), engine.compare(phlb, ev["phlb"], "phlb")]


def _interpolate_into(engine, dst, ev, name, t):
    """dst = a1 data1 + a2 data2 over dst's bounds: the event's data pair of `name` (pu or pv)
    at the instant t (balance.time_interpolation with InterpolFractions' weights)."""
    a1, a2 = interpol_fractions(t, date(ev.meta["pu_t1"]), date(ev.meta["pu_t2"]))
    d1, o1 = on_device(engine.dev, ev[f"{name}1"])
    d2, o2 = on_device(engine.dev, ev[f"{name}2"])
    dst._box(9, _section(d1, dst), _section(d2, dst), a1, a2)
    engine.sync()
    o1.free()
    o2.free()


def replay_massflow(zm, evs, engine):
    """Setup_MassFlow from the massflow events {region: event}: each region's data pair
    interpolated to the step's middle against its pu, pv; then dynam0 / coarsen on the dumped
    m, pu, pv against am, bm, cm."""
    st = engine.zeros(zm, 1)
    reports = {r: [] for r in evs}
    for r, ev in evs.items():
        if "pu1" in ev:
            t1, t2 = date(ev.meta["tr1"]), date(ev.meta["tr2"])
            for name in ("pu", "pv"):
                _interpolate_into(engine, st[r][name], ev, name, t1 + (t2 - t1) / 2)
                g = zm.g(r)
                inner = st[r][name][0 : g.im, 1 : g.jm, 1 : zm.lm] if name == "pu" else \
                    st[r][name][1 : g.im, 1 : g.jm + 1, 1 : zm.lm]  # fmt: skip
                reports[r].append(engine.compare(inner, ev[name], name))
        for k in ("m", "pu", "pv", "dxyp"):
            engine.copy_into(st[r][k], ev[k])
    P.setup_massflow(zm, st, evs[1].meta["ndyn"])
    for r, ev in evs.items():
        reports[r] += [engine.compare(st[r][k], ev[k], k) for k in ("am", "bm", "cm")]
    return reports


def replay_cfl(zm, evs, engine, caps=P.CFL_CAPS):
    """Check_CFL of a read interval from its cfl events {region: event}: (ndyn, n, tries)."""
    st = engine.zeros(zm, 1)
    for r, ev in evs.items():
        for name in ("m", "sp", "dxyp"):
            engine.copy_into(st[r][name], ev[name])
    m = evs[1].meta
    t0 = date(m["tread1"])

    def interpolate(zoom, s, i, ndyn):
        t = t0 + timedelta(seconds=(i - 0.5) * ndyn)
        for r, ev in evs.items():
            for name in ("pu", "pv"):
                _interpolate_into(engine, s[r][name], ev, name, t)

    return P.check_cfl(zm, st, m["ndyn_in"], m["n_in"], m["nread"], interpolate=interpolate, caps=caps)


def scalar_report(name, model, ours):
    """harness.compare of two one-element arrays."""
    a, b = np.array([model], dtype=float), np.array([ours], dtype=float)
    ia, ib = a.view(np.int64)[0], b.view(np.int64)[0]
    if ia == ib:
        return {"name": name, "equal": True, "n_diff": 0, "max_ulp": 0, "max_abs": 0.0, "max_rel": 0.0}

    def ordered(i):
        return int(np.int64(np.iinfo(np.int64).min) - np.int64(i)) if i < 0 else int(i)

    with np.errstate(all="ignore"):
        d = abs(a[0] - b[0])
        ulp = int(abs(np.int64(ordered(ia)) - np.int64(ordered(ib))))
        rel = d / np.maximum(abs(a[0]), abs(b[0]))
    return {"name": name, "equal": False, "n_diff": 1, "max_ulp": ulp, "max_abs": float(d), "max_rel": float(rel),
            "first": (0,), "first_values": (float(a[0]), float(b[0]))}  # fmt: skip


# ------------------------------------------------------------------ the set
class Results(list):
    """[(event, kind, reports, notes)]; `failures` [(seq, tag, repr of the exception)]."""

    def __init__(self, items=(), failures=()):
        super().__init__(items)
        self.failures = list(failures)


def replay(dump_dir, dev, tags=None, limit=None, rank=None, verbose=False, out=None):
    """Every replayable event of a dump set on the device, each from the model's own inputs."""
    out = sys.stdout if out is None else out
    if rank is None:
        events = load_events(dump_dir, merge=True)
    else:
        events = [e for e in load_events(dump_dir) if e.meta.get("rank", 0) == rank]
    first = {}
    for e in events:
        first.setdefault(e.region, e)
    zm = build_tree(first)
    infer_status(zm, events)
    dxyp = {r: e["dxyp"] for r, e in first.items()}
    engine = DeviceEngine(dev)
    results, pending = Results(), {"cfl": {}, "massflow": {}}

    def wanted(kind):
        return tags is None or kind in tags

    def emit(ev, kind, reports, notes=None):
        if limit is None or len(results) < limit:
            results.append((ev, kind, reports, notes or {}))
            if verbose or not all(x["equal"] for x in reports):
                print(f"e{ev.seq:05d} {kind:>8} r{ev.region}  {summary_line(reports)}", file=out)

    try:
        for k, ev in enumerate(events):
            if limit is not None and len(results) >= limit:
                break
            kind = ev.tag[4:] if ev.tag.startswith("bef_") else ev.tag
            try:
                if ev.tag in pending and wanted(ev.tag):
                    group = pending[ev.tag]
                    group[ev.region] = ev
                    if len(group) < zm.nregions:
                        continue
                    pending[ev.tag] = {}
                    if ev.tag == "cfl":
                        ndyn, n, tries = replay_cfl(zm, group, engine)
                        reports = [scalar_report("ndyn", group[1].meta["ndyn_out"], ndyn),
                                   scalar_report("n", group[1].meta["n_out"], n)]  # fmt: skip
                        emit(group[1], "cfl", reports, {"iterations": tries, "ndyn": ndyn, "n": n})
                    else:
                        for r, reports in replay_massflow(zm, group, engine).items():
                            emit(group[r], "massflow", reports)
                    continue
                if ev.tag == "m2phlb":
                    if wanted("m2phlb"):
                        emit(ev, "m2phlb", replay_m2phlb(zm, ev, dxyp, engine))
                    continue
                if not ev.tag.startswith("bef_") or kind not in "xyzvsc" or not wanted(kind):
                    continue
                try:
                    aft, inner = span(events, k)
                except ValueError:  # the set ends inside the pair
                    continue
                notes = {"injections": len(inner)} if kind == "s" else {}
                emit(ev, kind, replay_operator(zm, ev, aft, inner, engine), notes)
                for e in (ev, aft, *inner):
                    e.release()
            except Exception as exc:  # recorded; the replay carries on with the next event
                results.failures.append((ev.seq, ev.tag, repr(exc)))
                print(f"e{ev.seq:05d} {ev.tag:>8}: FAILED {exc!r}", file=out)
    finally:
        engine.free()
    return results


def summary_line(reports):
    bad = [r for r in reports if not r["equal"]]
    if not bad:
        return "bitwise"
    return "  ".join(f"{r['name']} {r['max_ulp']} ulp ({r['n_diff']} cells)" for r in bad)


def summarize(results):
    """{kind: (events, bitwise events)}."""
    n, ok = Counter(), Counter()
    for _, kind, reports, _ in results:
        n[kind] += 1
        ok[kind] += all(r["equal"] for r in reports)
    return {k: (n[k], ok[k]) for k in n}


def main(argv=None):
    import argparse

    from .device import Device

    p = argparse.ArgumentParser(description="Replay a pydyn_dump set with the state on the GPU.")
    p.add_argument("dump_dir")
    p.add_argument("--tags", help="comma-separated subset of " + ",".join(KINDS))
    p.add_argument("--limit", type=int)
    p.add_argument("--rank", type=int)
    p.add_argument("-v", "--verbose", action="store_true")
    a = p.parse_args(argv)
    dev = Device(0)
    res = replay(a.dump_dir, dev, tags=None if a.tags is None else set(a.tags.split(",")), limit=a.limit,
                 rank=a.rank, verbose=a.verbose)  # fmt: skip
    for kind, (n, ok) in summarize(res).items():
        print(f"{kind:>8}: {ok}/{n} bitwise")
    for seq, tag, err in res.failures:
        print(f"e{seq:05d} {tag}: {err}")
    dev.close()
    return 0 if not res.failures and all(ok == n for n, ok in summarize(res).values()) else 1


if __name__ == "__main__":
    sys.exit(main())
