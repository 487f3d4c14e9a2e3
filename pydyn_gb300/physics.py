"""The physics of a step on the device: Calc_Kzz per region at the step's start, and the `v`, `s`
and `c` operators on the columns each region owns (pydyn zoom/physics.py:33-78, with
diffusion.calc_kzz, chem.loss_rates / decay and the emission's do_add_2d), recomposed for a
region tree as pydyn forward.py:411-451 runs them for one region:

    Calc_Kzz     after Setup_MassFlow, on every region: spm the meteo surface pressure at the
                 step's middle, sp the region's own at the step's start, pu / pv the step's
    v            kernels.convec on the owned columns, dt = ndyn / (2 tref), dkg the step's; the
                 inverse of each column is kept for the step's second `v` of the same air mass
    s            flux x area x dt added to rm and taken from rzm at level 1, tracer 1
    c            the loss rates and decay exp(-L dt) of each owned cell, applied to the CH4
                 tracers' mass and slopes; OH carries a diurnal factor at the time of the
                 region's half step (status // 6) -- put in device memory before each step

Everything a step enqueues reads its time-dependent inputs (weights, OH factors, the step
counter) from device memory, so one captured graph serves every step."""

from contextlib import contextmanager

import numpy as np

from . import _native as N
from . import kernels as K
from .device import DevArray
from .state import TRACERS

N_OPERATORS = 6
LEVEL, TRACER, CH4_TRACERS = 1, 1, (1,)


def _interior(st, r):
    g, f, lm = st.zoom.g(r), st[r], st.zoom.lm
    return [f["m"][1 : g.im, 1 : g.jm, 1:lm], *(f[q][1 : g.im, 1 : g.jm, 1:lm] for q in TRACERS)]


class Physics:
    """The device-resident physics inputs of a run (from a pydyn_gb300.synth.Physics) and the
    bodies that use them."""

    def __init__(self, dev, zoom, spec, dxyp):
        """dxyp: {region: DevArray (jm)} the cell areas.  A spec of kind "convection" carries
        convection's inputs with a given dkg alone: no Calc_Kzz, emission or chemistry."""
        self.dev, self.zoom, self.spec = dev, zoom, spec
        self.full = spec.kind == "full"
        self.lmax = spec.lmax
        up = lambda a, dtype=np.float64: DevArray.from_host(dev, np.ascontiguousarray(a, dtype=dtype))  # noqa: E731
        self.at, self.bt = up(zoom.at), up(zoom.bt)
        self.epoch = DevArray.from_host(dev, np.zeros(1, dtype=np.int32))
        self.r = {}
        for r in zoom.regions():
            g, R = zoom.g(r), spec.region[r]
            own = zoom.owned(r)
            top = R["conv"]["cloud_top"]

            def listed(mask, top=top):  # deepest clouds first: a warp's columns share their matrices' zeros
                c = np.argwhere(mask).astype(np.int32)
                return c[np.argsort(-top[c[:, 0], c[:, 1]], kind="stable")]

            # the owned columns in two segments: outside every child's footprint, and inside one
            # (the footprint's edge under a child's ring, which update_parent writes first)
            inside = np.zeros_like(own)
            for ch in zoom.children[r]:
                inside[zoom.ibeg[ch] - 1 : zoom.iend[ch], zoom.jbeg[ch] - 1 : zoom.jend[ch]] = True
            cols = listed(own)
            ncol = len(cols)
            d = {
                "conv": {k: up(v, np.int32 if k.startswith("cloud") else np.float64) for k, v in R["conv"].items()},
                # dkg: Calc_Kzz's output each step, or the case's given field (convection-only inputs)
                "dkg": DevArray.zeros(dev, (0, g.im - 1), (0, g.jm - 1), (0, self.lmax - 1)) if self.full
                       else up(R["dkg"]),
                "cols": up(cols if ncol else np.zeros((0, 2)), np.int32),
                "ncol": ncol,
                "cache": self._inverse_cache(ncol),
                "dxyp": dxyp[r],
                "grid": ((g.xend - g.xbeg) / g.im, (g.yend - g.ybeg) / g.jm, float(g.ybeg)),
            }  # fmt: skip
            if self.full:
                d.update({
                    "t": up(R["kzz"]["t"]), "q": up(R["kzz"]["q"]),
                    "surface": [up(R["kzz"]["surface"][k]) for k in K.KZZ_SURFACE],
                    "spm": [up(s) for s in R["kzz"]["spm"]],
                    "spm_now": DevArray.zeros(dev, (0, g.im - 1), (0, g.jm - 1)),
                    "krates": DevArray.zeros(dev, (0, g.im - 1), (0, g.jm - 1), (0, zoom.lm - 1), (0, 1)),
                    "chem": {k: up(v) for k, v in R["chem"].items()},
                    "flux": up(R["flux"]),
                    "factors": DevArray.zeros(dev, (0, 2 * g.tref - 1), (0, g.im - 1)),
                    # chemistry's paired-call cache: 8 doubles per owned cell, keyed by the step counter
                    "chem_cache": DevArray.zeros(dev, (0, max(ncol, 1) * zoom.lm * 8 - 1)),
                })  # fmt: skip
            else:
                d["chem_cache"] = None
            segs = [("far", listed(own & ~inside)), ("edge", listed(own & inside))] if inside.any() else []
            d["segments"] = [{"name": "all", "cols": d["cols"], "ncol": ncol, "cache": d["cache"],
                              "chem_cache": d["chem_cache"]}] if not segs else [
                {"name": name, "cols": up(c if len(c) else np.zeros((0, 2)), np.int32), "ncol": len(c),
                 "cache": self._inverse_cache(len(c)),
                 "chem_cache": DevArray.zeros(dev, (0, max(len(c), 1) * zoom.lm * 8 - 1)) if self.full else None}
                for name, c in segs]  # fmt: skip
            if segs:  # the whole list's caches are the segments' now
                for a in (*d["cache"][:3], d["chem_cache"]):
                    if a is not None:
                        a.free()
                d["cache"], d["chem_cache"] = None, None
            self.r[r] = d
        self.ndyn = None

    def _inverse_cache(self, ncol):
        """Convection's kept inverses of ncol columns, the masses they were made from, their tags."""
        dev, n = self.dev, self.lmax
        return (DevArray.zeros(dev, (0, max(ncol, 1) * n * n - 1)), DevArray.zeros(dev, (0, max(ncol, 1) * n - 1)),
                DevArray.from_host(dev, np.full(max(ncol, 1), -1, dtype=np.int32)), self.epoch)  # fmt: skip

    # -------------------------------------------------------------- host side, outside capture
    pending = {}  # region -> (device, event): a forked preparation not yet joined
    only = None  # a segment name: the physics bodies act on that segment's columns alone

    def segment_names(self, region):
        return [s["name"] for s in self.r[region]["segments"]]

    @contextmanager
    def only_segment(self, name):
        """Inside the block the physics bodies act on one segment of the owned columns."""
        self.only = name
        try:
            yield
        finally:
            self.only = None

    def _segments(self, region):
        return [s for s in self.r[region]["segments"] if s["ncol"] and self.only in (None, s["name"])]

    def init_state(self, st):
        """sp and phlb of every region from its initial air mass (m2phlb1 / m2phlb), so that the
        first step's Calc_Kzz and chemistry see the pressures of the state they start from."""
        for r in self.zoom.regions():
            if r == 1:
                st.lib.m2phlb1(self.zoom, st, 1)
            else:
                st.lib.m2phlb(self.zoom, st, r)

    def put_factors(self, t0, ndyn):
        """The OH factors of every region's half steps of the step from t0, into device memory
        (stream-ordered: a step already enqueued still reads the previous ones)."""
        if not self.full:
            return
        for r, d in self.r.items():
            d["factors"].upload(self.spec.factors(r, t0, ndyn))

    # -------------------------------------------------------------- enqueued (capturable)
    def prepare(self, fwd, ndyn):
        """After Setup_MassFlow: the step counter, spm, Calc_Kzz of every region, and the rate
        constants of the step's temperature on the owned columns (every chemistry call of the
        step uses them).  Returns the driver's (conv, kwargs)."""
        self.prepare_step(ndyn)
        for r in self.r:
            self.prepare_region(fwd, r)
        return self.driver_args()

    def join(self, region):
        """A forked preparation of the region (pending) joins the stream the caller enqueues on
        (the device's current context): every stream that runs a body reading Calc_Kzz's
        output waits for it -- a region's physics can run on more than one stream (its
        segments) -- and a stream that waited already adds nothing but a redundant edge."""
        dev_event = self.pending.get(region)
        if dev_event is not None:
            dev, event = dev_event
            dev.wait(event)

    def join_all(self):
        """The run's stream waits for every forked preparation; the step is done with them."""
        for r in list(self.pending):
            self.join(r)
        self.pending = {}

    def prepare_step(self, ndyn):
        """The step's half-step length and the step counter (convection's kept inverses)."""
        self.ndyn = ndyn
        N.check(self.dev.L.gb_iadd(self.dev.h, self.epoch.ptr, 1), "gb_iadd")

    def prepare_region(self, fwd, r):
        """Region r's spm at the step's middle, Calc_Kzz and the rate constants (nothing for
        convection-only inputs)."""
        if not self.full:
            return
        d, g, f = self.r[r], self.zoom.g(r), fwd.st[r]
        fwd.interp_into(d["spm_now"], d["spm"][0], d["spm"][1])
        dx, dy, ybeg = d["grid"]
        K.calc_kzz(d["spm_now"], f["sp"][1 : g.im, 1 : g.jm, 1], f["pu"], f["pv"], d["t"], d["q"],
                   d["surface"], self.at, self.bt, d["dxyp"], self.lmax, dx, dy, ybeg, d["dkg"])  # fmt: skip
        if d["ncol"]:
            K.chem_krates(d["t"], d["krates"], d["cols"])

    def driver_args(self):
        """The driver's (conv, kwargs) of a prepared step."""
        if not self.full:
            return {r: self for r in self.r}, {}
        return {r: self for r in self.r}, {"sources": self.sources, "chemistry": self.chemistry}

    def convec_region(self, zoom, st, region, ndyn, inverse="crout"):
        if inverse != "crout":
            raise NotImplementedError("convec_region: the device solves with the Crout inverse only")
        self.join(region)
        d = self.r[region]
        c = d["conv"]
        dt = ndyn / (2.0 * zoom.g(region).tref)
        for s in self._segments(region):  # column by column: the segments' order changes nothing
            K.convec(*_interior(st, region), c["entu"], c["detu"], c["entd"], c["detd"], d["dkg"], c["cloud_top"],
                     c["cloud_lfs"], s["cols"], dt, self.lmax, cache=s["cache"])  # fmt: skip

    def sources(self, zoom, st, region):
        d = self.r[region]
        g, f = zoom.g(region), st[region]
        rm = f["rm"][1 : g.im, 1 : g.jm, 1 : zoom.lm]
        rzm = f["rzm"][1 : g.im, 1 : g.jm, 1 : zoom.lm]
        for s in self._segments(region):
            K.sources(rm, rzm, d["flux"], s["cols"], LEVEL, TRACER, area=d["dxyp"],
                      scale=self.spec.half_step(region, self.ndyn))  # fmt: skip

    def chemistry(self, zoom, st, region):
        self.join(region)
        d = self.r[region]
        g, f = zoom.g(region), st[region]
        h = zoom.status[region] // N_OPERATORS
        c = d["chem"]
        for s in self._segments(region):
            K.chemistry(d["t"], f["phlb"][1 : g.im, 1 : g.jm, 1 : zoom.lm + 1], c["lat"], c,
                        self.spec.half_step(region, self.ndyn), s["cols"], CH4_TRACERS, *_interior(st, region)[1:],
                        oh_factor=d["factors"][h], krates=d["krates"], cache=(s["chem_cache"], self.epoch),
                        **self.spec.settings)  # fmt: skip

    def free(self):
        seen = set()

        def rel(a):
            if isinstance(a, DevArray) and id(a) not in seen:
                seen.add(id(a))
                a.free()

        def walk(v):
            if isinstance(v, dict):
                for x in v.values():
                    walk(x)
            elif isinstance(v, (list, tuple)):
                for x in v:
                    walk(x)
            else:
                rel(v)

        for d in self.r.values():
            for k, v in d.items():
                if k != "dxyp":  # the state's
                    walk(v)
        for a in (self.at, self.bt, self.epoch):
            rel(a)


def convec_region(zoom, st, region, conv, ndyn, inverse="crout"):
    """The `v` body (zoom/physics.py:33): conv is the run's Physics."""
    conv.convec_region(zoom, st, region, ndyn, inverse)


def sources_region(zoom, st, region, injections):
    """The `s` body with explicit injections (zoom/physics.py:55): each (x (im, jm) DevArray kg,
    level, tracer) added to rm and taken from rzm on the owned cells."""
    g, f = zoom.g(region), st[region]
    cols = _owned_cols(zoom, st, region)
    for x, level, tracer in injections:
        K.sources(f["rm"][1 : g.im, 1 : g.jm, 1 : zoom.lm], f["rzm"][1 : g.im, 1 : g.jm, 1 : zoom.lm], x, cols, level,
                  tracer)  # fmt: skip


def chemistry_region(zoom, st, region, decay, tracers):
    """The `c` body with an explicit decay (zoom/physics.py:67): decay, a DevArray over the scope's
    cells (ni, nj, lm), multiplies the tracers' mass and slopes there, with factor 1.0 on the
    cells the region does not own (its children's footprints)."""
    g, f, lm = zoom.g(region), st[region], zoom.lm
    si, sj = zoom.scope(region)
    ni, nj = si.stop - si.start, sj.stop - sj.start
    fac = st.const(region, "chem_factor", lambda: np.ones((ni, nj, lm)))
    fac.assign(decay.reshape_axes(decay.shape, decay.strides))
    for i0, i1, j0, j1 in _footprints(zoom, region):
        fac[i0 - si.start : i1 - si.start, j0 - sj.start : j1 - sj.start].fill(1.0)
    for t in tracers:
        for name in TRACERS:
            q = f[name][si.start + 1 : si.stop, sj.start + 1 : sj.stop, 1:lm, t]
            q.binary("*", q, fac.reshape_axes(fac.shape, fac.strides, q.lower))


def _footprints(zoom, region):
    """The cells of the region's scope that it does not own, as inclusive 0-based boxes (i0, i1,
    j0, j1), one per child: the part of the child's footprint the child owns (the ring of parent
    cells under the child's edge stays the parent's).  Together exactly the scope's unowned
    cells."""
    si, sj = zoom.scope(region)
    own = zoom.owned(region)
    boxes, cover = [], np.zeros_like(own)
    for c in zoom.children[region]:
        i0, i1 = max(zoom.ibeg[c] - 1, si.start), min(zoom.iend[c] - 1, si.stop - 1)
        j0, j1 = max(zoom.jbeg[c] - 1, sj.start), min(zoom.jend[c] - 1, sj.stop - 1)
        if i0 > i1 or j0 > j1:
            continue
        taken = np.argwhere(~own[i0 : i1 + 1, j0 : j1 + 1])
        if len(taken) == 0:
            continue
        (a0, b0), (a1, b1) = taken.min(axis=0), taken.max(axis=0)
        box = (i0 + int(a0), i0 + int(a1), j0 + int(b0), j0 + int(b1))
        boxes.append(box)
        cover[box[0] : box[1] + 1, box[2] : box[3] + 1] = True
    scope = np.zeros_like(own)
    scope[si, sj] = True
    if not np.array_equal(cover, scope & ~own):
        raise NotImplementedError("chemistry_region: the scope's unowned cells are not the children's footprints")
    return boxes


def _owned_cols(zoom, st, region):
    return st.const(region, "owned_cols", lambda: np.argwhere(zoom.owned(region)).astype(np.int32))
