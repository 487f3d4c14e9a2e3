"""ORACLE -- test infrastructure.  Whole read intervals on the host (pydyn forward.py:388-451
recomposed for a region tree): Check_CFL on a copy of m and sp, then each step's interpolated
meteo, Setup_MassFlow and the operator sequence -- the oracle's restatement of pydyn's driver
(oracle.driver) over the oracle's bodies (oracle.zoom) on the oracle's own region tree
(oracle.tree).  Only the synthetic inputs come from the package (pydyn_gb300.synth, a pure NumPy
generator that loads no native code)."""

import hashlib

import numpy as np

from pydyn_gb300 import synth

from . import driver as D
from . import tree as T
from .zoom import HostState

STATE_FIELDS = ("m", "rm", "rxm", "rym", "rzm", "am", "bm", "cm", "pu", "pv", "sp", "phlb")


def digest(st):
    h = hashlib.sha1()
    for r in sorted(st.fields):
        for name in STATE_FIELDS:
            h.update(np.ascontiguousarray(st[r][name].data, dtype="<f8").tobytes())
    return h.hexdigest()


def oracle_tree(zoom):
    """The oracle's own Zoom of a tree the input generator describes (its regions' parameters)."""
    regions = []
    for g in zoom.region[1:]:
        rg = g.redgrid
        if rg is not None:
            rg = T.RedGrid(rg.im, rg.jm, [row + 1 for row, _, _ in rg.bands], [c for _, c, _ in rg.bands])
        regions.append(T.Region(g.name, g.im, g.jm, g.xbeg, g.xend, g.ybeg, g.yend, g.xref, g.yref, g.zref, g.tref,
                                g.parent, g.xcyc, g.touch_sp, g.touch_np, rg))  # fmt: skip
    return T.Zoom(regions, zoom.lm, zoom.at, zoom.bt)


class OracleRun:
    def __init__(self, config, lm, seed, nt=1, umax=40.0, physics=False, lmax=None):
        """physics: False, True (or "full") or "convection", as pydyn_gb300.forward.Forward's."""
        gen_zoom, self.met, fields = synth.case(config, lm, seed, nt, umax=umax)
        self.zoom = oracle_tree(gen_zoom)
        self.st, self.cst = HostState(self.zoom, nt), HostState(self.zoom, nt)
        self.st.load(fields)
        for r in self.zoom.regions():
            self.cst[r]["dxyp"].data[...] = fields[r]["dxyp"]
        self.meteo = {r: [self.met.fluxes(r, k) for k in (0, 1)] for r in self.zoom.regions()}
        self.physics = None
        if physics:
            from .physics import OraclePhysics

            kind = "full" if physics is True else physics
            spec = synth.Physics(gen_zoom, self.met, seed, lm if lmax is None else lmax, kind=kind)
            self.physics = OraclePhysics(self.zoom, spec)
            self.physics.init(self.st)
        self.t = 0.0

    def interpolate(self, st, t):
        a1, a2 = synth.weights(t)
        for r in self.zoom.regions():
            (pu0, pv0), (pu1, pv1) = self.meteo[r]
            st[r]["pu"].data[...] = a1 * pu0 + a2 * pu1
            st[r]["pv"].data[...] = a1 * pv0 + a2 * pv1

    def interval(self, ndyn_max=3600, nread=3600):
        zoom, st, cst, t0 = self.zoom, self.st, self.cst, self.t
        for r in zoom.regions():
            for name in ("m", "sp"):
                cst[r][name].data[...] = st[r][name].data
        ndyn, n, _ = D.check_cfl_zoom(zoom, cst, ndyn_max, nread // ndyn_max, nread,
                                      lambda z, s, i, nd: self.interpolate(s, t0 + (i - 0.5) * nd))  # fmt: skip
        for k in range(n):
            self.interpolate(st, t0 + k * ndyn + ndyn / 2.0)
            D.setup_massflow(zoom, st, ndyn)
            conv, kw = (None, {}) if self.physics is None else self.physics.step(st, t0 + k * ndyn, ndyn)
            D.step(zoom, st, conv, ndyn, limits=True, **kw)
        self.t = t0 + nread
        return ndyn, n
