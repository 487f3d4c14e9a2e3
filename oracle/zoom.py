"""ORACLE -- test infrastructure.  The region bodies of pydyn's zoom.host (pydyn zoom/host.py,
zoom/advect.py, zoom/check_cfl.py, zoom/massflow.py, zoom/exchange.py, zoom/physics.py) on host
NumPy arrays with Fortran bounds, the per-line and per-column work done by the C oracle
(oracle/src).  A HostState plugs into the package's operator sequence (pydyn_gb300.driver) the
way pydyn's ZoomState plugs into pydyn.zoom: the sequence is data-independent control, pinned
with the bodies by the whole-interval digests of pydyn itself (tests/golden/steps.json)."""

import sys

import numpy as np

from . import kernels as O

TRACERS = ("rm", "rxm", "rym", "rzm")
FIELDS = ("m", "rm", "rxm", "rym", "rzm", "am", "bm", "cm", "pu", "pv", "sp", "phlb", "dxyp")


class FA:
    """A NumPy array addressed with inclusive Fortran bounds; sections are views."""

    def __init__(self, data, lower):
        self.data, self.lower = data, tuple(lower)

    def _ix(self, item):
        if not isinstance(item, tuple):
            item = (item,)
        out = []
        for lo, ix in zip(self.lower, item, strict=False):
            if isinstance(ix, slice):
                out.append(slice(None if ix.start is None else ix.start - lo, None if ix.stop is None else ix.stop - lo + 1))
            else:
                out.append(ix - lo)
        return (*out, Ellipsis)

    def __getitem__(self, item):
        return self.data[self._ix(item)]

    def __setitem__(self, item, value):
        self.data[self._ix(item)] = value


def _bounds(name, im, jm, lm, nt):
    cells = [(-1, im + 2), (-1, jm + 2)]
    faces = [(0, im + 1), (0, jm + 1), (0, lm + 1)]
    table = {"m": [*cells, (1, lm)], "am": faces, "bm": faces, "cm": faces, "pu": [(0, im), (1, jm), (1, lm)],
             "pv": [(1, im), (1, jm + 1), (1, lm)], "sp": [*cells, (1, 1)], "phlb": [*cells, (1, lm + 1)],
             "dxyp": [(1, jm)]}  # fmt: skip
    for q in TRACERS:
        table[q] = [*cells, (1, lm), (1, nt)]
    return table[name]


class HostState:
    """Every region's host arrays (FA) and `lib` = this module's bodies."""

    def __init__(self, zoom, nt):
        self.zoom, self.nt = zoom, nt
        self.fields = {}
        for r in zoom.regions():
            g = zoom.g(r)
            self.fields[r] = {}
            for name in FIELDS:
                b = _bounds(name, g.im, g.jm, zoom.lm, nt)
                self.fields[r][name] = FA(np.zeros([hi - lo + 1 for lo, hi in b]), [lo for lo, _ in b])
        self.lib = sys.modules[__name__]
        self.saved = {}
        self.cfl_failed = False

    def __getitem__(self, r):
        return self.fields[r]

    def load(self, host_fields):
        for r, f in host_fields.items():
            for name, a in f.items():
                self.fields[r][name].data[...] = a

    def arrays(self):
        return {r: {k: v.data for k, v in f.items()} for r, f in self.fields.items()}


def _interior(st, r):
    g, f, lm = st.zoom.g(r), st[r], st.zoom.lm
    return [f["m"][1 : g.im, 1 : g.jm, 1:lm], *(f[q][1 : g.im, 1 : g.jm, 1:lm] for q in TRACERS)]


def _clust(zoom, r):
    g = zoom.g(r)
    return None if g.redgrid is None else g.redgrid.clust


# ------------------------------------------------------------------ region 1 advection (zoom/advect.py)
def _dynamu_region1(zoom, st, js, je, limits, stats, max_nloop=50):
    g, f, lm = zoom.g(1), st[1], zoom.lm
    m, *q = _interior(st, 1)
    O.advect_x(m, *q, f["am"][0 : g.im, 1 : g.jm, 1:lm], clust=_clust(zoom, 1), halo=True, js=js, je=je,
               limits=limits, max_nloop=max_nloop)  # fmt: skip


def _dynamv_region1(zoom, st, limits, stats, max_nloop=10):
    g, f, lm = zoom.g(1), st[1], zoom.lm
    m, *q = _interior(st, 1)
    O.advect_y(m, *q, f["bm"][1 : g.im, 1 : g.jm + 1, 1:lm], full=f["bm"].data, full_l0=1, limits=limits,
               max_nloop=max_nloop)  # fmt: skip


def _dynamw_region1(zoom, st, limits, stats, iter_limit=15):
    g, f, lm = zoom.g(1), st[1], zoom.lm
    m, *q = _interior(st, 1)
    O.advect_z(m, *q, f["cm"][1 : g.im, 1 : g.jm, 0:lm], limits=limits, iter_limit=iter_limit)


# ------------------------------------------------------------------ Check_CFL bodies (zoom/check_cfl.py)
def cfl_begin(st):
    st.cfl_failed = False


def cfl_all_ok(st):
    return not st.cfl_failed


def _dynamum_region1(zoom, st, js, je, max_nloop):
    if st.cfl_failed:
        return False
    g, f, lm = zoom.g(1), st[1], zoom.lm
    r = O.advect_x(f["m"][1 : g.im, 1 : g.jm, 1:lm], None, None, None, None, f["am"][0 : g.im, 1 : g.jm, 1:lm],
                   clust=_clust(zoom, 1), halo=True, js=js, je=je, max_nloop=max_nloop, mass_only=True)  # fmt: skip
    st.cfl_failed |= r is None
    return r is not None


def _dynamvm_region1(zoom, st, max_nloop):
    if st.cfl_failed:
        return False
    g, f, lm = zoom.g(1), st[1], zoom.lm
    r = O.advect_y(f["m"][1 : g.im, 1 : g.jm, 1:lm], None, None, None, None, f["bm"][1 : g.im, 1 : g.jm + 1, 1:lm],
                   max_nloop=max_nloop, mass_only=True)  # fmt: skip
    st.cfl_failed |= r is None
    return r is not None


def _dynamwm(zoom, st, region, is_, ie, js, je, iter_limit):
    if st.cfl_failed:
        return False
    g, f, lm = zoom.g(region), st[region], zoom.lm
    r = O.advect_z(f["m"][1 : g.im, 1 : g.jm, 1:lm], None, None, None, None, f["cm"][1 : g.im, 1 : g.jm, 0:lm],
                   scope=(is_ - 1, ie, js - 1, je), iter_limit=iter_limit, mass_only=True)  # fmt: skip
    st.cfl_failed |= r is None
    return r is not None


# ------------------------------------------------------------------ dynam0, m2phlb (zoom/massflow.py)
def dynam0(zoom, st, region, ndyn):
    g, f, lm = zoom.g(region), st[region], zoom.lm
    im, jm = g.im, g.jm
    for name in ("am", "bm", "cm"):
        f[name].data[...] = 0.0
    O.fluxes_from_meteo(f["pu"][0:im, 1:jm, 1:lm], f["pv"][1:im, 1 : jm + 1, 1:lm], zoom.bt, ndyn / (2.0 * g.tref),
                        f["am"][0:im, 1:jm, 1:lm], f["bm"][1:im, 1 : jm + 1, 1:lm], f["cm"][1:im, 1:jm, 0:lm])  # fmt: skip
    if g.xcyc == 1:
        a = f["am"]
        a[0, :, :] = a[im, :, :].copy()
        a[im + 1, :, :] = a[1, :, :].copy()


def m2phlb1(zoom, st, region=1):
    g, f, lm = zoom.g(region), st[region], zoom.lm
    f["sp"].data[...] = 0.0
    O.m2phlb(f["m"][1 : g.im, 1 : g.jm, 1:lm], f["sp"][1 : g.im, 1 : g.jm, 1], f["phlb"][1 : g.im, 1 : g.jm, 1 : lm + 1],
             f["dxyp"].data, zoom.at, zoom.bt)  # fmt: skip


def m2phlb(zoom, st, region):
    g, f, lm = zoom.g(region), st[region], zoom.lm
    f["sp"].data[...] = 0.0
    O.m2phlb(f["m"][1 : g.im, 1 : g.jm, 1:lm], f["sp"][1 : g.im, 1 : g.jm, 1], f["phlb"][1 : g.im, 1 : g.jm, 1 : lm + 1],
             f["dxyp"].data, zoom.at, zoom.bt, zoom.ref(region, "x"), zoom.ref(region, "y"), zoom.jbeg[region],
             st[g.parent]["dxyp"].data)  # fmt: skip


# ------------------------------------------------------------------ save / restore / scale / assign (zoom/host.py)
def assign(dst, src, region, names):
    for k in names:
        dst[region][k].data[...] = src[region][k].data


def save(st, key, names):
    st.saved[key] = {(r, k): f[k].data.copy() for r, f in st.fields.items() for k in names}


def restore(st, key):
    for (r, k), v in st.saved[key].items():
        st[r][k].data[...] = v


def scale(st, names, factor):
    for f in st.fields.values():
        for k in names:
            f[k].data[...] = f[k].data * factor


# ------------------------------------------------------------------ the children's exchange: none on a single region
class _Nothing:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False


def outer_x_faces_zeroed(zoom, st, region, second):
    if region != 1:
        raise NotImplementedError("oracle: children")
    return _Nothing()


def outer_y_faces_zeroed(zoom, st, region, second):
    if region != 1:
        raise NotImplementedError("oracle: children")
    return _Nothing()


def put_xedges(zoom, st, region, tracers=True):
    if zoom.children[region]:
        raise NotImplementedError("oracle: children")


def put_yedges(zoom, st, region, tracers=True):
    if zoom.children[region]:
        raise NotImplementedError("oracle: children")


def coarsen_ambm(zoom, st, region):
    if zoom.children[region]:
        raise NotImplementedError("oracle: children")
