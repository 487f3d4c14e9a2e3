"""ORACLE -- test infrastructure.  The region bodies of pydyn's zoom.host (pydyn zoom/host.py,
zoom/advect.py, zoom/check_cfl.py, zoom/massflow.py, zoom/exchange.py, zoom/physics.py) on host
NumPy arrays with Fortran bounds, the per-line and per-column work done by the C oracle
(oracle/src).  A HostState plugs into the oracle's restatement of pydyn's driver (oracle.driver) -- or
into the package's planned sequence, which the lockstep tests run on both sides -- the way
pydyn's ZoomState plugs into pydyn.zoom; the bodies and the sequence are pinned by the
whole-interval digests of pydyn itself (tests/golden/steps.json).  A mass-only body returns the
rehearsal's ok, as pydyn's do; `report` is accepted and ignored (the host knows at once)."""

import sys

import numpy as np

from . import exchange as X
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


def _dynamum_region1(zoom, st, js, je, max_nloop, report=True):
    if st.cfl_failed:
        return False
    g, f, lm = zoom.g(1), st[1], zoom.lm
    r = O.advect_x(f["m"][1 : g.im, 1 : g.jm, 1:lm], None, None, None, None, f["am"][0 : g.im, 1 : g.jm, 1:lm],
                   clust=_clust(zoom, 1), halo=True, js=js, je=je, max_nloop=max_nloop, mass_only=True)  # fmt: skip
    st.cfl_failed |= r is None
    return r is not None


def _dynamvm_region1(zoom, st, max_nloop, report=True):
    if st.cfl_failed:
        return False
    g, f, lm = zoom.g(1), st[1], zoom.lm
    r = O.advect_y(f["m"][1 : g.im, 1 : g.jm, 1:lm], None, None, None, None, f["bm"][1 : g.im, 1 : g.jm + 1, 1:lm],
                   max_nloop=max_nloop, mass_only=True)  # fmt: skip
    st.cfl_failed |= r is None
    return r is not None


def _dynamwm(zoom, st, region, is_, ie, js, je, iter_limit, report=True):
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
    """A save under "check_cfl" opens a rehearsal: its failure flag is cleared (as the device's)."""
    if key == "check_cfl":
        st.cfl_failed = False
    st.saved[key] = {(r, k): f[k].data.copy() for r, f in st.fields.items() for k in names}


def restore(st, key):
    for (r, k), v in st.saved[key].items():
        st[r][k].data[...] = v


def scale(st, names, factor):
    for f in st.fields.values():
        for k in names:
            f[k].data[...] = f[k].data * factor


# ------------------------------------------------------------------ the children (zoom/advect.py, check_cfl.py, exchange.py)
class _OuterFaces:
    """outer_{x,y}_faces_zeroed (zoom/advect.py:117-151): a child's outer interface fluxes zeroed
    around its advection in the second half of the parent step, restored after."""

    def __init__(self, arr, planes):
        self.arr, self.planes, self.kept = arr, planes, []

    def __enter__(self):
        for ix in self.planes:
            self.kept.append((ix, self.arr[ix].copy()))
            self.arr[ix] = 0.0
        return self

    def __exit__(self, *a):
        for ix, v in self.kept:
            self.arr[ix] = v
        return False


def outer_x_faces_zeroed(zoom, st, region, second):
    g = zoom.g(region)
    if region == 1 or not (second and g.im // g.xref < zoom.g(1).im):
        return _OuterFaces(None, [])
    xr = zoom.ref(region, "x")
    return _OuterFaces(st[region]["am"], [(xr - 1, slice(None), slice(None)), (g.im - xr + 1, slice(None), slice(None))])


def outer_y_faces_zeroed(zoom, st, region, second):
    g = zoom.g(region)
    if region == 1 or not second:
        return _OuterFaces(None, [])
    yr = zoom.ref(region, "y")
    planes = []
    if g.touch_sp != 1:
        planes.append((slice(None), yr, slice(None)))
    if g.touch_np != 1:
        planes.append((slice(None), g.jm - yr + 2, slice(None)))
    return _OuterFaces(st[region]["bm"], planes)


def put_xedges(zoom, st, region, tracers=True):
    X.put_xedges(zoom, st, region, tracers)


def put_yedges(zoom, st, region, tracers=True):
    X.put_yedges(zoom, st, region, tracers)


def mix_edges(zoom, st, region, tracers=True):
    X.mix_edges(zoom, st, region, tracers)


def update_parent(zoom, st, region, tracers=True):
    X.update_parent(zoom, st, region, tracers)


def _uncompress_xedges(zoom, st, region, js, je, ls, le, tracers=True):
    X.uncompress_xedges(zoom, st, region, js, je, ls, le, tracers)


def _uncompress_yedges(zoom, st, region, is_, ie, ls, le, tracers=True):
    X.uncompress_yedges(zoom, st, region, is_, ie, ls, le, tracers)


def _coarsen_block(zoom, st, region):
    X.coarsen_block(zoom, st, region)


def coarsen_ambm(zoom, st, region):
    X.coarsen_ambm(zoom, st, region)


def _dynamu_child(zoom, st, region, js, je, ls, le, limits, stats, max_nloop=50):
    X.compress_xedges(zoom, st, region, js, je, ls, le)
    g, f = zoom.g(region), st[region]
    xr = zoom.ref(region, "x")
    is_, ie = xr, g.im - xr + 1
    cells = (slice(is_ - 1, ie + 1), slice(js, je), slice(ls, le))
    O.advect_x_held(f["m"][cells], *(f[q][cells] for q in TRACERS), f["am"][is_ - 1 : ie, js:je, ls:le],
                    limits=limits, max_nloop=max_nloop)  # fmt: skip


def _dynamv_child(zoom, st, region, is_, ie, ls, le, limits, stats, max_nloop=10):
    X.compress_yedges(zoom, st, region, is_, ie, ls, le)
    g, f = zoom.g(region), st[region]
    yr = zoom.ref(region, "y")
    js, je = yr, g.jm - yr + 1
    cells = (slice(is_, ie), slice(js - 1, je + 1), slice(ls, le))
    O.advect_y_held(f["m"][cells], *(f[q][cells] for q in TRACERS), f["bm"][is_:ie, js : je + 1, ls:le],
                    f["bm"].data, ls, limits=limits, max_nloop=max_nloop)  # fmt: skip


def _dynamw_child(zoom, st, region, is_, ie, js, je, limits, stats, iter_limit=15):
    g, f, lm = zoom.g(region), st[region], zoom.lm
    m, *q = _interior(st, region)
    O.advect_z(m, *q, f["cm"][1 : g.im, 1 : g.jm, 0:lm], scope=(is_ - 1, ie, js - 1, je), limits=limits,
               iter_limit=iter_limit)  # fmt: skip


def _dynamum_child(zoom, st, region, js, je, ls, le, max_nloop, report=True):
    if st.cfl_failed:
        return False
    X.compress_xedges(zoom, st, region, js, je, ls, le, tracers=False)
    g, f = zoom.g(region), st[region]
    xr = zoom.ref(region, "x")
    is_, ie = xr, g.im - xr + 1
    ok = O.advect_x_held(f["m"][is_ - 1 : ie + 1, js:je, ls:le], None, None, None, None,
                         f["am"][is_ - 1 : ie, js:je, ls:le], max_nloop=max_nloop, mass_only=True)  # fmt: skip
    if not ok:
        st.cfl_failed = True
        return False
    X.uncompress_xedges(zoom, st, region, js, je, ls, le, tracers=False)
    X.mix_edges(zoom, st, region, tracers=False)
    return True


def _dynamvm_child(zoom, st, region, is_, ie, ls, le, max_nloop, report=True):
    if st.cfl_failed:
        return False
    X.compress_yedges(zoom, st, region, is_, ie, ls, le, tracers=False)
    g, f = zoom.g(region), st[region]
    yr = zoom.ref(region, "y")
    js, je = yr, g.jm - yr + 1
    ok = O.advect_y_held(f["m"][is_:ie, js - 1 : je + 1, ls:le], None, None, None, None,
                         f["bm"][is_:ie, js : je + 1, ls:le], f["bm"].data, ls, max_nloop=max_nloop,
                         mass_only=True)  # fmt: skip
    if not ok:
        st.cfl_failed = True
        return False
    X.uncompress_yedges(zoom, st, region, is_, ie, ls, le, tracers=False)
    X.mix_edges(zoom, st, region, tracers=False)
    return True


# ------------------------------------------------------------------ physics (zoom/physics.py)
def convec_region(zoom, st, region, conv, ndyn, inverse="crout"):
    """kernels.convec on the owned columns, dt = ndyn / (2 tref) (zoom/physics.py:33-52)."""
    if conv is None or conv["lmax"] == 0:
        return
    cols = np.argwhere(zoom.owned(region)).astype(np.int32)
    if len(cols) == 0:
        return
    dt = ndyn / (2.0 * zoom.g(region).tref)
    O.convec(*_interior(st, region), conv["entu"], conv["detu"], conv["entd"], conv["detd"], conv["cloud_top"],
             conv["cloud_lfs"], conv["dkg"], dt, conv["lmax"], cols=cols)  # fmt: skip


def sources_region(zoom, st, region, injections):
    """do_add_2d on the owned cells (zoom/physics.py:55-64)."""
    g, f = zoom.g(region), st[region]
    own = zoom.owned(region)
    for x, level, tracer in injections:
        rm = f["rm"][1 : g.im, 1 : g.jm, level, tracer]
        rzm = f["rzm"][1 : g.im, 1 : g.jm, level, tracer]
        rm[own] = rm[own] + x[own]
        rzm[own] = rzm[own] - x[own]


def chemistry_region(zoom, st, region, decay, tracers):
    """The scope's decay on the owned cells, factor 1.0 elsewhere (zoom/physics.py:67-78)."""
    g, f = zoom.g(region), st[region]
    factor = np.ones((g.im, g.jm, zoom.lm))
    factor[zoom.scope(region)] = decay
    factor[~zoom.owned(region)] = 1.0
    for t in tracers:
        for name in TRACERS:
            q = f[name][1 : g.im, 1 : g.jm, 1 : zoom.lm, t]
            q[...] = q * factor
