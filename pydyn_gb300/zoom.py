"""The device bodies the driver runs through `st.lib` -- the names of pydyn's zoom.host.BODIES
(pydyn zoom/host.py:42-48), each taking (zoom, st, region, ...) as the host body does and
leaving the device state as the host body leaves the host state.  Region 1's advection goes to
the row / column kernels on its interior views; a child's to the held-end kernels on its scope;
the exchange statements are box statements on Fortran sections.

The Check_CFL bodies keep pydyn's contract: each returns whether the rehearsal still holds
after it -- pydyn's Check_CFL takes that as the region's ok flag and unwinds at the first False
(pydyn zoom/check_cfl.py:87-91, 148-152, 201).  The outcome lives in a device flag that every
later rehearsal kernel honours; returning it costs one device-to-host read per body.  The
package's own planned rehearsal (pydyn_gb300.plan) passes report=False and reads the flag once
per rehearsed step instead (cfl_all_ok), so a rehearsal can be captured in a graph.  Nothing
else here waits for the device."""

from contextlib import contextmanager

import numpy as np

from . import kernels as K
from .state import TRACERS

BODIES = (
    "_coarsen_block _dynamu_child _dynamu_region1 _dynamum_child _dynamum_region1 _dynamv_child "
    "_dynamv_region1 _dynamvm_child _dynamvm_region1 _dynamw_child _dynamw_region1 _dynamwm "
    "_uncompress_xedges _uncompress_yedges assign chemistry_region coarsen_ambm convec_region dynam0 "
    "m2phlb m2phlb1 mix_edges outer_x_faces_zeroed outer_y_faces_zeroed put_xedges put_yedges "
    "restore save scale sources_region update_parent"
).split()


def _interior(st, r):
    """m and the tracers on the region's interior (pydyn zoom/state.py:45-50)."""
    g, f, lm = st.zoom.g(r), st[r], st.zoom.lm
    return [f["m"][1 : g.im, 1 : g.jm, 1:lm], *(f[q][1 : g.im, 1 : g.jm, 1:lm] for q in TRACERS)]


def _clust(st, r):
    g = st.zoom.g(r)
    if g.redgrid is None:
        return None
    return st.const(r, "clust", lambda: g.redgrid.clust.astype(np.int32))


def _levels(st):
    z = st.zoom
    return st.const(0, "at", lambda: z.at), st.const(0, "bt", lambda: z.bt)


# ------------------------------------------------------------------ region 1 advection
def _dynamu_region1(zoom, st, js, je, limits, stats, max_nloop=50):
    """dynamu(1): every row on the reduced grid, the periodic halos written (zoom/advect.py:237)."""
    g, f, lm = zoom.g(1), st[1], zoom.lm
    m, *q = _interior(st, 1)
    am = f["am"][0 : g.im, 1 : g.jm, 1:lm]
    K.advect_x(m, *q, am, clust=_clust(st, 1), halo=True, js=js, je=je, limits=limits, max_nloop=max_nloop)


def _dynamv_region1(zoom, st, limits, stats, max_nloop=10):
    """dynamv(1) on the interior, the whole halo'd bm layer rescaled (zoom/advect.py:201-226)."""
    g, f, lm = zoom.g(1), st[1], zoom.lm
    m, *q = _interior(st, 1)
    bm = f["bm"]
    K.advect_y(m, *q, bm[1 : g.im, 1 : g.jm + 1, 1:lm], bm_full=bm, bm_full_l0=1, limits=limits, max_nloop=max_nloop)


def _dynamw_region1(zoom, st, limits, stats, iter_limit=15):
    """dynamw(1) on the interior (zoom/advect.py:229-233)."""
    g, f, lm = zoom.g(1), st[1], zoom.lm
    m, *q = _interior(st, 1)
    K.advect_z(m, *q, f["cm"][1 : g.im, 1 : g.jm, 0:lm], limits=limits, iter_limit=iter_limit)


# ------------------------------------------------------------------ Check_CFL bodies
def cfl_begin(st):
    st.dev.cfl_reset()


def cfl_all_ok(st):
    """The rehearsal's outcome so far (a device -> host read of one flag)."""
    if st.dev.capturing:
        raise RuntimeError("Check_CFL: a captured rehearsal's outcome is read after the graph's replay")
    return not st.dev.cfl_failed()


def _outcome(st, report):
    """A mass-only body's return: the rehearsal's outcome after it (True when not reported)."""
    return cfl_all_ok(st) if report else True


def _dynamum_region1(zoom, st, js, je, max_nloop, report=True):
    """cfl.dynamum on region 1 with its halos (zoom/check_cfl.py:94-110)."""
    g, f, lm = zoom.g(1), st[1], zoom.lm
    K.cfl_x(f["m"][1 : g.im, 1 : g.jm, 1:lm], f["am"][0 : g.im, 1 : g.jm, 1:lm], clust=_clust(st, 1), halo=True,
            js=js, je=je, max_nloop=max_nloop)  # fmt: skip
    return _outcome(st, report)


def _dynamvm_region1(zoom, st, max_nloop, report=True):
    """cfl.dynamvm on region 1 (zoom/check_cfl.py:156-161)."""
    g, f, lm = zoom.g(1), st[1], zoom.lm
    K.cfl_y(f["m"][1 : g.im, 1 : g.jm, 1:lm], f["bm"][1 : g.im, 1 : g.jm + 1, 1:lm], max_nloop=max_nloop)
    return _outcome(st, report)


def _dynamwm(zoom, st, region, is_, ie, js, je, iter_limit, report=True):
    """dynamwm: the search over the region, the mass advanced on the scope (check_cfl.py:206)."""
    g, f, lm = zoom.g(region), st[region], zoom.lm
    K.cfl_z(f["m"][1 : g.im, 1 : g.jm, 1:lm], f["cm"][1 : g.im, 1 : g.jm, 0:lm], scope=(is_ - 1, ie, js - 1, je),
            iter_limit=iter_limit)  # fmt: skip
    return _outcome(st, report)


# ------------------------------------------------------------------ mass fluxes, pressure
def dynam0(zoom, st, region, ndyn):
    """advect.F90 dynam0 for any region (zoom/massflow.py:188-203): am, bm, cm zeroed whole,
    dt = ndyn / (2 tref), the cyclic x halo faces."""
    g, f, lm = zoom.g(region), st[region], zoom.lm
    im, jm = g.im, g.jm
    dt = ndyn / (2.0 * g.tref)
    for name in ("am", "bm", "cm"):
        f[name].fill(0.0)
    _, bt = _levels(st)
    K.fluxes_from_meteo(f["pu"][0:im, 1:jm, 1:lm], f["pv"][1:im, 1 : jm + 1, 1:lm], bt, dt,
                        f["am"][0:im, 1:jm, 1:lm], f["bm"][1:im, 1 : jm + 1, 1:lm], f["cm"][1:im, 1:jm, 0:lm])  # fmt: skip
    if g.xcyc == 1:
        a = f["am"]
        a[0, :, :].assign(a[im, :, :])
        a[im + 1, :, :].assign(a[1, :, :])


def m2phlb1(zoom, st, region=1):
    """m2phlb1 (zoom/massflow.py:24-32): sp zeroed whole, then sp and phlb from the column mass."""
    g, f, lm = zoom.g(region), st[region], zoom.lm
    at, bt = _levels(st)
    f["sp"].fill(0.0)
    K.m2phlb(f["m"][1 : g.im, 1 : g.jm, 1:lm], f["sp"][1 : g.im, 1 : g.jm, 1], f["phlb"][1 : g.im, 1 : g.jm, 1 : lm + 1],
             f["dxyp"], at, bt)  # fmt: skip


def m2phlb(zoom, st, region):
    """m2phlb of a child (zoom/massflow.py:35-56): the ring's pressure rescaled to the parent cell."""
    g, f, lm = zoom.g(region), st[region], zoom.lm
    at, bt = _levels(st)
    ring = (zoom.ref(region, "x"), zoom.ref(region, "y"), zoom.jbeg[region], st[g.parent]["dxyp"])
    f["sp"].fill(0.0)
    K.m2phlb(f["m"][1 : g.im, 1 : g.jm, 1:lm], f["sp"][1 : g.im, 1 : g.jm, 1], f["phlb"][1 : g.im, 1 : g.jm, 1 : lm + 1],
             f["dxyp"], at, bt, ring=ring)  # fmt: skip


# ------------------------------------------------------------------ save / restore / scale / assign
def assign(dst, src, region, names):
    for k in names:
        dst[region][k].assign(src[region][k])


def save(st, key, names):
    """Device copies of the named arrays of every region, for restore(st, key); the copies are
    kept and reused by the next save under the same key (fixed addresses for graph replay).
    A save under the key "check_cfl" opens a Check_CFL rehearsal and clears the device's
    rehearsal flag with it: pydyn's Check_CFL saves m and the fluxes at the start of every try
    (pydyn zoom/check_cfl.py:275) and calls nothing else a device could reset the flag in."""
    from .device import DevArray

    if key == "check_cfl":
        cfl_begin(st)
    slot = st.saved.setdefault(key, {})
    for r, f in st.fields.items():
        for k in names:
            a = f[k]
            if (r, k) not in slot:
                slot[(r, k)] = DevArray.zeros(st.dev, *((lo, lo + n - 1) for lo, n in zip(a.lower, a.shape, strict=True)))
            slot[(r, k)].assign(a)


def restore(st, key):
    for (r, k), v in st.saved[key].items():
        st[r][k].assign(v)


def scale(st, names, factor):
    for f in st.fields.values():
        for k in names:
            f[k].scaled(f[k], factor)


# ------------------------------------------------------------------ the exchange (children)
@contextmanager
def outer_x_faces_zeroed(zoom, st, region, second):
    """A child's outer x interface fluxes zeroed around its x advection in the second half of
    the parent step, restored after (zoom/advect.py:117-131)."""
    g = zoom.g(region)
    if region == 1 or not (second and g.im // g.xref < zoom.g(1).im):
        yield
        return
    xr = zoom.ref(region, "x")
    am = st[region]["am"]
    keep = _scratch_pair(st, region, "outer_x", am[xr - 1, :, :])
    keep[0].assign(am[xr - 1, :, :])
    keep[1].assign(am[g.im - xr + 1, :, :])
    am[xr - 1, :, :].fill(0.0)
    am[g.im - xr + 1, :, :].fill(0.0)
    yield
    am[xr - 1, :, :].assign(keep[0])
    am[g.im - xr + 1, :, :].assign(keep[1])


@contextmanager
def outer_y_faces_zeroed(zoom, st, region, second):
    """The same for a child's y interface fluxes (zoom/advect.py:134-151)."""
    g = zoom.g(region)
    if region == 1 or not second:
        yield
        return
    yr = zoom.ref(region, "y")
    bm = st[region]["bm"]
    keep = _scratch_pair(st, region, "outer_y", bm[:, yr, :])
    if g.touch_sp != 1:
        keep[0].assign(bm[:, yr, :])
        bm[:, yr, :].fill(0.0)
    if g.touch_np != 1:
        keep[1].assign(bm[:, g.jm - yr + 2, :])
        bm[:, g.jm - yr + 2, :].fill(0.0)
    yield
    if g.touch_sp != 1:
        bm[:, yr, :].assign(keep[0])
    if g.touch_np != 1:
        bm[:, g.jm - yr + 2, :].assign(keep[1])


def _scratch_pair(st, region, key, like):
    from .device import DevArray

    k = (region, key)
    if k not in st.consts:
        shape = like.shape
        st.consts[k] = tuple(DevArray.zeros(st.dev, *((0, n - 1) for n in shape)) for _ in range(2))
    return st.consts[k]


def put_xedges(zoom, st, region, tracers=True):
    from . import exchange

    exchange.put_xedges(zoom, st, region, tracers)


def put_yedges(zoom, st, region, tracers=True):
    from . import exchange

    exchange.put_yedges(zoom, st, region, tracers)


def update_parent(zoom, st, region, tracers=True):
    from . import exchange

    exchange.update_parent(zoom, st, region, tracers)


def mix_edges(zoom, st, region, tracers=True):
    from . import exchange

    exchange.mix_edges(zoom, st, region, tracers)


def _uncompress_xedges(zoom, st, region, js, je, ls, le, tracers=True):
    from . import exchange

    exchange.uncompress_xedges(zoom, st, region, js, je, ls, le, tracers)


def _uncompress_yedges(zoom, st, region, is_, ie, ls, le, tracers=True):
    from . import exchange

    exchange.uncompress_yedges(zoom, st, region, is_, ie, ls, le, tracers)


def _coarsen_block(zoom, st, region):
    from . import exchange

    exchange.coarsen_block(zoom, st, region)


def coarsen_ambm(zoom, st, region):
    from . import exchange

    exchange.coarsen_ambm(zoom, st, region)


def _dynamu_child(zoom, st, region, js, je, ls, le, limits, stats, max_nloop=50):
    from . import child

    child.dynamu(zoom, st, region, js, je, ls, le, limits, max_nloop)


def _dynamv_child(zoom, st, region, is_, ie, ls, le, limits, stats, max_nloop=10):
    from . import child

    child.dynamv(zoom, st, region, is_, ie, ls, le, limits, max_nloop)


def _dynamw_child(zoom, st, region, is_, ie, js, je, limits, stats, iter_limit=15):
    """dynamw of a child: the search over the whole region, the sub-steps on the scope
    (zoom/advect.py:444-472)."""
    g, f, lm = zoom.g(region), st[region], zoom.lm
    m, *q = _interior(st, region)
    K.advect_z(m, *q, f["cm"][1 : g.im, 1 : g.jm, 0:lm], scope=(is_ - 1, ie, js - 1, je), limits=limits,
               iter_limit=iter_limit)  # fmt: skip


def _dynamum_child(zoom, st, region, js, je, ls, le, max_nloop, report=True):
    """dynamum (mass only) of a child with its edge exchange (zoom/check_cfl.py:113-137)."""
    from . import child

    child.dynamum(zoom, st, region, js, je, ls, le, max_nloop)
    return _outcome(st, report)


def _dynamvm_child(zoom, st, region, is_, ie, ls, le, max_nloop, report=True):
    """dynamvm (mass only) of a child with its edge exchange (zoom/check_cfl.py:164-193)."""
    from . import child

    child.dynamvm(zoom, st, region, is_, ie, ls, le, max_nloop)
    return _outcome(st, report)


# ------------------------------------------------------------------ physics on owned cells
def convec_region(zoom, st, region, conv, ndyn, inverse="crout"):
    from . import physics

    physics.convec_region(zoom, st, region, conv, ndyn, inverse)


def sources_region(zoom, st, region, injections):
    from . import physics

    physics.sources_region(zoom, st, region, injections)


def chemistry_region(zoom, st, region, decay, tracers):
    from . import physics

    physics.chemistry_region(zoom, st, region, decay, tracers)
