"""The parent <-> child exchange bodies on the device: each a single fused kernel of
csrc/exchange.cu over the regions' whole (halo'd) arrays.  Reference: pydyn zoom/exchange.py
(put_xedges :17, put_yedges :63, _compress/_uncompress :108-175, mix_edges :178,
update_parent :233) and zoom/massflow.py (_coarsen_block :334, coarsen_ambm :400)."""

import ctypes

from . import _native as N
from .state import TRACERS

_REGION_FIELDS = ("m", *TRACERS, "am", "bm", "cm")


def _views(st, r):
    """The eight gb_views (m, rm, rxm, rym, rzm, am, bm, cm) of region r, as a ctypes array."""
    key = ("views", r)
    if key not in st.consts:
        arr = (N.GBView * 8)()
        for k, name in enumerate(_REGION_FIELDS):
            arr[k] = st[r][name].view()
        st.consts[key] = arr
    return st.consts[key]


def _lib(st):
    return st.dev.L, st.dev.h


def _wide(zoom, r):
    """A region spanning 360 degrees: periodic boundaries instead of x edges."""
    g = zoom.g(r)
    return g.im // g.xref == zoom.g(1).im


def put_xedges(zoom, st, region, tracers=True):
    L, h = _lib(st)
    for child in zoom.children[region]:
        if _wide(zoom, child):
            continue
        xr, yr, zr = (zoom.ref(child, a) for a in "xyz")
        N.check(L.gb_put_xedges(h, _views(st, region), _views(st, child), zoom.ibeg[child], zoom.iend[child],
                                zoom.jbeg[child], zoom.lbeg[child], xr, yr, zr, 1.0 / (yr * zr), 1.0 / (xr * yr * zr),
                                int(tracers)), "put_xedges")  # fmt: skip


def put_yedges(zoom, st, region, tracers=True):
    L, h = _lib(st)
    for child in zoom.children[region]:
        xr, yr, zr = (zoom.ref(child, a) for a in "xyz")
        N.check(L.gb_put_yedges(h, _views(st, region), _views(st, child), zoom.jbeg[child], zoom.jend[child],
                                zoom.ibeg[child], zoom.lbeg[child], xr, yr, zr, 1.0 / (xr * zr), 1.0 / (xr * yr * zr),
                                int(tracers)), "put_yedges")  # fmt: skip


def compress_xedges(zoom, st, region, js, je, ls, le, tracers=True):
    xr = zoom.ref(region, "x")
    if xr == 1 or _wide(zoom, region):
        return
    L, h = _lib(st)
    N.check(L.gb_compress_xedges(h, _views(st, region), xr, js, je, ls, le, int(tracers), 0), "compress_xedges")


def uncompress_xedges(zoom, st, region, js, je, ls, le, tracers=True):
    xr = zoom.ref(region, "x")
    if xr == 1 or _wide(zoom, region):
        return
    L, h = _lib(st)
    N.check(L.gb_compress_xedges(h, _views(st, region), xr, js, je, ls, le, int(tracers), 1), "uncompress_xedges")


def compress_yedges(zoom, st, region, is_, ie, ls, le, tracers=True):
    yr = zoom.ref(region, "y")
    if yr == 1 or region == 1:
        return
    L, h = _lib(st)
    N.check(L.gb_compress_yedges(h, _views(st, region), yr, is_, ie, ls, le, int(tracers), 0), "compress_yedges")


def uncompress_yedges(zoom, st, region, is_, ie, ls, le, tracers=True):
    yr = zoom.ref(region, "y")
    if yr == 1 or region == 1:
        return
    L, h = _lib(st)
    N.check(L.gb_compress_yedges(h, _views(st, region), yr, is_, ie, ls, le, int(tracers), 1), "uncompress_yedges")


def mix_edges(zoom, st, region, tracers=True):
    g = zoom.g(region)
    xr, yr, zr = (zoom.ref(region, a) for a in "xyz")
    if zr != 1:
        raise ValueError("mix_edges: zooming in z direction not supported!")
    xedges = not (xr == 1 or _wide(zoom, region))
    if not xedges and region == 1:
        return
    ysp, ynp = g.touch_sp != 1, g.touch_np != 1
    L, h = _lib(st)
    N.check(L.gb_mix_edges(h, _views(st, region), xr, yr, int(xedges), int(ysp), int(ynp), int(tracers)), "mix_edges")


def update_parent(zoom, st, region, tracers=True):
    if region == 1:
        return
    xr, yr, zr = (zoom.ref(region, a) for a in "xyz")
    if zr != 1:
        raise ValueError("update_parent: zooming in z direction not supported")
    L, h = _lib(st)
    parent = zoom.g(region).parent
    N.check(L.gb_update_parent(h, _views(st, parent), _views(st, region), zoom.ibeg[region], zoom.jbeg[region], xr, yr,
                               int(tracers)), "update_parent")  # fmt: skip


def coarsen_block(zoom, st, region):
    parent = zoom.g(region).parent
    xr, yr, zr, tr = (zoom.ref(region, a) for a in "xyzt")
    if zr != 1:
        raise ValueError("coarsen_region: zooming in z direction not supported")
    L, h = _lib(st)
    N.check(L.gb_coarsen_block(h, _views(st, parent), _views(st, region), zoom.ibeg[region], zoom.jbeg[region],
                               zoom.lbeg[region], xr, yr, float(tr)), "coarsen_block")  # fmt: skip


def coarsen_ambm(zoom, st, region):
    L, h = _lib(st)
    for child in zoom.children[region]:
        gc = zoom.g(child)
        xr, yr, zr = (zoom.ref(child, a) for a in "xyz")
        N.check(L.gb_coarsen_ambm(h, _views(st, region), _views(st, child), zoom.ibeg[child], zoom.iend[child],
                                  zoom.jbeg[child], zoom.jend[child], zoom.lbeg[child], zoom.lend[child], xr, yr, zr,
                                  int(not _wide(zoom, child)), int(gc.touch_sp != 1), int(gc.touch_np != 1)),
                "coarsen_ambm")  # fmt: skip


_ = ctypes
