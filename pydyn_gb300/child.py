"""A child region's x and y advection and their mass-only Check_CFL forms on the device: the
edges compressed onto one cell, then the held-end row / column kernels on the region's scope.
Reference: pydyn zoom/advect.py:278-412 (_dynamu_child, _rows_child, _substeps_child,
_dynamv_child) and zoom/check_cfl.py:113-193 (_dynamum_child, _dynamvm_child)."""

import ctypes

import numpy as np

from . import _native as N
from . import exchange as X
from .device import views
from .state import TRACERS


class _HostBox:
    """The inclusive (i0, i1, j0, j1) face box a child's columns own: a host int32[4]."""

    def __init__(self, box):
        self.arr = (ctypes.c_int32 * 4)(*box)

    @property
    def ptr(self):
        return ctypes.addressof(self.arr)


def _own_box(st, key, box):
    k = ("own", key)
    if k not in st.consts:
        st.consts[k] = (_HostBox(box),)
    return st.consts[k][0]


def dynamu(zoom, st, region, js, je, ls, le, limits, max_nloop):
    """compress_xedges, then every (j, l) row of cells is-1 .. ie+1 (is = xr, ie = im-xr+1),
    faces is-1 .. ie, the end cells held."""
    X.compress_xedges(zoom, st, region, js, je, ls, le)
    g, f = zoom.g(region), st[region]
    xr = zoom.ref(region, "x")
    is_, ie = xr, g.im - xr + 1
    cells = (slice(is_ - 1, ie + 1), slice(js, je), slice(ls, le))
    q = [f[name][cells] for name in TRACERS]
    L, h = st.dev.L, st.dev.h
    N.check(L.gb_advect_x_held(h, *views(f["m"][cells], *q, f["am"][is_ - 1 : ie, js:je, ls:le]), int(limits),
                               max_nloop), "advect_x_held")  # fmt: skip


def dynamv(zoom, st, region, is_, ie, ls, le, limits, max_nloop):
    """compress_yedges, then per layer the columns is..ie of cells js-1 .. je+1 (js = yr,
    je = jm-yr+1), faces js .. je+1; one nloop per layer, the whole halo'd layer rescaled."""
    X.compress_yedges(zoom, st, region, is_, ie, ls, le)
    g, f = zoom.g(region), st[region]
    yr = zoom.ref(region, "y")
    js, je = yr, g.jm - yr + 1
    cells = (slice(is_, ie), slice(js - 1, je + 1), slice(ls, le))
    q = [f[name][cells] for name in TRACERS]
    own = _own_box(st, (region, is_, ie), (is_, ie, js, je + 1))  # data index = Fortran index (lower bound 0)
    L, h = st.dev.L, st.dev.h
    N.check(L.gb_advect_y_held(h, *views(f["m"][cells], *q, f["bm"][is_:ie, js : je + 1, ls:le], f["bm"]), ls,
                               own.ptr, int(limits), max_nloop), "advect_y_held")  # fmt: skip


def dynamum(zoom, st, region, js, je, ls, le, max_nloop):
    """compressm_xedges, the mass-only held rows, uncompressm_xedges and mixm_edges."""
    X.compress_xedges(zoom, st, region, js, je, ls, le, tracers=False)
    g, f = zoom.g(region), st[region]
    xr = zoom.ref(region, "x")
    is_, ie = xr, g.im - xr + 1
    L, h = st.dev.L, st.dev.h
    N.check(L.gb_cfl_x_held(h, *views(f["m"][is_ - 1 : ie + 1, js:je, ls:le], f["am"][is_ - 1 : ie, js:je, ls:le]),
                            max_nloop), "cfl_x_held")  # fmt: skip
    X.uncompress_xedges(zoom, st, region, js, je, ls, le, tracers=False)
    X.mix_edges(zoom, st, region, tracers=False)


def dynamvm(zoom, st, region, is_, ie, ls, le, max_nloop):
    """compressm_yedges, the mass-only held columns (the scope's faces rescaled, the whole layer
    restored times nloop), uncompressm_yedges and mixm_edges."""
    X.compress_yedges(zoom, st, region, is_, ie, ls, le, tracers=False)
    g, f = zoom.g(region), st[region]
    yr = zoom.ref(region, "y")
    js, je = yr, g.jm - yr + 1
    own = _own_box(st, (region, is_, ie), (is_, ie, js, je + 1))
    L, h = st.dev.L, st.dev.h
    N.check(L.gb_cfl_y_held(h, *views(f["m"][is_:ie, js - 1 : je + 1, ls:le], f["bm"][is_:ie, js : je + 1, ls:le],
                                      f["bm"]), ls, own.ptr, max_nloop), "cfl_y_held")  # fmt: skip
    X.uncompress_yedges(zoom, st, region, is_, ie, ls, le, tracers=False)
    X.mix_edges(zoom, st, region, tracers=False)


_ = ctypes
