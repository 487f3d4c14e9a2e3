"""pydyn.kernels / pydyn.cfl on device arrays: the same calls and in-place semantics, the work
done by the sm_103a kernels of libgbdyn.  Each function takes the DevArray views the reference
function takes (any strides) and leaves them as the reference leaves them.  Nothing comes back
to the host but what the caller asks for; errors found on the device (a sub-cycle cap, non-zero
boundary faces) are raised at the next `Device.sync()`, or at once with `sync=True`.

Sub-cycle caps are the reference's defaults: x 50, y 10, z 15 (kernels.py:129,223,295) and
Check_CFL's 10, 1, 1 (cfl.py:136)."""

import ctypes

import numpy as np

from . import _native as N
from .device import DevArray, views

MAX_NLOOP_X, MAX_NLOOP_Y, ITER_LIMIT_Z = 50, 10, 15
CFL_MAX_NLOOP_X, CFL_MAX_NLOOP_Y, CFL_MAX_NLOOP_Z = 10, 1, 1

__all__ = [
    "advect_x",
    "advect_y",
    "advect_z",
    "cfl_x",
    "cfl_y",
    "cfl_z",
    "fluxes_from_meteo",
    "m2phlb",
]


def _lib(a):
    return a.dev.L, a.dev.h


def _tracer_strides(*qs):
    st = {q.strides for q in qs}
    if len(st) != 1:
        raise ValueError("pydyn_gb300: rm, rxm, rym, rzm views must share their strides")


def _done(dev, rc, what, sync):
    N.check(rc, what)
    if sync:
        dev.sync()


def advect_x(m, rm, rxm, rym, rzm, am, clust=None, halo=False, js=1, je=None, limits=True,
             max_nloop=MAX_NLOOP_X, nloop=None, amax=None, sync=False):
    """dynamu on every (j, l) row (kernels.advect_x :129; with `clust` the reduced grid of
    redgrid.advect_x_reduced :93; with `halo` the periodic halos of zoom _dynamu_region1 :237).
    clust: DevArray (jm,) int32 of cluster sizes or None.  nloop/amax: optional DevArray
    outputs (jm*lm,) of each row's sub-cycle count and largest Courant number."""
    _tracer_strides(rm, rxm, rym, rzm)
    L, h = _lib(m)
    je = m.shape[1] if je is None else je
    rc = L.gb_advect_x(h, *views(m, rm, rxm, rym, rzm, am), None if clust is None else clust.ptr, int(halo), js, je,
                       int(limits), max_nloop, None if nloop is None else nloop.ptr,
                       None if amax is None else amax.ptr)  # fmt: skip
    _done(m.dev, rc, "advect_x", sync)


def advect_y(m, rm, rxm, rym, rzm, bm, bm_full=None, bm_full_l0=0, limits=True, max_nloop=MAX_NLOOP_Y,
             nloop=None, sync=False):
    """dynamv (kernels.advect_y :223), the layers' nloop on the device; bm_full: region 1's
    halo'd bm whose outside faces are rescaled with each layer (zoom _rescale_layer_halo :212)."""
    _tracer_strides(rm, rxm, rym, rzm)
    L, h = _lib(m)
    rc = L.gb_advect_y(h, *views(m, rm, rxm, rym, rzm, bm, bm_full), bm_full_l0, int(limits), max_nloop,
                       None if nloop is None else nloop.ptr)  # fmt: skip
    _done(m.dev, rc, "advect_y", sync)


def advect_z(m, rm, rxm, rym, rzm, cm, scope=None, limits=True, iter_limit=ITER_LIMIT_Z, sync=False):
    """dynamw (kernels.advect_z :295); scope (si0, si1, sj0, sj1), 0-based half-open: the columns
    the trial mass and the sub-steps act on, the search looking at every column (zoom
    _dynamw_child :444)."""
    _tracer_strides(rm, rxm, rym, rzm)
    L, h = _lib(m)
    im, jm = m.shape[0], m.shape[1]
    si0, si1, sj0, sj1 = (0, im, 0, jm) if scope is None else scope
    rc = L.gb_advect_z_scope(h, *views(m, rm, rxm, rym, rzm, cm), si0, si1, sj0, sj1, int(limits), iter_limit)
    _done(m.dev, rc, "advect_z", sync)


def cfl_x(m, am, clust=None, halo=False, js=1, je=None, max_nloop=CFL_MAX_NLOOP_X):
    """cfl.dynamum (:140) with the region-1 halos of zoom/check_cfl.py:94-110; a failure sets
    the device's Check_CFL flag (Device.cfl_failed)."""
    L, h = _lib(m)
    je = m.shape[1] if je is None else je
    N.check(L.gb_cfl_x(h, *views(m, am), None if clust is None else clust.ptr, int(halo), js, je, max_nloop),
            "cfl_x")


def cfl_y(m, bm, max_nloop=CFL_MAX_NLOOP_Y):
    """cfl.dynamvm (:170)."""
    L, h = _lib(m)
    N.check(L.gb_cfl_y(h, *views(m, bm), max_nloop), "cfl_y")


def cfl_z(m, cm, scope=None, iter_limit=CFL_MAX_NLOOP_Z):
    """cfl.dynamwm / zoom _dynamwm (cfl.py:186, zoom/check_cfl.py:206)."""
    L, h = _lib(m)
    im, jm = m.shape[0], m.shape[1]
    si0, si1, sj0, sj1 = (0, im, 0, jm) if scope is None else scope
    N.check(L.gb_cfl_z(h, *views(m, cm), si0, si1, sj0, sj1, iter_limit), "cfl_z")


def fluxes_from_meteo(pu, pv, bt, dt, am, bm, cm):
    """kernels.fluxes_from_meteo (:102) into am, bm, cm (DevArray views); bt a DevArray (lm+1)."""
    L, h = _lib(pu)
    N.check(L.gb_fluxes_from_meteo(h, *views(pu, pv), bt.ptr, float(dt), *views(am, bm, cm)), "fluxes_from_meteo")


def m2phlb(m, sp, phlb, dxyp, at, bt, ring=None):
    """zoom m2phlb1 (massflow.py:24) -- ring = (xr, yr, jbeg, dxyp_parent) for m2phlb (:35).
    m (im, jm, lm), sp (im, jm), phlb (im, jm, lm+1); dxyp, at, bt, dxyp_parent DevArrays."""
    L, h = _lib(m)
    xr, yr, jbeg, par = (0, 0, 0, None) if ring is None else ring
    N.check(L.gb_m2phlb(h, *views(m, sp, phlb), dxyp.ptr, at.ptr, bt.ptr, xr, yr, jbeg,
                        None if par is None else par.ptr), "m2phlb")  # fmt: skip


def convec(m, rm, rxm, rym, rzm, entu, detu, entd, detd, dkg, cloud_top, cloud_lfs, cols, dt, lmax, cache=None):
    """kernels.convec (:423) on the listed owned columns: cols a DevArray (ncol, 2) int32 of
    0-based (i, j); cloud_top / cloud_lfs DevArrays (im, jm) int32; cache: None or
    (inv, m, tag, epoch) DevArrays keeping each column's inverse for the paired call."""
    _tracer_strides(rm, rxm, rym, rzm)
    if cloud_top.strides != cloud_lfs.strides:
        raise ValueError("convec: cloud_top and cloud_lfs must share their strides")
    L, h = _lib(m)
    ncol = cols.shape[0]
    c = (None, None, None, None) if cache is None else tuple(x.ptr for x in cache)
    N.check(L.gb_convec(h, *views(m, rm, rxm, rym, rzm, entu, detu, entd, detd, dkg), cloud_top.ptr, cloud_lfs.ptr,
                        cloud_top.strides[0], cloud_top.strides[1], cols.ptr, ncol, float(dt), int(lmax), *c),
            "convec")  # fmt: skip


KZZ_SURFACE = ("oro", "lsm", "sr", "srols", "u10m", "v10m", "sshf", "slhf", "ewss", "nsss")


def calc_kzz(spm, sp, pu, pv, t, q, surface, at, bt, dxyp, lmax_conv, dx, dy, ybeg, dkg, pblh=None):
    """diffusion.calc_kzz (diffusion.py:266-276) into dkg (im, jm, lmax_conv) and, if given,
    pblh (im, jm).  surface: the 10 (im, jm) DevArrays in KZZ_SURFACE order (or a mapping of
    those names); at, bt (lm+1) and dxyp (jm) contiguous DevArrays."""
    if isinstance(surface, dict):
        surface = [surface[k] for k in KZZ_SURFACE]
    if len(surface) != len(KZZ_SURFACE):
        raise ValueError(f"calc_kzz: {len(KZZ_SURFACE)} surface fields, got {len(surface)}")
    L, h = _lib(t)
    surf = (N.GBView * len(KZZ_SURFACE))(*(s.view() for s in surface))
    N.check(L.gb_calc_kzz(h, *views(spm, sp, pu, pv, t, q), surf, at.ptr, bt.ptr, dxyp.ptr, int(lmax_conv),
                          float(dx), float(dy), float(ybeg), *views(dkg, pblh)),
            "calc_kzz")  # fmt: skip


CHEM_FIELDS = ("strat_press", "strat_oh", "strat_cl", "strat_od", "oh_3d", "pl_trop", "cl_trop", "soil")


def _chem_args(temper, phlb, lat, fields, oh_factor, oh_scale, cl_scale, o1d_scale, soil_rate, dt):
    f = {k: fields.get(k) for k in CHEM_FIELDS}
    return (*views(temper, phlb), lat.ptr, *views(*(f[k] for k in CHEM_FIELDS)),
            None if oh_factor is None else oh_factor.ptr, float(oh_scale), float(cl_scale), float(o1d_scale),
            float(soil_rate), float(dt))  # fmt: skip


def loss_rates(temper, phlb, lat, fields, dt, loss=None, decay=None, oh_factor=None, oh_scale=1.0, cl_scale=1.0,
               o1d_scale=1.0, soil_rate=0.0):
    """chem.loss_rates and chem.decay (chem.py:114-170) of every column into loss (im, jm, lm, 4)
    and decay (im, jm, lm).  fields: DevArrays by CHEM_FIELDS name (pl_trop / cl_trop and soil
    optional, as the sinks are on); lat (jm) radians; oh_factor (im) multiplies oh_3d."""
    L, h = _lib(temper)
    N.check(L.gb_loss_rates(h, *_chem_args(temper, phlb, lat, fields, oh_factor, oh_scale, cl_scale, o1d_scale,
                                           soil_rate, dt), *views(loss, decay)), "loss_rates")  # fmt: skip


def chemistry(temper, phlb, lat, fields, dt, cols, tracers, rm, rxm, rym, rzm, oh_factor=None, oh_scale=1.0,
              cl_scale=1.0, o1d_scale=1.0, soil_rate=0.0, krates=None, cache=None):
    """chemistry_region (zoom/physics.py:67): the decay of each listed column's cells applied to
    the mass and slopes of the (1-based) `tracers`.  krates: chem_krates(temper)'s, or None.
    cache: None or (array of 8 doubles per listed cell, step counter int32 DevArray): the
    rates a later call on the same pressures in the same step takes again."""
    _tracer_strides(rm, rxm, rym, rzm)
    mask = 0
    for t in tracers:
        mask |= 1 << (int(t) - 1)
    L, h = _lib(temper)
    N.check(L.gb_chemistry(h, *_chem_args(temper, phlb, lat, fields, oh_factor, oh_scale, cl_scale, o1d_scale,
                                          soil_rate, dt), cols.ptr, cols.shape[0], mask,
                           *views(rm, rxm, rym, rzm, krates), None if cache is None else cache[0].ptr,
                           None if cache is None else cache[1].ptr), "chemistry")  # fmt: skip


def chem_krates(temper, krates, cols=None):
    """The rate constants of the temperature (chem.py:137-140) into krates (im, jm, lm, 2) on the
    listed columns (cols a DevArray (ncol, 2) int32, or None: every column)."""
    L, h = _lib(temper)
    N.check(L.gb_chem_krates(h, *views(temper), None if cols is None else cols.ptr,
                             0 if cols is None else cols.shape[0], *views(krates)), "chem_krates")  # fmt: skip


def sources(rm, rzm, flux, cols, level, tracer, area=None, scale=1.0):
    """sources_region (zoom/physics.py:55): rm(level) += x, rzm(level) -= x on the listed columns,
    x = (flux area) scale, or flux itself without area."""
    _tracer_strides(rm, rzm)
    L, h = _lib(rm)
    N.check(L.gb_sources(h, *views(rm, rzm, flux), None if area is None else area.ptr, float(scale), int(level),
                         int(tracer), cols.ptr, cols.shape[0]), "sources")  # fmt: skip


# ------------------------------------------------------------------ the adjoint (one tracer)
def advect_z_last(m, n_out):
    """The n_advz of the context's last dynamw into n_out (a DevArray (1,) int32)."""
    L, h = _lib(m)
    N.check(L.gb_advect_z_last(h, n_out.ptr), "advect_z_last")


def adjoint_x(m, rm_b, rxm_b, rym_b, rzm_b, am, clust=None, max_nloop=MAX_NLOOP_X):
    """The transpose of advect_x (unlimited slopes) on the tracer adjoints, in place: m and am as
    the forward call got them."""
    _tracer_strides(rm_b, rxm_b, rym_b, rzm_b)
    L, h = _lib(m)
    N.check(L.gb_adjoint_x(h, *views(m, rm_b, rxm_b, rym_b, rzm_b, am), None if clust is None else clust.ptr,
                           max_nloop), "adjoint_x")  # fmt: skip


def adjoint_y(m, rm_b, rxm_b, rym_b, rzm_b, bm, nloop):
    """The transpose of advect_y (unlimited slopes): m and bm (im, jm+1, lm) as the forward call
    got them, nloop the per-level counts it returned."""
    _tracer_strides(rm_b, rxm_b, rym_b, rzm_b)
    L, h = _lib(m)
    N.check(L.gb_adjoint_y(h, *views(m, rm_b, rxm_b, rym_b, rzm_b, bm), nloop.ptr), "adjoint_y")


def adjoint_z(m, rm_b, rxm_b, rym_b, rzm_b, cm, n_advz):
    """The transpose of advect_z (unlimited slopes): m and cm as the forward call got them."""
    _tracer_strides(rm_b, rxm_b, rym_b, rzm_b)
    L, h = _lib(m)
    N.check(L.gb_adjoint_z(h, *views(m, rm_b, rxm_b, rym_b, rzm_b, cm), n_advz.ptr), "adjoint_z")


def adjoint_convec(rm_b, rxm_b, rym_b, rzm_b, inv, cols, lmax):
    """The transpose of convec on the listed columns with the inverses it applied."""
    _tracer_strides(rm_b, rxm_b, rym_b, rzm_b)
    L, h = _lib(rm_b)
    N.check(L.gb_adjoint_convec(h, *views(rm_b, rxm_b, rym_b, rzm_b), inv.ptr, cols.ptr, cols.shape[0], int(lmax)),
            "adjoint_convec")  # fmt: skip


def adjoint_sources(rm_b, rzm_b, grad, cols, level, area, scale):
    """grad (im, jm) += area scale (rm_b - rzm_b)(level) on the listed columns: the flux gradient
    of one sources call."""
    L, h = _lib(rm_b)
    N.check(L.gb_adjoint_sources(h, *views(rm_b, rzm_b, grad), area.ptr, float(scale), int(level), cols.ptr,
                                 cols.shape[0]), "adjoint_sources")  # fmt: skip


def to_device(dev, arr, dtype=np.float64):
    """A DevArray copy of a host array (0-based bounds)."""
    return DevArray.from_host(dev, np.asarray(arr, dtype=dtype))


_ = ctypes
