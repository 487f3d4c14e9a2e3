"""ORACLE -- test infrastructure.  ctypes bindings of oracle/src/*.c on NumPy arrays, with the
call shapes of pydyn.kernels / pydyn.cfl (each wrapper names the reference function it restates).
Arrays must be float64 (int32 where noted); any strides; modified in place like the reference."""

import ctypes

import numpy as np

from .build import build


class OV(ctypes.Structure):
    _fields_ = [("p", ctypes.c_void_p), ("n", ctypes.c_int64 * 4), ("s", ctypes.c_int64 * 4)]


def ov(a):
    """A strided view descriptor of a NumPy float64 array (rank <= 4)."""
    if a is None:
        return None
    if a.dtype != np.float64:
        raise TypeError("oracle: float64 arrays only")
    v = OV()
    v.p = a.ctypes.data
    for k in range(4):
        v.n[k] = a.shape[k] if k < a.ndim else 1
        v.s[k] = a.strides[k] // 8 if k < a.ndim else 0
    return v


_LIB = []


def lib():
    if not _LIB:
        L = ctypes.CDLL(str(build()))
        P = ctypes.POINTER(OV)
        I = ctypes.c_int
        i32 = ctypes.c_void_p
        L.or_advect_x.argtypes = [P, P, P, P, P, P, i32, I, I, I, I, I, I, i32, ctypes.c_void_p]
        L.or_advect_y.argtypes = [P, P, P, P, P, P, P, I, I, I, I, i32]
        L.or_advect_z.argtypes = [P, P, P, P, P, P, I, I, I, I, I, I, I, i32]
        L.or_fluxes_from_meteo.argtypes = [P, P, ctypes.c_void_p, ctypes.c_double, P, P, P]
        L.or_advect_x_held.argtypes = [P, P, P, P, P, P, I, I, I]
        D, VP = ctypes.c_double, ctypes.c_void_p
        L.or_calc_kzz.argtypes = [P, P, P, P, P, P, P, VP, VP, VP, I, D, D, D, P, P]
        L.or_loss_rates.argtypes = [P, P, VP, P, P, P, P, P, P, P, P, VP, D, D, D, D, D, P, P]
        L.or_convec.argtypes = [P, P, P, P, P, P, P, P, P, P, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                ctypes.c_int64, ctypes.c_void_p, I, ctypes.c_double, I]
        L.or_advect_y_held.argtypes = [P, P, P, P, P, P, P, I, I, I, I]
        L.or_m2phlb.argtypes = [P, P, P, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, I, I, I, ctypes.c_void_p]
        _LIB.append(L)
    return _LIB[0]


def _ref(v):
    return ctypes.byref(v) if v is not None else None


def _ptr(a):
    return None if a is None else a.ctypes.data


class CFLError(RuntimeError):
    """The oracle's pydyn.kernels.CFLError (kernels.py:60)."""


def advect_x(m, rm, rxm, rym, rzm, am, clust=None, halo=False, js=1, je=None, limits=True, max_nloop=50,
             mass_only=False):
    """kernels.advect_x / redgrid.advect_x_reduced / zoom _dynamu_region1 / cfl.dynamum
    (kernels.py:129, redgrid.py:93, zoom/advect.py:237, cfl.py:140).  Returns
    (nloop (jm, lm), alpha_max (jm, lm)); raises CFLError (tracers) or returns None (mass_only)
    when a row exceeds its cap."""
    jm, lm = m.shape[1], m.shape[2]
    je = jm if je is None else je
    cl = None if clust is None else np.ascontiguousarray(clust, dtype=np.int32)
    nloop = np.zeros((jm, lm), dtype=np.int32)
    amax = np.zeros((jm, lm))
    views = [ov(q) for q in (m, rm if rm is not None else m, rxm if rxm is not None else m,
                             rym if rym is not None else m, rzm if rzm is not None else m, am)]  # fmt: skip
    rc = lib().or_advect_x(*map(_ref, views), _ptr(cl), int(halo), js, je, int(limits), max_nloop,
                           int(mass_only), nloop.ctypes.data, amax.ctypes.data)  # fmt: skip
    if rc:
        if mass_only:
            return None
        raise CFLError("dynamu: nloop too high")
    return nloop, amax


def advect_y(m, rm, rxm, rym, rzm, bm, full=None, full_l0=0, limits=True, max_nloop=10, mass_only=False):
    """kernels.advect_y (+ zoom _rescale_layer_halo on `full`) / cfl.dynamvm (kernels.py:223,
    zoom/advect.py:201-226, cfl.py:170).  Returns the layers' nloop."""
    lm = m.shape[2]
    nloop = np.zeros(lm, dtype=np.int32)
    q = [x if x is not None else m for x in (rm, rxm, rym, rzm)]
    rc = lib().or_advect_y(*map(_ref, [ov(m), *map(ov, q), ov(bm), ov(full)]), full_l0, int(limits), max_nloop,
                           int(mass_only), nloop.ctypes.data)  # fmt: skip
    if rc == 2:
        raise ValueError("advect_y: non-zero flux through the polar outer faces")
    if rc == 1:
        if mass_only:
            return None
        raise CFLError("dynamv: nloop too high")
    return nloop


def advect_z(m, rm, rxm, rym, rzm, cm, scope=None, limits=True, iter_limit=15, mass_only=False):
    """kernels.advect_z / zoom _dynamw_child / cfl.dynamwm (kernels.py:295, zoom/advect.py:444,
    cfl.py:186): scope = (si0, si1, sj0, sj1) 0-based half-open, default the whole region.
    Returns n_advz."""
    im, jm = m.shape[0], m.shape[1]
    si0, si1, sj0, sj1 = (0, im, 0, jm) if scope is None else scope
    n = np.zeros(1, dtype=np.int32)
    q = [x if x is not None else m for x in (rm, rxm, rym, rzm)]
    rc = lib().or_advect_z(*map(_ref, [ov(m), *map(ov, q), ov(cm)]), si0, si1, sj0, sj1, int(limits), iter_limit,
                           int(mass_only), n.ctypes.data)  # fmt: skip
    if rc == 2:
        raise ValueError("dynamw: non-zero halo interfaces in cm")
    if rc == 1:
        if mass_only:
            return None
        raise CFLError("dynamw: too many CFL violations!")
    return int(n[0])


def advect_x_held(m, rm, rxm, rym, rzm, am, limits=True, max_nloop=50, mass_only=False):
    """A child's held-end rows (zoom/advect.py:278-345; check_cfl.py:113-137 with mass_only):
    m (n, nj, nl), am (n-1, nj, nl).  False when a row exceeded its cap (mass_only)."""
    q = [x if x is not None else m for x in (rm, rxm, rym, rzm)]
    rc = lib().or_advect_x_held(*map(_ref, [ov(m), *map(ov, q), ov(am)]), int(limits), max_nloop, int(mass_only))
    if rc and not mass_only:
        raise CFLError("dynuamu: nloop too high")
    return not rc


def advect_y_held(m, rm, rxm, rym, rzm, bm, full, full_l0, limits=True, max_nloop=10, mass_only=False):
    """A child's held-end columns (zoom/advect.py:348-412; check_cfl.py:162-193 with mass_only):
    m (ni, n, nl), bm (ni, n-1, nl) the scope's faces, full the whole halo'd bm."""
    q = [x if x is not None else m for x in (rm, rxm, rym, rzm)]
    rc = lib().or_advect_y_held(*map(_ref, [ov(m), *map(ov, q), ov(bm), ov(full)]), full_l0, int(limits), max_nloop,
                                int(mass_only))  # fmt: skip
    if rc and not mass_only:
        raise CFLError("nloop too high in dynamv")
    return not rc


def convec(m, rm, rxm, rym, rzm, entu, detu, entd, detd, cloud_top, cloud_lfs, dkg, dt, lmax, cols=None):
    """kernels.convec (kernels.py:423-457) with the Crout inverse, on the listed (i, j) columns
    (default every column of m (im, jm, lm))."""
    im, jm = m.shape[0], m.shape[1]
    if cols is None:
        cols = np.array([(i, j) for i in range(im) for j in range(jm)], dtype=np.int32)
    cols = np.ascontiguousarray(cols, dtype=np.int32)
    top = np.asarray(cloud_top)
    lfs = np.asarray(cloud_lfs)
    if top.dtype != np.int32 or lfs.dtype != np.int32 or top.strides != lfs.strides:
        top, lfs = np.ascontiguousarray(top, dtype=np.int32), np.ascontiguousarray(lfs, dtype=np.int32)
    lib().or_convec(*map(_ref, map(ov, (m, rm, rxm, rym, rzm, entu, detu, entd, detd, dkg))), top.ctypes.data,
                    lfs.ctypes.data, top.strides[0] // 4, top.strides[1] // 4, cols.ctypes.data, len(cols),
                    float(dt), int(lmax))  # fmt: skip


KZZ_SURFACE = ("oro", "lsm", "sr", "srols", "u10m", "v10m", "sshf", "slhf", "ewss", "nsss")


def calc_kzz(spm, sp, pu, pv, t, q, surface, at, bt, dxyp, lmax_conv, dx=6.0, dy=4.0, ybeg=-90.0):
    """diffusion.calc_kzz (diffusion.py:266-276): (dkg (im, jm, lmax_conv), pblh (im, jm))."""
    im, jm = t.shape[0], t.shape[1]
    dkg = np.zeros((im, jm, lmax_conv))
    pblh = np.zeros((im, jm))
    surf = (OV * 10)(*[ov(np.asarray(surface[k], dtype=np.float64)) for k in KZZ_SURFACE])
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (at, bt, dxyp)]
    lib().or_calc_kzz(*map(_ref, map(ov, (spm, sp, pu, pv, t, q))), surf, *(a.ctypes.data for a in arrs),
                      int(lmax_conv), float(dx), float(dy), float(ybeg), _ref(ov(dkg)), _ref(ov(pblh)))  # fmt: skip
    return dkg, pblh


def loss_rates(temper, phlb, lat, strat_press, strat_oh, strat_cl, strat_od, oh_3d, pl_trop=None, cl_trop=None,
               soil=None, oh_scale=1.0, cl_scale=1.0, o1d_scale=1.0, soil_rate=0.0, dt=None, oh_factor=None):
    """chem.loss_rates (chem.py:114-150) and, with dt, chem.decay (:168-170): (loss (im, jm, lm, 4),
    decay (im, jm, lm) or None).  oh_factor (im): a per-longitude multiplier of oh_3d, or None.
    Raises ValueError for levels that are not strictly descending (chem.py:47-49)."""
    im, jm, lm = temper.shape
    loss = np.zeros((im, jm, lm, 4))
    decay = None if dt is None else np.zeros((im, jm, lm))
    f64 = [None if a is None else np.asarray(a, dtype=np.float64) for a in (lat, oh_factor)]
    lat_c = np.ascontiguousarray(f64[0])
    fac = None if f64[1] is None else np.ascontiguousarray(f64[1])
    arrs = [None if a is None else np.asarray(a, dtype=np.float64)
            for a in (temper, phlb, None, strat_press, strat_oh, strat_cl, strat_od, oh_3d, pl_trop, cl_trop, soil)]
    views = [ov(a) for a in arrs]  # arrs keeps every converted array alive through the call
    rc = lib().or_loss_rates(_ref(views[0]), _ref(views[1]), lat_c.ctypes.data, *map(_ref, views[3:]), _ptr(fac),
                             float(oh_scale), float(cl_scale), float(o1d_scale), float(soil_rate),
                             float(dt if dt is not None else 0.0), _ref(ov(loss)), _ref(ov(decay)))  # fmt: skip
    if rc:
        raise ValueError("rebin: levels not strictly descending")
    return loss, decay


def fluxes_from_meteo(pu, pv, bt, dt, am, bm, cm):
    """kernels.fluxes_from_meteo (kernels.py:102-125) into the given am, bm, cm."""
    bt = np.ascontiguousarray(bt, dtype=np.float64)
    lib().or_fluxes_from_meteo(*map(_ref, (ov(pu), ov(pv))), bt.ctypes.data, float(dt),
                               *map(_ref, (ov(am), ov(bm), ov(cm))))  # fmt: skip


def m2phlb(m, sp, phlb, dxyp, at, bt, xr=0, yr=0, jbeg=0, dxyp_parent=None):
    """zoom/massflow.py:24-56 (m2phlb1; m2phlb's ring with xr > 0) into sp (im, jm), phlb."""
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (dxyp, at, bt)]
    par = None if dxyp_parent is None else np.ascontiguousarray(dxyp_parent, dtype=np.float64)
    lib().or_m2phlb(*map(_ref, (ov(m), ov(sp), ov(phlb))), *(a.ctypes.data for a in arrs), xr, yr, jbeg,
                    _ptr(par))  # fmt: skip
