"""Meteo_Setup_Mass's balancing on the device (pydyn balance.py:183-219, zoom_meteo.py:135-209):
the horizontal mass fluxes of a meteo instant made consistent with its surface-pressure
tendency, level by level, in up to three Richardson tries.

    setup_mass(pu, pv, pw, sp1, sp2, levi_db, area, dt)        region 1 (a periodic globe)
    setup_mass_child(raw, parent, sp1, sp2, levi_db, area, dt, rf, poisson)   a child

Arrays are device arrays (pydyn_gb300.device.DevArray) in pydyn's layout without halos: pu
(im+1, jm, lm), pv (im, jm+1, lm), pw (im, jm, lm+1), sp1/sp2 (im, jm), levi_db (lm), area (jm).
The host takes only the decisions pydyn takes (the checks' verdicts: two numbers read back per
check).  The Poisson solve is the device's own discrete Fourier transform in float64, so the
balanced fluxes equal pydyn's to rounding, not bitwise (pydyn's own FFTW and NumPy paths differ
from each other the same way); the mass change, the checks, the Match and the direct products
are pydyn's element statements in its order."""

import ctypes
from typing import NamedTuple

import numpy as np

from . import _native as N
from .device import DevArray

MB_MAX_TRIES = 3
MB_TOL_PRE = (1.0e-4, 1.0e-3)  # meteo.F90 Meteo_Setup_Mass: (rms, max) of the pre-check
MB_TOL_TIGHT = (1.0e-7, 1.0e-6)  # ... and of the Richardson loop
PI = 3.14159265358979  # the eigenvalues' PI (a default-real literal in the Fortran)
MATCH_U, MATCH_V, MATCH_CELL = 0, 1, 2


def _view(a):
    return ctypes.byref(a.view())


class PoissonSolver:
    """The periodic Poisson solve of an (im, jm) grid on a device: its twiddle tables
    (cos, sin of 2 pi t / N) and the 5-point Laplacian's eigenvalues (pydyn balance.py:97-104)."""

    def __init__(self, dev, im, jm):
        self.dev, self.im, self.jm = dev, im, jm
        tw = [np.concatenate([np.cos(2.0 * np.pi * np.arange(n) / n), np.sin(2.0 * np.pi * np.arange(n) / n)])
              for n in (im, jm)]  # fmt: skip
        i, j = np.arange(im)[:, None], np.arange(jm)[None, :]
        fac = 2.0 * (np.cos(2 * PI * i / im) + np.cos(2 * PI * j / jm) - 2.0)
        fac[0, 0] = 1.0
        self.tw_i, self.tw_j = (DevArray.from_host(dev, t) for t in tw)
        self.fac = DevArray.from_host(dev, np.ascontiguousarray(fac))

    def balance(self, pu, pv, pw, dm_dt):
        """One BalanceMassFluxes_m: every level's residual divergence corrected (in place)."""
        N.check(self.dev.L.gb_balance_fft(self.dev.h, _view(pu), _view(pv), _view(pw), _view(dm_dt), self.tw_i.ptr,
                                          self.tw_j.ptr, self.fac.ptr), "gb_balance_fft")  # fmt: skip

    def free(self):
        for a in (self.tw_i, self.tw_j, self.fac):
            a.free()


def fill_mass_change(dev, sp1, sp2, levi_db, area, dt_sec, out=None):
    """FillMassChange / dt (pydyn balance.py:76-82): kg/s per cell and level, a device array."""
    im, jm, lm = sp1.shape[0], sp1.shape[1], levi_db.shape[0]
    out = DevArray.zeros(dev, (0, im - 1), (0, jm - 1), (0, lm - 1)) if out is None else out
    N.check(dev.L.gb_fill_mass_change(dev.h, _view(out), _view(sp1), _view(sp2), levi_db.ptr, area.ptr,
                                      float(dt_sec)), "gb_fill_mass_change")  # fmt: skip
    return out


def check_mass_balance(dev, pu, pv, sp1, sp2, dt_sec, area, rms_max, mav_max, out=None):
    """CheckMassBalance (pydyn balance.py:85-94): (ok, rms, max) of the relative mismatch of the
    column convergence and the surface-pressure tendency (two numbers read back)."""
    buf = DevArray.zeros(dev, (0, 1)) if out is None else out
    N.check(dev.L.gb_mass_check(dev.h, _view(pu), _view(pv), _view(sp1), _view(sp2), area.ptr, float(dt_sec),
                                buf.ptr), "gb_mass_check")  # fmt: skip
    rms, mav = (float(x) for x in buf.host())
    if out is None:
        buf.free()
    return not (rms > rms_max or mav > mav_max), rms, mav


def setup_mass(pu, pv, pw, sp1, sp2, levi_db, area, dt_sec, max_tries=MB_MAX_TRIES, solver=None):
    """The balancing part of Meteo_Setup_Mass for region 1 and one meteo instant (pydyn
    balance.py:202-219): pu, pv balanced in place; returns dict(tries, ok, pre, post, solver).
    Raises ValueError when the input fails the pre-check, as pydyn does."""
    dev = pu.dev
    own = solver is None
    solver = PoissonSolver(dev, sp1.shape[0], sp1.shape[1]) if own else solver
    dm_dt = fill_mass_change(dev, sp1, sp2, levi_db, area, dt_sec)
    buf = DevArray.zeros(dev, (0, 1))
    try:
        ok0, rms0, mav0 = check_mass_balance(dev, pu, pv, sp1, sp2, dt_sec, area, *MB_TOL_PRE, out=buf)
        if not ok0:
            raise ValueError(f"setup_mass: unbalanced input fluxes (rms {rms0:.3e}, max {mav0:.3e})")
        for tries in range(1, max_tries + 1):  # noqa: B007
            solver.balance(pu, pv, pw, dm_dt)
            ok, rms, mav = check_mass_balance(dev, pu, pv, sp1, sp2, dt_sec, area, *MB_TOL_TIGHT, out=buf)
            if ok:
                break
    finally:
        dm_dt.free()
        buf.free()
        if own:
            solver.free()
    return {"tries": tries, "ok": ok, "pre": (rms0, mav0), "post": (rms, mav), "solver": "dft"}


# ------------------------------------------------------------------ a child
class Refinement(NamedTuple):
    """A child's cells per parent cell and the parent cells it covers (1-based, inclusive),
    as GetRefinement answers (pydyn zoom_meteo.py:58-84)."""

    ri: int
    rj: int
    ci1: int
    ci2: int
    cj1: int
    cj2: int

    @classmethod
    def of(cls, zoom, r):
        return cls(zoom.ref(r, "x"), zoom.ref(r, "y"), zoom.ibeg[r], zoom.iend[r], zoom.jbeg[r], zoom.jend[r])


class PoissonDirect:
    """EnsurePoissonCache's direct matrices of an (ri, rj) cell block (pydyn zoom_meteo.py:135-
    161): column k is the correction (u, v) of the unit divergence at cell k (column-major),
    made by the device's periodic solve -- all n unit divergences at once, as n levels."""

    def __init__(self, dev, ri, rj, matrices=None):
        """matrices: (m_to_u, m_to_v) to take as they are instead of making them."""
        n = ri * rj
        if n > 64:
            raise ValueError(f"PoissonDirect: {ri} x {rj} cells; the device's direct solve takes at most 64")
        self.dev, self.ri, self.rj = dev, ri, rj
        if matrices is not None:
            self.load(*matrices)
            return
        solver = PoissonSolver(dev, ri, rj)
        pu = DevArray.zeros(dev, (0, ri), (0, rj - 1), (0, n - 1))
        pv = DevArray.zeros(dev, (0, ri - 1), (0, rj), (0, n - 1))
        pw = DevArray.zeros(dev, (0, ri - 1), (0, rj - 1), (0, n))
        unit = np.zeros((ri, rj, n))
        for k in range(n):
            unit[k % ri, k // ri, k] = -1.0  # the residual is -dm_dt: a unit divergence at cell k
        dm = DevArray.from_host(dev, unit)
        solver.balance(pu, pv, pw, dm)
        u, v = pu.host(), pv.host()  # (ri+1, rj, n), (ri, rj+1, n)
        for a in (pu, pv, pw, dm):
            a.free()
        solver.free()
        self.m_to_u = np.stack([u[:, :, k].reshape(-1, order="F") for k in range(n)], axis=1)
        self.m_to_v = np.stack([v[:, :, k].reshape(-1, order="F") for k in range(n)], axis=1)
        self.load(self.m_to_u, self.m_to_v)

    def load(self, m_to_u, m_to_v):
        """Put the matrices on the device, each column contiguous (the device reads them so)."""
        self.m_to_u, self.m_to_v = m_to_u, m_to_v
        self._mu = DevArray.from_host(self.dev, np.ascontiguousarray(m_to_u.T))
        self._mv = DevArray.from_host(self.dev, np.ascontiguousarray(m_to_v.T))

    def balance(self, pu, pv, pw, dm_dt, rf):
        """BalanceMassFluxes_m against the parent (pydyn zoom_meteo.py:163-181), in place."""
        N.check(self.dev.L.gb_balance_direct(self.dev.h, _view(pu), _view(pv), _view(pw), _view(dm_dt), self._mu.ptr,
                                             self._mv.ptr, *rf), "gb_balance_direct")  # fmt: skip

    def free(self):
        self._mu.free()
        self._mv.free()


def match(kind, parent, child, rf):
    """Match 'sum' of a child's x faces (MATCH_U), y faces (MATCH_V) or cells (MATCH_CELL) to its
    parent's (pydyn zoom_meteo.py:87-119), in place, every level."""
    dev = child.dev
    N.check(dev.L.gb_match_sum(dev.h, int(kind), _view(parent), _view(child), *rf), "gb_match_sum")


def _copy(a):
    out = DevArray.zeros(a.dev, *((lo, lo + n - 1) for lo, n in zip(a.lower, a.shape, strict=True)))
    out.assign(a)
    return out


def setup_mass_child(raw, parent, sp1, sp2, levi_db, area, dt_sec, rf, poisson, max_tries=MB_MAX_TRIES):
    """The balancing part of Meteo_Setup_Mass for a child and one meteo instant (pydyn
    zoom_meteo.py:184-209): the raw fluxes (pu, pv, pw) copied and matched to the parent's
    balanced ones, checked, balanced in the Richardson loop.  Returns (pu, pv, pw, info)."""
    pu, pv, pw = (_copy(q) for q in raw)
    ppu, ppv, ppw = parent
    match(MATCH_U, ppu, pu, rf)
    match(MATCH_V, ppv, pv, rf)
    match(MATCH_CELL, ppw, pw, rf)
    dev = pu.dev
    dm_dt = fill_mass_change(dev, sp1, sp2, levi_db, area, dt_sec)
    buf = DevArray.zeros(dev, (0, 1))
    try:
        ok0, rms0, mav0 = check_mass_balance(dev, pu, pv, sp1, sp2, dt_sec, area, *MB_TOL_PRE, out=buf)
        if not ok0:
            raise ValueError(f"setup_mass_child: unbalanced matched fluxes (rms {rms0:.3e}, max {mav0:.3e})")
        for tries in range(1, max_tries + 1):  # noqa: B007
            poisson.balance(pu, pv, pw, dm_dt, rf)
            ok, rms, mav = check_mass_balance(dev, pu, pv, sp1, sp2, dt_sec, area, *MB_TOL_TIGHT, out=buf)
            if ok:
                break
    finally:
        dm_dt.free()
        buf.free()
    return pu, pv, pw, {"tries": tries, "ok": ok, "pre": (rms0, mav0), "post": (rms, mav)}
