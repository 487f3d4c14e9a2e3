"""ORACLE -- test infrastructure.  A NumPy restatement of pydyn's Meteo_Setup_Mass balancing
(pydyn balance.py:76-124 and 183-219, zoom_meteo.py:87-181): the mass change of each cell, the
mass-balance check, the doubly periodic Poisson correction of region 1 through NumPy's FFT (as
pydyn's NumpyPoisson), and a child's Match 'sum' and per-parent-cell direct solve.  Arrays are
pydyn's layout without halos: pu (im+1, jm, lm), pv (im, jm+1, lm), pw (im, jm, lm+1)."""

import numpy as np

GRAV = 9.80665
PI = 3.14159265358979
MB_TOL_PRE = (1.0e-4, 1.0e-3)
MB_TOL_TIGHT = (1.0e-7, 1.0e-6)


def seqsum(q, axis=0):
    """The sum along `axis` in index order (pydyn ops.py:235-240)."""
    q = np.moveaxis(q, axis, 0)
    acc = q[0].copy()
    for term in q[1:]:
        acc = acc + term
    return acc


def convergence(pu, pv):
    """pu's and pv's faces into each cell (pydyn ops.py:273-274)."""
    return pu[:-1] - pu[1:] + pv[:, :-1] - pv[:, 1:]


def fill_mass_change(sp1, sp2, levi_db, area, dt):
    """balance.py:76-82."""
    dm = np.abs(levi_db) * (sp2 - sp1)[..., None] / GRAV
    dm = dm * area[None, :, None]
    return dm / dt


def check_mass_balance(pu, pv, sp1, sp2, dt, area, rms_max, mav_max):
    """balance.py:85-94: (ok, rms, max)."""
    d = convergence(seqsum(pu, axis=2), seqsum(pv, axis=2)) * GRAV / area[None, :]
    diff = (d - (sp2 - sp1) / dt) / ((sp1 + sp2) / 2.0)
    rms = np.sqrt(np.sum(diff**2) / diff.size)
    mav = np.max(np.abs(diff))
    return not (rms > rms_max or mav > mav_max), float(rms), float(mav)


def poisson_factor(im, jm):
    """balance.py:97-104: the periodic 5-point Laplacian's eigenvalues, fac(0, 0) = 1."""
    i = np.arange(im)[:, None]
    j = np.arange(jm)[None, :]
    fac = 2.0 * (np.cos(2 * PI * i / im) + np.cos(2 * PI * j / jm) - 2.0)
    fac[0, 0] = 1.0
    return fac


def psi(m, fac):
    """balance.py:113-124: the inverse Laplacian of m through NumPy's FFT."""
    im, jm = m.shape
    X = np.fft.fft2(m)
    X.real[...] = X.real / fac
    X.imag[...] = X.imag / fac
    X[0, 0] = 0.0
    A = np.fft.ifft2(X) * (im * jm)
    return A.real / float(im * jm)


def poisson_correction(m, fac):
    """balance.py:183-189: (u (im+1, jm), v (im, jm+1)) gauged to u(0, :) = v(:, 0) = 0."""
    p = psi(m, fac)
    u = np.diff(p, axis=0, prepend=p[-1:], append=p[:1])
    v = np.diff(p, axis=1, prepend=p[:, -1:], append=p[:, :1])
    return u - u[0], v - v[:, :1]


def balance_mass_fluxes(pu, pv, pw, dm_dt, fac):
    """balance.py:192-199, in place."""
    resid = convergence(pu, pv) + pw[..., :-1] - pw[..., 1:] - dm_dt
    for k in range(dm_dt.shape[2]):
        u, v = poisson_correction(resid[..., k], fac)
        pu[..., k] += u
        pv[..., k] += v


def setup_mass(pu, pv, pw, sp1, sp2, levi_db, area, dt, max_tries=3):
    """balance.py:202-219: pu, pv balanced in place; returns (tries, ok, pre, post)."""
    fac = poisson_factor(*sp1.shape)
    dm_dt = fill_mass_change(sp1, sp2, levi_db, area, dt)
    ok0, rms0, mav0 = check_mass_balance(pu, pv, sp1, sp2, dt, area, *MB_TOL_PRE)
    if not ok0:
        raise ValueError(f"setup_mass: unbalanced input fluxes (rms {rms0:.3e}, max {mav0:.3e})")
    for tries in range(1, max_tries + 1):  # noqa: B007
        balance_mass_fluxes(pu, pv, pw, dm_dt, fac)
        ok, rms, mav = check_mass_balance(pu, pv, sp1, sp2, dt, area, *MB_TOL_TIGHT)
        if ok:
            break
    return tries, ok, (rms0, mav0), (rms, mav)


# ------------------------------------------------------------------ a child (zoom_meteo.py)
def cells(rf):
    """(ci, cj, fi, fj) of every covered parent cell, cj outer (zoom_meteo.py:79-84); rf =
    (ri, rj, ci1, ci2, cj1, cj2)."""
    ri, rj, ci1, ci2, cj1, cj2 = rf
    for cj in range(cj1, cj2 + 1):
        for ci in range(ci1, ci2 + 1):
            yield ci, cj, (ci - ci1) * ri, (cj - cj1) * rj


def match_cell_sum(pg, tg, rf):
    """zoom_meteo.py:87-97."""
    ri, rj = rf[0], rf[1]
    for ci, cj, fi, fj in cells(rf):
        block = tg[fi : fi + ri, fj : fj + rj]
        fsum = seqsum(block.reshape(ri * rj, *block.shape[2:], order="F"), axis=0)
        block[...] = block + ((pg[ci - 1, cj - 1] - fsum) / (rj * ri))


def match_u_sum(pg, tg, rf):
    """zoom_meteo.py:100-108."""
    ri, rj, ci1, ci2, cj1, cj2 = rf
    for cj in range(cj1, cj2 + 1):
        fj = (cj - cj1) * rj
        for ci in range(ci1 - 1, ci2 + 1):
            fi = (ci - (ci1 - 1)) * ri
            face = tg[fi, fj : fj + rj]
            face[...] = face + (pg[ci, cj - 1] - seqsum(face, axis=0)) / rj


def match_v_sum(pg, tg, rf):
    """zoom_meteo.py:111-119."""
    ri, rj, ci1, ci2, cj1, cj2 = rf
    for cj in range(cj1 - 1, cj2 + 1):
        fj = (cj - (cj1 - 1)) * rj
        for ci in range(ci1, ci2 + 1):
            fi = (ci - ci1) * ri
            face = tg[fi : fi + ri, fj]
            face[...] = face + (pg[ci - 1, cj] - seqsum(face, axis=0)) / ri


def direct_matrices(ri, rj):
    """zoom_meteo.py:141-161 (PoissonDirect): column k is the correction of the unit divergence
    at cell k (column-major) -- (m_to_u ((ri+1) rj, n), m_to_v (ri (rj+1), n))."""
    n, fac = ri * rj, poisson_factor(ri, rj)
    mu, mv = np.empty(((ri + 1) * rj, n)), np.empty((ri * (rj + 1), n))
    for k in range(n):
        unit = np.zeros(n)
        unit[k] = 1.0
        u, v = poisson_correction(unit.reshape(ri, rj, order="F"), fac)
        mu[:, k] = u.reshape(-1, order="F")
        mv[:, k] = v.reshape(-1, order="F")
    return mu, mv


def balance_mass_fluxes_child(pu, pv, pw, dm_dt, rf, mu, mv):
    """zoom_meteo.py:163-181 (the residual of every level first, then per parent cell the
    direct correction added to its block's faces), in place."""
    ri, rj = rf[0], rf[1]
    resid = convergence(pu, pv) + pw[..., :-1] - pw[..., 1:] - dm_dt
    for _ci, _cj, fi, fj in cells(rf):
        m = resid[fi : fi + ri, fj : fj + rj]
        vec = m.reshape(ri * rj, *m.shape[2:], order="F")
        u = np.zeros((mu.shape[0], *m.shape[2:]))
        v = np.zeros((mv.shape[0], *m.shape[2:]))
        for k in range(vec.shape[0]):
            u = u + mu[:, k][:, None] * vec[k]
            v = v + mv[:, k][:, None] * vec[k]
        pu[fi : fi + ri + 1, fj : fj + rj] += u.reshape(ri + 1, rj, *m.shape[2:], order="F")
        pv[fi : fi + ri, fj : fj + rj + 1] += v.reshape(ri, rj + 1, *m.shape[2:], order="F")


def setup_mass_child(raw, parent, sp1, sp2, levi_db, area, dt, rf, mu, mv, max_tries=3):
    """zoom_meteo.py:184-209: (pu, pv, pw, tries, ok)."""
    pu, pv, pw = (q.copy() for q in raw)
    ppu, ppv, ppw = parent
    match_u_sum(ppu, pu, rf)
    match_v_sum(ppv, pv, rf)
    match_cell_sum(ppw, pw, rf)
    dm_dt = fill_mass_change(sp1, sp2, levi_db, area, dt)
    ok0, rms0, mav0 = check_mass_balance(pu, pv, sp1, sp2, dt, area, *MB_TOL_PRE)
    if not ok0:
        raise ValueError(f"setup_mass_child: unbalanced matched fluxes (rms {rms0:.3e}, max {mav0:.3e})")
    for tries in range(1, max_tries + 1):  # noqa: B007
        balance_mass_fluxes_child(pu, pv, pw, dm_dt, rf, mu, mv)
        ok, rms, mav = check_mass_balance(pu, pv, sp1, sp2, dt, area, *MB_TOL_TIGHT)
        if ok:
            break
    return pu, pv, pw, tries, ok
