"""Seeded synthetic inputs of the benchmark configurations, identical to the bit on any host.

The generator uses NumPy's PCG64 stream (`Generator.random`, `integers`) and only IEEE-exact
operations (+ - * /, sqrt, ldexp): its own sine, cosine and exponential below are polynomial
evaluations after an exact range reduction, so that the x86 container that makes the golden
fixtures and the aarch64 GPU machine regenerate the same bits (NumPy's vectorised transcendentals
differ between the two).  Reductions use math.fsum (exactly rounded).

Configurations (dims as the benchmark names them):
    glb6x4      60 x 45 x 25, reduced grid jred (1, 2, 3, 45) clustsize (60, 20, 10, 60)
    glb3x2      120 x 90 x 34, reduced grid of the production fixture
    glb3x2+nam1x1  the above with a 90 x 70 child at 140W-50W, 10N-80N, xref 3, yref 2, tref 2
    glb3x2+nam72x44  glb3x2 with a 72 x 44 child at 132W-60W, 20N-64N, xref 3, yref 2, tref 2
                   (the tree pydyn's own GPU benchmark times)

Air mass from a surface pressure of 1e5 Pa +- 2 % smooth noise on hybrid a / b levels; mass
fluxes from a seeded streamfunction of eight low spherical modes (winds up to 40 m/s, so the
horizontal flow is divergence-free up to rounding) plus a small seeded velocity potential (so
the vertical flux the column balance makes is not zero and z sub-cycles); two meteo instants six
hours apart that each step interpolates between.  Tracer: mixing ratio 1.8e-6 plus a Gaussian
blob of 2e-7, slopes zero."""

import math

import numpy as np

from .tree import RedGrid, Region, Zoom

AE = 6.371e6
GRAV = 9.80665
PI = 3.14159265358979  # the reference's PI (balance.py), a default-real literal

G6_JRED, G6_CLUST = (1, 2, 3, 45), (60, 20, 10, 60)
G3_JRED = (1, 2, 3, 4, 5, 6, 7, 84, 85, 86, 87, 88, 89, 90)
G3_CLUST = (40, 8, 8, 4, 4, 4, 2, 2, 4, 4, 4, 8, 8, 40)


# ------------------------------------------------------------------ deterministic elementary functions
def _poly(x, coeffs):
    acc = np.full_like(x, coeffs[-1])
    for c in coeffs[-2::-1]:
        acc = acc * x + c
    return acc


_SIN = [(-1.0) ** k / math.factorial(2 * k + 1) for k in range(11)]
_COS = [(-1.0) ** k / math.factorial(2 * k) for k in range(11)]
_HALF_PI_HI = 1.5707963267341256  # pi/2 split so that k * HI is exact for |k| < 2**20
_HALF_PI_LO = 6.077100506506192e-11


def sin_cos(x):
    """(sin x, cos x) to ~1 ulp for |x| < 1e5, by quadrant reduction and Taylor series."""
    x = np.asarray(x, dtype=np.float64)
    k = np.floor(x / (_HALF_PI_HI + _HALF_PI_LO) + 0.5)
    r = (x - k * _HALF_PI_HI) - k * _HALF_PI_LO
    r2 = r * r
    s = r * _poly(r2, _SIN)
    c = _poly(r2, _COS)
    q = np.mod(k, 4.0)
    sin = np.where(q == 0, s, np.where(q == 1, c, np.where(q == 2, -s, -c)))
    cos = np.where(q == 0, c, np.where(q == 1, -s, np.where(q == 2, -c, s)))
    return sin, cos


_EXP = [1.0 / math.factorial(k) for k in range(16)]
_LN2 = 0.6931471805599453


def exp(x):
    """e**x to ~1 ulp for moderate x: x = k ln2 + r, a Taylor series of r, ldexp."""
    x = np.asarray(x, dtype=np.float64)
    k = np.floor(x / _LN2 + 0.5)
    r = x - k * _LN2
    return np.ldexp(_poly(r, _EXP), k.astype(np.int64))


def _normalise(a):
    top = max(abs(float(a.max())), abs(float(a.min())))
    return a / top if top > 0 else a


# ------------------------------------------------------------------ grids and levels
def levels(lm, top=2000.0):
    """Hybrid coefficients at the lm+1 interfaces, surface first: a from `top` Pa... down to 0
    at the model top with b 1 -> 0 (the benchmark's fixed a / b)."""
    frac = np.array([(lm - l) / lm for l in range(lm + 1)])
    at = top * np.array([l / lm for l in range(lm + 1)]) * frac * 4.0
    bt = frac * frac
    at[0], at[lm], bt[lm] = 0.0, 0.0, 0.0
    return at, bt


def cell_area(g):
    """dxyp (jm): AE^2 dlon (sin(lat north) - sin(lat south)) of the region's rows."""
    dx, dy = (g.xend - g.xbeg) / g.im, (g.yend - g.ybeg) / g.jm
    edges = np.array([g.ybeg + dy * j for j in range(g.jm + 1)]) * (PI / 180.0)
    s, _ = sin_cos(edges)
    return (AE * AE * (dx * PI / 180.0)) * (s[1:] - s[:-1])


def glb6x4():
    g = Region("glb6x4", 60, 45, xcyc=1, touch_sp=1, touch_np=1, redgrid=RedGrid(60, 45, G6_JRED, G6_CLUST))
    return [g]


def glb3x2():
    g = Region("glb3x2", 120, 90, xcyc=1, touch_sp=1, touch_np=1, redgrid=RedGrid(120, 90, G3_JRED, G3_CLUST))
    return [g]


def nam1x1():
    """The 90 x 70 child over North America.  141W-51W rather than 140W-50W: the benchmark's
    corners are not on glb3x2's 3-degree lines, and TM5's nint would place the footprint at
    parent cells 14..43 (141W-51W) while the child's own fluxes sit one degree east, so its
    boundary fluxes would not match the parent's and cells near the interface would drain.
    The footprint (i 14..43, j 51..85) and every size are the benchmark's."""
    return Region("nam1x1", 90, 70, xbeg=-141, xend=-51, ybeg=10, yend=80, xref=3, yref=2, tref=2, parent=1)


def nam72x44():
    """The 72 x 44 child over North America of pydyn's own GPU benchmark tree: 132W-60W,
    20N-64N at xref 3, yref 2, tref 2 -- corners on glb3x2's 3 x 2 degree lines, footprint
    i 17..40, j 56..77."""
    return Region("nam1x1", 72, 44, xbeg=-132, xend=-60, ybeg=20, yend=64, xref=3, yref=2, tref=2, parent=1)


def two():
    """A 24 x 18 parent (15 x 10 degrees) and one child at nam1x1's refinements (xref 3,
    yref 2, tref 2): the shape of the reference's small tree tests."""
    glb = Region("glb", 24, 18, xcyc=1, touch_sp=1, touch_np=1)
    child = Region("child", 24, 16, xbeg=-105, xend=15, ybeg=-30, yend=50, xref=3, yref=2, tref=2, parent=1)
    return [glb, child]


def one():
    """A 24 x 18 global region alone (15 x 10 degrees) with a reduced grid on its two outer rows
    at each pole: the adjoint's small case, where the reference's forward can be applied to
    basis vectors."""
    g = Region("one", 24, 18, xcyc=1, touch_sp=1, touch_np=1, redgrid=RedGrid(24, 18, (1, 2, 17, 18), (24, 6, 6, 24)))
    return [g]


def three():
    """A grandchild: region 2 at 2 x 2 / tref 2, region 3 at 3 x 2 / tref 2 relative to it."""
    glb = Region("glb", 24, 18, xcyc=1, touch_sp=1, touch_np=1)
    mid = Region("mid", 16, 16, xbeg=-90, xend=30, ybeg=-40, yend=40, xref=2, yref=2, tref=2, parent=1)
    fine = Region("fine", 30, 16, xbeg=-75, xend=0, ybeg=-20, yend=20, xref=6, yref=4, tref=4, parent=2)
    return [glb, mid, fine]


def tree(name, lm):
    regions = {"glb6x4": glb6x4, "glb3x2": glb3x2, "glb3x2+nam1x1": lambda: [*glb3x2(), nam1x1()],
               "glb3x2+nam72x44": lambda: [*glb3x2(), nam72x44()], "two": two,
               "three": three, "one": one}[name]()  # fmt: skip
    at, bt = levels(lm)
    return Zoom(regions, lm, at, bt)


# ------------------------------------------------------------------ fields on a region
def _centres(g):
    dx, dy = (g.xend - g.xbeg) / g.im, (g.yend - g.ybeg) / g.jm
    lon = np.array([g.xbeg + dx * (i + 0.5) for i in range(g.im)])
    lat = np.array([g.ybeg + dy * (j + 0.5) for j in range(g.jm)])
    return lon * (PI / 180.0), lat * (PI / 180.0)


def _corners(g):
    dx, dy = (g.xend - g.xbeg) / g.im, (g.yend - g.ybeg) / g.jm
    lon = np.array([g.xbeg + dx * i for i in range(g.im + 1)])
    lat = np.array([g.ybeg + dy * j for j in range(g.jm + 1)])
    return lon * (PI / 180.0), lat * (PI / 180.0)


class Modes:
    """A seeded sum of low spherical modes cos(lat)^p cos(m lon + a) sin(n lat + b)."""

    def __init__(self, rng, count=8):
        r = rng.random((count, 6))
        self.m = np.floor(r[:, 0] * 3.0) + 1.0
        self.n = np.floor(r[:, 1] * 3.0) + 1.0
        self.a = r[:, 2] * (2 * PI)
        self.b = r[:, 3] * (2 * PI)
        self.w = r[:, 4] * 2.0 - 1.0

    def __call__(self, lon, lat):
        lon, lat = np.broadcast_arrays(np.asarray(lon, dtype=float), np.asarray(lat, dtype=float))
        _, clat = sin_cos(lat)
        out = np.zeros(lon.shape)
        for m, n, a, b, w in zip(self.m, self.n, self.a, self.b, self.w, strict=True):
            _, c = sin_cos(m * lon + a)
            s, _ = sin_cos(n * lat + b)
            out = out + w * (clat * c * s)
        return out


class Meteo:
    """The meteo of one configuration: surface pressure, streamfunction and potential modes
    per meteo instant, the region geometry, and the mass fluxes pu, pv of every region."""

    def __init__(self, zoom, seed, umax=40.0, chi_frac=0.05, wind_scale=1.0):
        self.zoom = zoom
        rng = np.random.default_rng(seed)
        self.sp_modes = Modes(rng, 6)
        self.psi = [Modes(rng, 8), Modes(rng, 8)]  # two meteo instants
        # the divergent part changes sign between the instants, so that the convergence a cell
        # sees averages out over the interpolation cycle and no column drains over a long run
        chi = Modes(rng, 8)
        neg = Modes.__new__(Modes)
        neg.m, neg.n, neg.a, neg.b, neg.w = chi.m, chi.n, chi.a, chi.b, -chi.w
        self.chi = [chi, neg]
        self.level_w = 0.4 + 0.6 * rng.random(zoom.lm)
        self.level_sign = np.where(rng.random(zoom.lm) < 0.15, -1.0, 1.0)
        self.umax, self.chi_frac, self.wind_scale = umax, chi_frac, wind_scale
        self.blob = rng.random(3)

    def surface_pressure(self, g):
        lon, lat = _centres(g)
        noise = _normalise(self.sp_modes(lon[:, None], lat[None, :]))
        return 1.0e5 * (1.0 + 0.02 * noise)

    def mass(self, g, sp):
        """m (im, jm, lm): the hybrid layer's pressure difference times the cell area over g."""
        at, bt = self.zoom.at, self.zoom.bt
        dxyp = cell_area(g)
        dp = (at[None, None, :-1] - at[None, None, 1:]) + (bt[None, None, :-1] - bt[None, None, 1:]) * sp[..., None]
        return dp * dxyp[None, :, None] / GRAV

    def fluxes(self, r, instant):
        """(pu (im+1, jm, lm), pv (im, jm+1, lm)) in kg/s of region r at a meteo instant.  The
        wind scales are the global region's, so every region samples one and the same flow and
        a child's boundary fluxes are its parent's."""
        if r != 1:
            self._winds(1, instant)
        return self._winds(r, instant)

    def _winds(self, r, instant):
        g = self.zoom.g(r)
        lonc, latc = _corners(g)
        lon, lat = _centres(g)
        psi = self.psi[instant](lonc[:, None], latc[None, :])  # (im+1, jm+1) corners
        chi = self.chi[instant](lon[:, None], lat[None, :])  # (im, jm) centres
        dx, dy = (g.xend - g.xbeg) / g.im, (g.yend - g.ybeg) / g.jm
        dyy = AE * dy * (PI / 180.0)
        _, clat = sin_cos(lat)
        dxx = AE * dx * (PI / 180.0) * clat  # (jm,)
        u_psi = (psi[:, 1:] - psi[:, :-1]) / dyy  # x faces (im+1, jm)
        # v on y faces: the streamfunction difference along x over the face's own width
        _, clat_f = sin_cos(latc)
        dxf = AE * dx * (PI / 180.0) * clat_f  # (jm+1,)
        dpsi_x = psi[1:, :] - psi[:-1, :]  # (im, jm+1)
        v_psi = -np.where(np.abs(dxf) > 1.0, dpsi_x / np.where(np.abs(dxf) > 1.0, dxf, 1.0)[None, :], 0.0)
        # velocity potential: gradient between neighbouring centres
        chi_w = np.concatenate([chi[-1:], chi, chi[:1]], axis=0) if g.xcyc else np.concatenate([chi[:1], chi, chi[-1:]])
        u_chi = (chi_w[1:] - chi_w[:-1]) / dxx[None, :]
        v_chi = np.zeros((g.im, g.jm + 1))
        v_chi[:, 1:-1] = (chi[:, 1:] - chi[:, :-1]) / dyy
        if r == 1:
            self._scale = getattr(self, "_scale", {})
            self._scale[instant] = (
                self.umax / max(float(np.abs(u_psi).max()), float(np.abs(v_psi).max())),
                self.chi_frac * self.umax / max(float(np.abs(u_chi).max()), float(np.abs(v_chi).max()), 1e-300),
            )
        scale, cs = self._scale[instant]
        u = (u_psi * scale + u_chi * cs) * self.wind_scale
        v = (v_psi * scale + v_chi * cs) * self.wind_scale
        if g.xcyc:
            u[g.im] = u[0]
        if g.touch_sp:
            v[:, 0] = 0.0
        if g.touch_np:
            v[:, g.jm] = 0.0
        # mass flux = wind * (layer pressure thickness / g) * face length, per level
        at, bt = self.zoom.at, self.zoom.bt
        dp = (at[:-1] - at[1:]) + (bt[:-1] - bt[1:]) * 1.0e5
        w = self.level_w * self.level_sign * dp / GRAV
        pu = (u * dyy)[..., None] * w[None, None, :]
        pv = (v * dxf[None, :])[..., None] * w[None, None, :]
        return pu, pv

    def tracer(self, r, m):
        """rm (im, jm, lm, 1): m times 1.8e-6 plus a 2e-7 Gaussian blob."""
        g = self.zoom.g(r)
        lon, lat = _centres(g)
        slon, clon = sin_cos(lon)
        slat, clat = sin_cos(lat)
        b = self.blob
        blon, blat = (b[0] * 2.0 - 1.0) * PI, (b[1] - 0.5) * PI * 0.6
        (sb,), (cb,) = sin_cos(np.array([blon]))
        (sa,), (ca,) = sin_cos(np.array([blat]))
        x0, y0, z0 = ca * cb, ca * sb, sa
        x = clat[None, :] * clon[:, None]
        y = clat[None, :] * slon[:, None]
        z = np.broadcast_to(slat[None, :], x.shape)
        d2 = (x - x0) * (x - x0) + (y - y0) * (y - y0) + (z - z0) * (z - z0)
        sigma2 = 0.08 + 0.1 * b[2]
        mix = 1.8e-6 + 2.0e-7 * exp(-d2 / (2.0 * sigma2))
        return (m * mix[..., None])[..., None]


KZZ_SURFACE = ("oro", "lsm", "sr", "srols", "u10m", "v10m", "sshf", "slhf", "ewss", "nsss")
CHEM_SETTINGS = {"oh_scale": 0.901, "cl_scale": 1.0, "o1d_scale": 1.0, "soil_rate": 2.0e-4}


class Physics:
    """The physics inputs of a configuration, per region, as host arrays:

    conv    entu, detu, entd, detd (im, jm, lmax) kg/s and cloud_top, cloud_lfs (im, jm) int32:
            40 % of the columns convective with cloud tops at levels 10-30, an updraft flux of
            up to 0.05 kg m-2 s-1 times the cell area shaped as sin^2 over the cloud (its peak
            mid-cloud, near 500 hPa), entrainment where it grows and detrainment where it
            falls, and a downdraft of 0.3 of it below the level of free sinking
    kzz     t, q (im, jm, lm); the ten surface fields of Calc_Kzz (im, jm); two instants of the
            surface pressure spm (the meteo's, interpolated to each step's middle)
    chem    lat (jm) radians; the zonal loss-rate columns strat_press (hPa, descending),
            strat_oh, strat_cl, strat_od (jm, ns) at 1e-9 - 1e-7 s-1; oh_3d (im, jm, lm) at
            1e5 - 3e6, times a diurnal factor per longitude (oh_factor); the tropospheric Cl
            column pl_trop (Pa, descending), cl_trop (im, jm, ntrop); soil (im, jm) on land,
            a source of at most 1e-8 s-1 at CHEM_SETTINGS' soil_rate
    emis    flux (im, jm) kg m-2 s-1, log-normal with mean 1e-10 (three times denser on a
            child), injected at level 1 as flux x area x the region's half step

    The temperature falls from 270-300 K at the surface to about 215 K at the top (200-300 K),
    so the Kzz boundary layers grow over heated land and stay shallow over the sea.

    kind = "convection" makes the inputs of pydyn's own GPU benchmark instead (convection with a
    given dkg; no Calc_Kzz, emission or chemistry): per region a rate of 5 % of the mean cell
    mass per 1800 s, entu, detu and dkg uniform in [0, rate), entd, detd in [0, 0.3 rate), and
    cloud_top, cloud_lfs uniform in 0..lmax -- nearly every column convective."""

    def __init__(self, zoom, met, seed, lmax, ns=24, ntrop=10, child_density=3.0, kind="full"):
        if kind not in ("full", "convection"):
            raise ValueError(f"synth.Physics: kind {kind!r} is neither 'full' nor 'convection'")
        self.zoom, self.lmax, self.ns, self.ntrop, self.kind = zoom, lmax, ns, ntrop, kind
        self.settings = dict(CHEM_SETTINGS)
        self.region = {}
        for r in zoom.regions():
            rng = np.random.default_rng([seed, 7919, r])
            if kind == "convection":
                self.region[r] = self._convection_only(rng, r, met)
            else:
                self.region[r] = self._region(rng, r, met, 1.0 if r == 1 else child_density)

    def _convection_only(self, rng, r, met):
        g, lmax = self.zoom.g(r), self.lmax
        m = met.mass(g, met.surface_pressure(g))
        rate = 0.05 * (math.fsum(m.ravel()) / m.size) / 1800.0
        shape = (g.im, g.jm, lmax)
        conv = {
            "entu": rate * rng.random(shape), "detu": rate * rng.random(shape),
            "entd": 0.3 * rate * rng.random(shape), "detd": 0.3 * rate * rng.random(shape),
            "cloud_top": np.floor(rng.random((g.im, g.jm)) * (lmax + 1)).astype(np.int32),
            "cloud_lfs": np.floor(rng.random((g.im, g.jm)) * (lmax + 1)).astype(np.int32),
        }  # fmt: skip
        return {"conv": conv, "dkg": rate * rng.random(shape)}

    def _region(self, rng, r, met, density):
        z, g = self.zoom, self.zoom.g(r)
        im, jm, lm, lmax = g.im, g.jm, z.lm, self.lmax
        lon, lat = _centres(g)
        slat, clat = sin_cos(lat)
        sp0 = met.surface_pressure(g)
        # levels: mid-layer sigma of each column
        at, bt = z.at, z.bt
        ph = at[None, None, :] + bt[None, None, :] * sp0[..., None]
        sig = ((ph[..., :-1] + ph[..., 1:]) * 0.5) / sp0[..., None]
        out = {}
        # ---- convection
        u = rng.random((im, jm))
        top = np.where(rng.random((im, jm)) < 0.4, 10 + np.floor(u * 21.0), 0.0).astype(np.int32)
        top = np.minimum(top, lmax).astype(np.int32)
        lfs = np.where(top > 0, 2 + np.floor(rng.random((im, jm)) * np.maximum(top - 2, 1)), 0.0).astype(np.int32)
        dxyp = cell_area(g)
        k = np.arange(lmax + 1, dtype=np.float64)[None, None, :]
        T = np.maximum(top, 1).astype(np.float64)[..., None]
        s, _ = sin_cos(PI * np.minimum(k, T) / T)
        peak = 0.05 * rng.random((im, jm)) * dxyp[None, :]
        flux = np.where((k <= T) & (top[..., None] > 0), s * s, 0.0) * peak[..., None]
        d = flux[..., 1:] - flux[..., :-1]
        noise = 1.0 + 0.2 * rng.random((im, jm, lmax))
        entu, detu = np.maximum(d, 0.0) * noise, np.maximum(-d, 0.0) * noise
        lev = np.arange(lmax)[None, None, :]
        down = (lev < lfs[..., None]).astype(np.float64)
        entd, detd = 0.3 * detu * down, 0.3 * entu * down
        out["conv"] = {"entu": entu, "detu": detu, "entd": entd, "detd": detd, "cloud_top": top, "cloud_lfs": lfs}
        # ---- Calc_Kzz
        ts = 300.0 - 30.0 * (slat * slat)
        t = 215.0 + (ts[None, :, None] - 215.0) * sig + (rng.random((im, jm, lm)) * 2.0 - 1.0)
        q = 0.015 * (sig * sig * sig) * (0.5 + 0.5 * rng.random((im, jm, lm))) + 1.0e-6
        land = _normalise(Modes(rng, 6)(lon[:, None], lat[None, :])) > 0.2
        r2 = lambda lo, hi: lo + (hi - lo) * rng.random((im, jm))  # noqa: E731
        surf = {
            "oro": np.where(land, GRAV * 2000.0 * rng.random((im, jm)), 0.0),
            "lsm": np.where(land, 100.0, 0.0),
            "sr": np.where(land, r2(0.05, 0.5), r2(1e-4, 1e-3)),
            "srols": np.where(land, r2(0.1, 1.0), r2(1e-3, 1e-2)),
            "u10m": r2(-8.0, 8.0),
            "v10m": r2(-8.0, 8.0),
            "sshf": np.where(land, r2(-250.0, 40.0), r2(-30.0, 15.0)),
            "slhf": np.where(land, r2(-200.0, 0.0), r2(-150.0, 0.0)),
            "ewss": np.where(land, r2(-0.1, 0.1), r2(-0.3, 0.3)),
            "nsss": np.where(land, r2(-0.1, 0.1), r2(-0.3, 0.3)),
        }
        sp1 = sp0 * (1.0 + 0.003 * _normalise(Modes(rng, 4)(lon[:, None], lat[None, :])))
        out["kzz"] = {"t": t, "q": q, "surface": surf, "spm": (sp0, sp1)}
        # ---- chemistry
        ns, nt = self.ns, self.ntrop
        kk = np.arange(ns, dtype=np.float64)
        col = 1000.0 * exp(-kk * (7.6 / (ns - 1)))  # 1000 hPa .. 0.5 hPa, descending
        press = col[None, :] * (1.0 + 0.01 * rng.random((jm, 1)))
        strat = {n: 1e-9 + (1e-7 - 1e-9) * rng.random((jm, ns)) for n in ("strat_oh", "strat_cl", "strat_od")}
        steps = 0.5 + rng.random((im, jm, nt))
        csum = np.cumsum(steps, axis=-1)
        pl = 1.0e5 - 9.0e4 * (csum - steps[..., :1]) / (csum[..., -1:] - steps[..., :1])
        out["chem"] = {
            "lat": lat, "strat_press": press, **strat,
            "oh_3d": 1e5 + (3e6 - 1e5) * rng.random((im, jm, lm)),
            "pl_trop": pl, "cl_trop": 1e3 * rng.random((im, jm, nt)),
            "soil": np.where(land, 5.0e-5 * rng.random((im, jm)), 0.0),  # soil_rate x soil <= 1e-8 s-1
        }  # fmt: skip
        # ---- emission: log-normal (Irwin-Hall normal deviate), mean 1e-10 kg m-2 s-1
        zdev = rng.random((12, im, jm)).sum(axis=0) - 6.0
        out["flux"] = density * 1.0e-10 * exp(zdev - 0.5)
        out["lon"] = lon
        return out

    def oh_factor(self, r, t):
        """(im,) the diurnal factor of OH at time t (s) for each longitude of region r: 0.2 at
        night, up to 1.0 at local noon."""
        lon = self.region[r]["lon"]
        _, c = sin_cos(2.0 * PI * (t / 86400.0) + lon - PI)
        return 0.2 + 0.8 * np.maximum(c, 0.0)

    def half_step(self, r, ndyn):
        """The region's half step dt = ndyn / (2 tref) (convec_region's, zoom/physics.py:50)."""
        return ndyn / (2.0 * self.zoom.g(r).tref)

    def factors(self, r, t0, ndyn):
        """(2 tref, im): the OH factor of each of the region's halves of the step from t0."""
        dt = self.half_step(r, ndyn)
        return np.stack([self.oh_factor(r, t0 + h * dt) for h in range(2 * self.zoom.g(r).tref)])


def case(name, lm, seed=0, nt=1, umax=40.0, wind_scale=1.0):
    """(zoom, meteo, {r: {field: host array}}): the initial state of every region in the
    declared (halo'd) shapes: m and rm from the meteo's surface pressure, slopes zero, dxyp.
    pu / pv are set per step by the run (interpolated between the meteo instants); wind_scale
    multiplies the winds (an ensemble member's perturbation)."""
    from .layout import bounds

    zoom = tree(name, lm)
    met = Meteo(zoom, seed, umax=umax, wind_scale=wind_scale)
    fields = {}
    for r in zoom.regions():
        g = zoom.g(r)
        sp = met.surface_pressure(g)
        m = met.mass(g, sp)
        rm = met.tracer(r, m)
        if nt > 1:
            rm = np.concatenate([rm * (k + 1) for k in range(nt)], axis=3)
        f = {}
        for fname in ("m", "rm", "rxm", "rym", "rzm", "dxyp"):
            shape = tuple(hi - lo + 1 for lo, hi in bounds(fname, g.im, g.jm, lm, nt))
            f[fname] = np.zeros(shape)
        f["m"][2 : g.im + 2, 2 : g.jm + 2] = m
        f["rm"][2 : g.im + 2, 2 : g.jm + 2] = rm
        f["dxyp"][:] = cell_area(g)
        fields[r] = f
    return zoom, met, fields


# ------------------------------------------------------------------ the ensemble's member classes
# class: (tree, levels, convection levels, the class's meteo seed)
ENSEMBLE_CLASSES = {
    "glb6x4": ("glb6x4", 25, 25, 11),
    "glb3x2": ("glb3x2", 34, 34, 41),
    "glb3x2+nam1x1": ("glb3x2+nam1x1", 34, 34, 42),
}
ENSEMBLE_MIX = (("glb6x4", 128), ("glb3x2", 96), ("glb3x2+nam1x1", 32))


# ------------------------------------------------------------------ the meteo's time weights
WINDOW = 6 * 3600.0  # seconds between the two meteo instants


def weights(t):
    """(alfa1, alfa2) of the two meteo instants at time t (s): a triangle wave between them."""
    cycle = t / WINDOW
    k = int(np.floor(cycle))
    frac = cycle - k
    return (1.0 - frac, frac) if k % 2 == 0 else (frac, 1.0 - frac)
