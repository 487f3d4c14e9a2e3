"""The sm_103a kernels against the reference's outputs (golden fixtures) and against the oracle
on larger seeded inputs: bitwise, every array the kernel writes; the same errors."""

import zlib
from pathlib import Path

import numpy as np
import pytest
from cases import TRACERS, run_device, run_oracle
from conftest import assert_bitwise
from make_golden import load

CASES = load(Path(__file__).parent / "golden" / "kernels.npz")


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_device_matches_reference(dev, name):
    ins, outs, meta = CASES[name]
    got, err = run_device(dev, ins, meta)
    assert err == meta.get("error"), f"{name}: error {err} vs {meta.get('error')}"
    for k, v in outs.items():
        assert_bitwise(got[k], v, f"{name}.{k}")


def _state(rng, im, jm, lm, nt, cfl):
    """Seeded admissible inputs: masses ~1e9, tracers with slopes, per-line fluxes of Courant ~cfl
    (x periodic rows of one sign; y and z closed lines moving each line to a positive target)."""
    m = 1e9 * rng.uniform(0.8, 1.2, (im, jm, lm))
    rm = m[..., None] * rng.uniform(0.5, 1.5, (im, jm, lm, nt)) * 1e-6
    slopes = [0.3 * rm * rng.uniform(-1, 1, rm.shape) for _ in range(3)]
    scale = cfl * m.mean()
    am = scale * rng.choice([-1.0, 1.0], (1, jm, lm)) * rng.uniform(0.8, 1.0, (im + 1, jm, lm))
    am[im] = am[0]

    def closed(axis, amp):
        target = m * (1.0 + amp * rng.uniform(-1, 1, m.shape))
        target *= m.sum(axis=axis, keepdims=True) / target.sum(axis=axis, keepdims=True)
        f = np.cumsum(m - target, axis=axis)
        shape = list(m.shape)
        shape[axis] = 1
        return np.concatenate([np.zeros(shape), f], axis=axis)

    amp = min(0.6 * cfl, 0.9)
    bm = closed(1, amp)
    bm[:, jm] = 0.0
    cm = closed(2, amp)
    cm[..., lm] = 0.0
    return {"m": m, "rm": rm, "rxm": slopes[0], "rym": slopes[1], "rzm": slopes[2]}, (am, bm, cm)


def _convection(rng, m, lmax, dt, frac=0.4):
    """Seeded convection inputs in kernels.convec's layout: a fraction of the columns convective
    with cloud tops in 10..30 (a smooth updraft flux peaking mid-cloud, a downdraft a third as
    strong below the level of free sinking), the rest diffusion only; dkg everywhere."""
    im, jm, lm = m.shape
    top = np.where(rng.random((im, jm)) < frac, rng.integers(10, 31, (im, jm)), 0).astype(np.int32)
    top = np.minimum(top, lmax).astype(np.int32)
    lfs = np.where(top > 0, rng.integers(2, np.maximum(top, 3)), 0).astype(np.int32)
    k = np.arange(lm + 1)[None, None, :]
    T = np.maximum(top, 1)[..., None]
    flux = np.where(k <= T, np.sin(np.pi * np.minimum(k, T) / T) ** 2, 0.0) * (0.05 * m.mean(axis=2, keepdims=True) / dt)
    d = np.diff(flux, axis=2)
    noise = 1.0 + 0.2 * rng.random(m.shape)
    entu, detu = np.maximum(d, 0.0) * noise, np.maximum(-d, 0.0) * noise
    entd, detd = 0.3 * detu[..., ::-1].copy(), 0.3 * entu[..., ::-1].copy()
    dkg = 0.02 * m[..., :lmax] / dt * rng.random((im, jm, lmax))
    return {"entu": entu, "detu": detu, "entd": entd, "detd": detd, "dkg": dkg, "cloud_top": top, "cloud_lfs": lfs}


@pytest.mark.gpu
@pytest.mark.parametrize(("shape", "lmax"), [((120, 90, 34, 1), 34), ((90, 70, 34, 1), 26), ((40, 30, 60, 2), 60)])
@pytest.mark.parametrize("lu_lanes", [8, 16, 32])
def test_convec_matches_oracle_at_size(dev, shape, lmax, lu_lanes):
    """Convection on every column, then again on the same air mass: the second call reuses the
    kept inverses, and both equal the oracle's two applications bitwise, for every width of
    the LU's lane groups."""
    from oracle import kernels as O

    from pydyn_gb300 import kernels as K
    from pydyn_gb300.device import DevArray

    im, jm, lm, nt = shape
    rng = np.random.default_rng(zlib.crc32(repr(shape).encode()))
    st, _ = _state(rng, im, jm, lm, nt, 0.5)
    conv = _convection(rng, st["m"], lmax, 1800.0)
    want = {k: v.copy() for k, v in st.items()}
    for _ in range(2):
        O.convec(want["m"], *(want[q] for q in TRACERS), conv["entu"], conv["detu"], conv["entd"], conv["detd"],
                 conv["cloud_top"], conv["cloud_lfs"], conv["dkg"], 1800.0, lmax)  # fmt: skip
    d = {k: DevArray.from_host(dev, v) for k, v in {**st, **conv}.items()}
    ncol = im * jm
    cols = DevArray.from_host(dev, np.array([(i, j) for i in range(im) for j in range(jm)], dtype=np.int32))
    cache = (DevArray.zeros(dev, (0, ncol * lmax * lmax - 1)), DevArray.zeros(dev, (0, ncol * lmax - 1)),
             DevArray.zeros(dev, (0, ncol - 1), dtype=np.int32), DevArray.from_host(dev, np.array([7], np.int32)))
    saved = dev.tuning()["lu_lanes"]
    dev.tune(lu_lanes=lu_lanes)
    try:
        before = dev.launches()
        for _ in range(2):
            K.convec(d["m"], *(d[q] for q in TRACERS), d["entu"], d["detu"], d["entd"], d["detd"], d["dkg"],
                     d["cloud_top"], d["cloud_lfs"], cols, 1800.0, lmax, cache=cache)  # fmt: skip
        dev.sync()
    finally:
        dev.tune(lu_lanes=saved)
    assert dev.launches() - before == 14  # two calls of seven launches
    tags = cache[2].host()
    assert (tags == 7).all()
    for k in ("m", *TRACERS):
        assert_bitwise(d[k].host(), want[k], f"convec.{k}")
    for a in (*d.values(), cols, *cache):
        a.free()


def _kzz_inputs(rng, im, jm, lm):
    """Calc_Kzz inputs on a global grid: a warm surface under a stable lapse rate, humidity
    falling with height, heat fluxes of both signs (some columns convective), land and sea."""
    at = 1.0e4 * np.sin(np.linspace(0.0, np.pi, lm + 1))
    bt = np.linspace(1.0, 0.0, lm + 1) ** 2
    sp = rng.uniform(9.5e4, 1.02e5, (im, jm))
    z = np.cumsum(np.full((im, jm, lm), 12000.0 / lm), axis=-1)
    t = 295.0 - 6.5e-3 * z + rng.uniform(-1.0, 1.0, (im, jm, lm))
    q = 1e-2 * np.exp(-z / 2500.0) * rng.uniform(0.5, 1.0, (im, jm, lm))
    pu = rng.uniform(-3e9, 3e9, (im + 1, jm, lm))
    pv = rng.uniform(-1e9, 1e9, (im, jm + 1, lm))
    surface = {"oro": rng.uniform(0.0, 2e4, (im, jm)), "lsm": rng.choice([0.0, 30.0, 100.0], (im, jm)),
               "sr": rng.uniform(1e-4, 0.5, (im, jm)), "srols": rng.uniform(1e-3, 1.0, (im, jm)),
               "u10m": rng.uniform(-8.0, 8.0, (im, jm)), "v10m": rng.uniform(-8.0, 8.0, (im, jm)),
               "sshf": rng.uniform(-200.0, 80.0, (im, jm)), "slhf": rng.uniform(-150.0, 20.0, (im, jm)),
               "ewss": rng.uniform(-0.2, 0.2, (im, jm)), "nsss": rng.uniform(-0.2, 0.2, (im, jm))}  # fmt: skip
    dy = 180.0 / jm
    lat = np.radians(-90.0 + dy * np.arange(jm + 1))
    dxyp = np.radians(360.0 / im) * np.diff(np.sin(lat)) * 6.371e6**2
    return sp * rng.uniform(0.998, 1.002, (im, jm)), sp, pu, pv, t, q, surface, at, bt, dxyp


@pytest.mark.gpu
@pytest.mark.parametrize(("shape", "lmax"), [((120, 90, 34), 34), ((90, 70, 34), 26), ((60, 45, 25), 25)])
def test_calc_kzz_matches_oracle_at_size(dev, shape, lmax):
    """Calc_Kzz over every column of a benchmark-sized region: dkg and pblh bitwise."""
    from oracle import kernels as O

    from pydyn_gb300 import kernels as K
    from pydyn_gb300.device import DevArray

    im, jm, lm = shape
    rng = np.random.default_rng(zlib.crc32(repr(("kzz", shape)).encode()))
    spm, sp, pu, pv, t, q, surface, at, bt, dxyp = _kzz_inputs(rng, im, jm, lm)
    dx, dy = 360.0 / im, 180.0 / jm
    want_dkg, want_pblh = O.calc_kzz(spm, sp, pu, pv, t, q, surface, at, bt, dxyp, lmax, dx, dy, -90.0)
    d = {k: DevArray.from_host(dev, v) for k, v in {"spm": spm, "sp": sp, "pu": pu, "pv": pv, "t": t, "q": q,
                                                    "at": at, "bt": bt, "dxyp": dxyp}.items()}  # fmt: skip
    ds = {k: DevArray.from_host(dev, v) for k, v in surface.items()}
    dkg = DevArray.zeros(dev, (0, im - 1), (0, jm - 1), (0, lmax - 1))
    pblh = DevArray.zeros(dev, (0, im - 1), (0, jm - 1))
    K.calc_kzz(d["spm"], d["sp"], d["pu"], d["pv"], d["t"], d["q"], ds, d["at"], d["bt"], d["dxyp"], lmax, dx, dy,
               -90.0, dkg, pblh)  # fmt: skip
    dev.sync()
    assert_bitwise(dkg.host(), want_dkg, "kzz.dkg")
    assert_bitwise(pblh.host(), want_pblh, "kzz.pblh")
    assert (want_dkg[..., : lmax - 1] > 0.0).mean() > 0.5
    for a in (*d.values(), *ds.values(), dkg, pblh):
        a.free()


@pytest.mark.gpu
@pytest.mark.parametrize(("shape", "ns", "ntrop"), [((120, 90, 34, 2), 30, 10), ((90, 70, 34, 1), 18, 6)])
def test_chemistry_and_sources_on_owned_columns_at_size(dev, shape, ns, ntrop):
    """The fused chemistry (rates, decay, applied to tracer 1's mass and slopes) and the
    emission on the owned columns of a benchmark-sized region (a 30 x 35 block not owned, as a
    child's footprint), against the oracle's rates and NumPy's q * decay and rm + x."""
    from make_golden import chem_inputs
    from oracle import kernels as O

    from pydyn_gb300 import kernels as K
    from pydyn_gb300.device import DevArray

    im, jm, lm, nt = shape
    rng = np.random.default_rng(zlib.crc32(repr(("chem", shape)).encode()))
    st, _ = _state(rng, im, jm, lm, nt, 0.5)
    ins = chem_inputs(rng, im, jm, lm, ns, ntrop)
    fac = rng.uniform(0.2, 1.0, im)
    flux = 1e-10 * rng.uniform(0.1, 3.0, (im, jm))
    area = rng.uniform(1e9, 1e11, jm)
    own = np.ones((im, jm), dtype=bool)
    own[13:43, 50:85] = False
    cols = np.argwhere(own).astype(np.int32)
    kw = {"oh_scale": 0.901, "cl_scale": 1.0, "o1d_scale": 1.0, "soil_rate": 2e-4}
    _, decay = O.loss_rates(ins["temper"], ins["phlb"], ins["lat"], ins["strat_press"], ins["strat_oh"],
                            ins["strat_cl"], ins["strat_od"], ins["oh_3d"], pl_trop=ins["pl_trop"],
                            cl_trop=ins["cl_trop"], soil=ins["soil"], dt=1800.0, oh_factor=fac, **kw)  # fmt: skip
    want = {k: v.copy() for k, v in st.items()}
    x = flux * area[None, :] * 1800.0
    want["rm"][..., 0, 0][own] = want["rm"][..., 0, 0][own] + x[own]
    want["rzm"][..., 0, 0][own] = want["rzm"][..., 0, 0][own] - x[own]
    for q in TRACERS:
        want[q][..., 0][own] = want[q][..., 0][own] * decay[own]
    d = {k: DevArray.from_host(dev, v) for k, v in {**st, **ins, "fac": fac, "flux": flux, "area": area}.items()}
    dcols = DevArray.from_host(dev, cols)
    krates = DevArray.zeros(dev, (0, im - 1), (0, jm - 1), (0, lm - 1), (0, 1))
    K.chem_krates(d["temper"], krates, dcols)  # the step's rate constants, made once
    K.sources(d["rm"], d["rzm"], d["flux"], dcols, 1, 1, area=d["area"], scale=1800.0)
    K.chemistry(d["temper"], d["phlb"], d["lat"], d, 1800.0, dcols, (1,), *(d[q] for q in TRACERS),
                oh_factor=d["fac"], krates=krates, **kw)  # fmt: skip
    dev.sync()
    krates.free()
    for k in ("m", *TRACERS):
        assert_bitwise(d[k].host(), want[k], f"chem.{k}")
    assert (decay < 1.0).mean() > 0.5
    for a in (*d.values(), dcols):
        a.free()


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(120, 90, 34, 1), (60, 45, 25, 2), (90, 70, 34, 1)])
@pytest.mark.parametrize("cfl", [0.3, 1.6])
@pytest.mark.parametrize("op", ["x", "y", "z", "xred"])
def test_device_matches_oracle_at_size(dev, shape, cfl, op):
    im, jm, lm, nt = shape
    rng = np.random.default_rng(zlib.crc32(repr((shape, cfl, op)).encode()))
    st, fluxes = _state(rng, im, jm, lm, nt, cfl)
    flux = fluxes["xyz".index(op[0])]
    ins = {**st, "flux": flux}
    if op == "xred":  # production-like bands: whole-row, coarse and fine clusters at both poles
        bands = {120: (40, 8, 4, 2), 60: (60, 20, 10, 5), 90: (30, 9, 3, 2)}[im]
        clust = np.ones(jm, dtype=np.int32)
        for k, c in enumerate(bands):
            clust[k] = clust[jm - 1 - k] = c
        ins["clust"] = clust
    meta = {"op": op}
    want, werr = run_oracle(ins, meta)
    got, gerr = run_device(dev, ins, meta)
    assert gerr == werr
    for k in ("m", *TRACERS, "flux") if werr is None else ():
        assert_bitwise(got[k], want[k], f"{op}.{k}")
