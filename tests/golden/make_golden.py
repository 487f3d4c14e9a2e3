"""Make the golden fixtures of tests/golden/ from the reference itself.

Run where the pydyn reference is importable, with PYDYN_REFERENCE set to its checkout (the
directory holding the `pydyn` package); the fixtures it writes are what the tests compare the oracle and the device
against on machines that do not have the reference:

    python tests/golden/make_golden.py kernels     -> tests/golden/kernels.npz
    python tests/golden/make_golden.py adjoint     -> tests/golden/adjoint.npz
    python tests/golden/make_golden.py balance     -> tests/golden/balance.npz
    python tests/golden/make_golden.py dumps       -> tests/golden/dumps.json

kernels.npz holds, per case, the inputs pydyn.synth makes and the outputs of the reference
function on them (pydyn.kernels, pydyn.redgrid, pydyn.cfl, pydyn.balance): keys
"<case>.in.<name>", "<case>.out.<name>", and "<case>.meta" (a JSON string).  The cases are
the reference's own test shapes (tests/test_gpu.py: IM, JM, LM, NT = 12, 9, 7, 3 at Courant
numbers 0.4, 1.3, 3.2; tests/common.py: the 12 x 6 x 5 reduced grid)."""

import json
import os
import sys
from pathlib import Path

import numpy as np

REF = Path(os.environ["PYDYN_REFERENCE"]) if os.environ.get("PYDYN_REFERENCE") else None
HERE = Path(__file__).resolve().parent


def _reference():
    if REF is None:
        raise SystemExit("make_golden: set PYDYN_REFERENCE to the pydyn reference checkout")
    sys.path.insert(0, str(REF))
    import pydyn  # noqa: F401

    return pydyn


def _gbmath():
    """libgbmath.so (built here if needed): the exp / log / pow / cos the device computes."""
    sys.path.insert(0, str(HERE.parents[1]))
    from pydyn_gb300.build import build

    return build()[1]


def chem_inputs(rng, im, jm, lm, ns, ntrop):
    """Inputs of chem.loss_rates on a global grid: half levels of a surface pressure falling as
    sigma**1.5, zonal columns on descending pressures (some below the surface), a tropospheric
    Cl column on descending pressures, temperatures 200-300 K, OH 1e5-3e6."""
    sp = rng.uniform(9e4, 1.02e5, (im, jm))
    phlb = sp[..., None] * np.linspace(1.0, 0.0, lm + 1)[None, None] ** 1.5
    press = np.sort(rng.uniform(0.5, 1000.0, (jm, ns)), axis=1)[:, ::-1]  # hPa
    pl = np.sort(rng.uniform(1e4, 1e5, (im, jm, ntrop)), axis=-1)[..., ::-1]
    return {
        "temper": rng.uniform(200.0, 300.0, (im, jm, lm)), "phlb": phlb,
        "lat": np.radians(-90 + 180.0 / jm * (np.arange(jm) + 0.5)), "strat_press": press,
        "strat_oh": rng.uniform(1e-9, 1e-7, (jm, ns)), "strat_cl": rng.uniform(1e-9, 1e-7, (jm, ns)),
        "strat_od": rng.uniform(1e-9, 1e-7, (jm, ns)), "oh_3d": rng.uniform(1e5, 3e6, (im, jm, lm)),
        "pl_trop": np.ascontiguousarray(pl), "cl_trop": rng.uniform(0, 1e3, (im, jm, ntrop)),
        "soil": rng.uniform(0, 1, (im, jm)),
    }  # fmt: skip


def kernel_cases():
    _reference()
    from pydyn import balance, cfl, kernels, redgrid, synth

    cases = {}

    def put(name, inputs, outputs, **meta):
        cases[name] = (inputs, outputs, meta)

    IM, JM, LM, NT = 12, 9, 7, 3
    for cfl_ in (0.4, 1.3, 3.2):
        rng = np.random.default_rng(int(cfl_ * 10))
        s = synth.state(rng, IM, JM, LM, NT)
        fl = synth.fluxes(rng, s.m, cfl=cfl_)
        for axis, fn in enumerate((kernels.advect_x, kernels.advect_y, kernels.advect_z)):
            name = f"{'xyz'[axis]}{round(cfl_ * 10):02d}"
            flux = fl[axis].copy()
            ins = {"m": s.m, "rm": s.rm, "rxm": s.rxm, "rym": s.rym, "rzm": s.rzm, "flux": flux.copy()}
            st = s.copy()
            try:
                stats = {}
                fn(st.m, st.rm, st.rxm, st.rym, st.rzm, flux, stats=stats)
                outs = {"m": st.m, "rm": st.rm, "rxm": st.rxm, "rym": st.rym, "rzm": st.rzm, "flux": flux}
                put(name, ins, outs, op="xyz"[axis], error=None, nloop_max=int(stats["nloop_max"]))
            except kernels.CFLError as e:
                put(name, ins, {}, op="xyz"[axis], error="CFLError", message=str(e))

    # the reduced grid (tests/common.py small_redgrid)
    IM, JM, LM, NT = 12, 6, 5, 2
    g = redgrid.RedGrid(IM, JM, jred=(1, 2, JM), clustsize=(IM, 4, 3))
    clust = np.ones(JM, dtype=np.int32)
    for j, c, _ in g.bands:
        clust[j] = c
    for k, cfl_ in enumerate((0.6, 1.7, 4.0)):
        rng = np.random.default_rng(40 + k)
        s = synth.state(rng, IM, JM, LM, NT)
        am = synth.fluxes(rng, s.m, cfl=cfl_)[0]
        st, a = s.copy(), am.copy()
        redgrid.advect_x_reduced(st.m, st.rm, st.rxm, st.rym, st.rzm, a, g)
        ins = {"m": s.m, "rm": s.rm, "rxm": s.rxm, "rym": s.rym, "rzm": s.rzm, "flux": am, "clust": clust}
        tag = f"{round(cfl_ * 10):02d}"
        put(f"xred{tag}", ins, {"m": st.m, "rm": st.rm, "rxm": st.rxm, "rym": st.rym, "rzm": st.rzm, "flux": a},
            op="xred", error=None)
        # Check_CFL's mass-only kernels on the same inputs
        m1, a1 = s.m.copy(), am.copy()
        r = cfl.dynamum(m1, a1, g)
        put(f"cflx{tag}", {"m": s.m, "flux": am, "clust": clust}, {"m": m1, "flux": a1} if r else {},
            op="cflx", error=None if r else "fail")
        bm = synth.fluxes(rng, s.m, cfl=cfl_)[1]
        m2, b2 = s.m.copy(), bm.copy()
        r = cfl.dynamvm(m2, b2)
        put(f"cfly{tag}", {"m": s.m, "flux": bm}, {"m": m2, "flux": b2} if r else {}, op="cfly",
            error=None if r else "fail")
        cm = synth.fluxes(rng, s.m, cfl=cfl_)[2]
        m3, c3 = s.m.copy(), cm.copy()
        r = cfl.dynamwm(m3, c3)
        put(f"cflz{tag}", {"m": s.m, "flux": cm}, {"m": m3, "flux": c3} if r else {}, op="cflz",
            error=None if r else "fail")

    # convection with diffusion (kernels.convec, the Crout inverse), the reference test's variants
    for k, kw in enumerate(({}, {"lfs_above_top": True}, {"strong_detu": True}, {"top_max": 3})):
        rng = np.random.default_rng(60 + k)
        lmax = 10
        s = synth.state(rng, 8, 6, 12, 2)
        conv = synth.convection(rng, s.m, lmax, 1800.0, **kw)
        st = s.copy()
        kernels.convec(st.m, st.rm, st.rxm, st.rym, st.rzm, **conv, dt=1800.0, lmax=lmax)
        ins = {"m": s.m, "rm": s.rm, "rxm": s.rxm, "rym": s.rym, "rzm": s.rzm, **conv}
        put(f"convec{k}", ins, {"m": st.m, "rm": st.rm, "rxm": st.rxm, "rym": st.rym, "rzm": st.rzm}, op="convec",
            lmax=lmax, dt=1800.0)

    # Calc_Kzz (diffusion.calc_kzz on pydyn.synth.kzz_inputs), pydyn's libm routed through the
    # package's gbmath so that the fixtures hold the bits the device must reproduce
    from pydyn import diffusion, ops

    ops.use_libm(str(_gbmath()))
    for k, (im, jm, lm, lmax, spm_scale) in enumerate(((12, 9, 8, 6, None), (16, 10, 34, 26, 1.003),
                                                      (12, 9, 8, 8, 0.998), (10, 6, 25, 25, None))):  # fmt: skip
        rng = np.random.default_rng(80 + k)
        args, grid = synth.kzz_inputs(rng, im, jm, lm, lmax)
        args = list(args)
        if spm_scale is not None:  # spm (the step's middle) apart from sp (its start)
            args[0] = args[1] * spm_scale
        dkg, parts = diffusion.calc_kzz(*args, **grid)
        spm, sp, pu, pv, t, q, surface, at, bt, dxyp, _ = args
        ins = {"spm": spm, "sp": sp, "pu": pu, "pv": pv, "t": t, "q": q, "at": at, "bt": bt, "dxyp": dxyp,
               **{f"surface.{name}": surface[name] for name in surface}}  # fmt: skip
        put(f"kzz{k}", ins, {"dkg": dkg, "pblh": parts["pblh"]}, op="kzz", lmax=lmax, **grid)

    # CH4 loss rates and decay (chem.loss_rates, chem.decay), pydyn's libm routed as above
    from pydyn import chem

    for k, (im, jm, lm, ns, ntrop, sinks, factor) in enumerate((
            (10, 8, 20, 12, 5, ("trop", "soil"), False), (10, 8, 20, 12, 5, ("soil",), False),
            (9, 7, 34, 30, 8, ("trop",), True), (12, 6, 34, 18, 12, ("trop", "soil"), True))):  # fmt: skip
        rng = np.random.default_rng(90 + k)
        ins = chem_inputs(rng, im, jm, lm, ns, ntrop)
        kw = {"oh_scale": 0.901, "cl_scale": 1.1, "o1d_scale": 1.0}
        if "trop" in sinks:
            kw.update(pl_trop=ins["pl_trop"], cl_trop=ins["cl_trop"])
        if "soil" in sinks:
            kw.update(soil=ins["soil"], soil_rate=2e-4)
        oh = ins["oh_3d"]
        if factor:  # the benchmark's diurnal cycle: a per-longitude multiplier of oh_3d
            ins["oh_factor"] = rng.uniform(0.2, 1.0, im)
            oh = oh * ins["oh_factor"][:, None, None]
        base = {n: ins[n] for n in ("temper", "phlb", "lat", "strat_press", "strat_oh", "strat_cl", "strat_od")}
        loss = chem.loss_rates(**base, oh_3d=oh, **kw)
        decay = chem.decay(loss, 1800.0)
        keep = {n: v for n, v in ins.items() if n in (*base, "oh_3d", "oh_factor", *kw)}
        put(f"chem{k}", keep, {"loss": loss, "decay": decay}, op="chem", dt=1800.0,
            **{n: v for n, v in kw.items() if isinstance(v, float)})

    # dynam0 and m2phlb1
    rng = np.random.default_rng(7)
    IM, JM, LM = 10, 8, 6
    pu = rng.normal(0.0, 1e9, (IM + 1, JM, LM))
    pv = rng.normal(0.0, 1e9, (IM, JM + 1, LM))
    bt = np.concatenate([[1.0], np.sort(rng.uniform(0, 1, LM - 1))[::-1], [0.0]])
    am, bm, cm = kernels.fluxes_from_meteo(pu, pv, bt, 900.0)
    put("fluxes", {"pu": pu, "pv": pv, "bt": bt}, {"am": am, "bm": bm, "cm": cm}, op="fluxes", dt=900.0)
    m = 1e9 * rng.uniform(0.8, 1.2, (IM, JM, LM))
    at = np.linspace(2000.0, 0.0, LM + 1)
    dxyp = 1e10 * rng.uniform(0.5, 1.5, JM)
    sp, phlb = balance.m2phlb1(m, at, bt, dxyp)
    put("m2phlb1", {"m": m, "at": at, "bt": bt, "dxyp": dxyp}, {"sp": sp, "phlb": phlb}, op="m2phlb1")
    return cases


def balance_inputs(rng, im, jm, lm, periodic=True, noise=3e-7):
    """Meteo_Setup_Mass inputs near balance: fluxes ~1e9 kg/s (x faces periodic and pole faces
    closed on a global grid), no vertical flux, level weights |db| summing to 1, and an sp2 whose
    tendency is the column convergence's up to a relative `noise`, so that the pre-check passes
    and the tight check asks for the Poisson correction."""
    GRAV = 9.80665
    area = 1.0e10 * (0.5 + rng.random(jm))
    db = rng.random(lm) + 0.2
    db = -(db / db.sum())
    pu = 1.0e9 * rng.standard_normal((im + 1, jm, lm))
    pv = 1.0e9 * rng.standard_normal((im, jm + 1, lm))
    if periodic:
        pu[im] = pu[0]
        pv[:, 0] = 0.0
        pv[:, jm] = 0.0
    pw = np.zeros((im, jm, lm + 1))
    sp1 = 1.0e5 * (1.0 + 0.01 * rng.standard_normal((im, jm)))
    dt = 10800.0
    su, sv = pu.sum(axis=2), pv.sum(axis=2)
    conv = su[:-1] - su[1:] + sv[:, :-1] - sv[:, 1:]
    sp2 = sp1 + dt * conv * GRAV / area[None, :] * (1.0 + noise * rng.standard_normal((im, jm)))
    return {"pu": pu, "pv": pv, "pw": pw, "sp1": sp1, "sp2": sp2, "levi_db": db, "area": area, "dt": dt}


def balance_cases():
    """pydyn's Meteo_Setup_Mass balancing on such inputs, with NumPy's FFT (balance.NumpyPoisson):
    region 1 (balance.setup_mass) and a child at 3 x 2 under a 10 x 8 parent
    (zoom_meteo.setup_mass_child with PoissonDirect)."""
    _reference()
    import types

    # pydyn.zoom_meteo imports pydyn.meteo, which imports netCDF4 for its archive reader; the
    # balancing functions read no file, so a stand-in module lets them import here
    sys.modules.setdefault("netCDF4", types.SimpleNamespace(Dataset=None))
    from pydyn import balance
    from pydyn import zoom_meteo as ZM

    cases = {}
    for k, (im, jm, lm) in enumerate(((24, 18, 5), (36, 20, 8))):
        rng = np.random.default_rng(300 + k)
        ins = balance_inputs(rng, im, jm, lm)
        pu, pv = ins["pu"].copy(), ins["pv"].copy()
        info = balance.setup_mass(pu, pv, ins["pw"], ins["sp1"], ins["sp2"], ins["levi_db"], ins["area"],
                                  ins["dt"], solver=balance.NumpyPoisson(im, jm))  # fmt: skip
        cases[f"balance{k}"] = ({n: v for n, v in ins.items() if n != "dt"}, {"pu": pu, "pv": pv},
                                {"op": "balance", "dt": ins["dt"], "tries": info["tries"], "ok": bool(info["ok"])})
    # a child: parent 10 x 8 (balanced), child under parent cells i 3..6, j 2..5 at 3 x 2
    rng = np.random.default_rng(320)
    imp, jmp, lm = 10, 8, 4
    rf = ZM.Refinement(3, 2, 3, 6, 2, 5)
    parent = balance_inputs(rng, imp, jmp, lm)
    ppw = 1.0e7 * rng.standard_normal((imp, jmp, lm + 1))
    im, jm = 4 * 3, 4 * 2
    raw = (1.0e9 / 3 * rng.standard_normal((im + 1, jm, lm)), 1.0e9 / 2 * rng.standard_normal((im, jm + 1, lm)),
           1.0e7 / 6 * rng.standard_normal((im, jm, lm + 1)))  # fmt: skip
    area = 1.0e9 * (0.5 + rng.random(jm))
    db = rng.random(lm) + 0.2
    db = -(db / db.sum())
    # the child's surface pressures follow its matched fluxes' column convergence
    mpu, mpv, mpw = (q.copy() for q in raw)
    ZM.match_u_sum(parent["pu"], mpu, rf)
    ZM.match_v_sum(parent["pv"], mpv, rf)
    su, sv = mpu.sum(axis=2), mpv.sum(axis=2)
    sp1 = 1.0e5 * (1.0 + 0.01 * rng.standard_normal((im, jm)))
    sp2 = sp1 + 10800.0 * (su[:-1] - su[1:] + sv[:, :-1] - sv[:, 1:]) * 9.80665 / area[None, :] * (
        1.0 + 3e-7 * rng.standard_normal((im, jm)))  # fmt: skip
    from pydyn import balance

    poisson = ZM.PoissonDirect(3, 2, solver=balance.NumpyPoisson(3, 2))
    pu, pv, pw, info = ZM.setup_mass_child(raw, (parent["pu"], parent["pv"], ppw), sp1, sp2, db, area, 10800.0, rf,
                                           poisson)  # fmt: skip
    ins = {"pu": raw[0], "pv": raw[1], "pw": raw[2], "ppu": parent["pu"], "ppv": parent["pv"], "ppw": ppw,
           "sp1": sp1, "sp2": sp2, "levi_db": db, "area": area, "m_to_u": poisson.m_to_u, "m_to_v": poisson.m_to_v}
    cases["balchild0"] = (ins, {"pu": pu, "pv": pv, "pw": pw},
                          {"op": "balchild", "dt": 10800.0, "rf": [3, 2, 3, 6, 2, 5], "tries": info["tries"],
                           "ok": bool(info["ok"])})  # fmt: skip
    return cases


STATE_FIELDS = ("m", "rm", "rxm", "rym", "rzm", "am", "bm", "cm", "pu", "pv", "sp", "phlb")


def digest(fields_by_region):
    """sha1 over every state array of every region (bit patterns, fixed order)."""
    import hashlib

    h = hashlib.sha1()
    for r in sorted(fields_by_region):
        for name in STATE_FIELDS:
            h.update(np.ascontiguousarray(fields_by_region[r][name], dtype="<f8").tobytes())
    return h.hexdigest()


class _RefPhysics:
    """The physics of a step composed from pydyn itself, as pydyn forward.py:411-451 composes it
    for one region, for every region of the tree: diffusion.calc_kzz after Setup_MassFlow (spm the
    meteo's at the step's middle, sp the region's at its start), zoom.physics' convec_region,
    sources_region and chemistry_region on chem.loss_rates / chem.decay, dt = ndyn / (2 tref)
    per region, OH times the diurnal factor of the region's half step.  pydyn's libm is routed
    through the package's gbmath."""

    def __init__(self, zref, spec, fields):
        from pydyn import ops

        ops.use_libm(str(_gbmath()))
        self.zref, self.spec, self.dxyp = zref, spec, {r: fields[r]["dxyp"] for r in fields}

    def init(self, st):
        for r in self.zref.regions():
            if r == 1:
                st.lib.m2phlb1(self.zref, st, 1)
            else:
                st.lib.m2phlb(self.zref, st, r)

    def step(self, st, t0, ndyn):
        from pydyn import chem, diffusion
        from pydyn import zoom as Z

        from pydyn_gb300 import synth

        spec, zref = self.spec, self.zref
        if spec.kind == "convection":  # pydyn's own GPU benchmark's physics: convection on a given dkg
            return {r: {**spec.region[r]["conv"], "dkg": spec.region[r]["dkg"], "lmax": spec.lmax}
                    for r in zref.regions()}, {}  # fmt: skip
        a1, a2 = synth.weights(t0 + ndyn / 2.0)
        conv = {}
        for r in zref.regions():
            g, R = zref.g(r), spec.region[r]
            k = R["kzz"]
            spm = a1 * k["spm"][0] + a2 * k["spm"][1]
            sp = st[r]["sp"][1 : g.im, 1 : g.jm, 1]
            dx, dy = (g.xend - g.xbeg) / g.im, (g.yend - g.ybeg) / g.jm
            dkg, _ = diffusion.calc_kzz(spm, sp, st[r]["pu"].data, st[r]["pv"].data, k["t"], k["q"], k["surface"],
                                        zref.at, zref.bt, self.dxyp[r], spec.lmax, dx=dx, dy=dy, ybeg=float(g.ybeg))  # fmt: skip
            conv[r] = {**R["conv"], "dkg": dkg, "lmax": spec.lmax}

        def sources(zoom, s, region):
            x = spec.region[region]["flux"] * self.dxyp[region][None, :] * spec.half_step(region, ndyn)
            s.lib.sources_region(zoom, s, region, [(x, 1, 1)])

        def chemistry(zoom, s, region):
            g, R = zoom.g(region), spec.region[region]
            c = R["chem"]
            fac = spec.factors(region, t0, ndyn)[zoom.status[region] // 6]
            phlb = s[region]["phlb"][1 : g.im, 1 : g.jm, 1 : zoom.lm + 1]
            loss = chem.loss_rates(R["kzz"]["t"], phlb, c["lat"], c["strat_press"], c["strat_oh"], c["strat_cl"],
                                   c["strat_od"], c["oh_3d"] * fac[:, None, None], pl_trop=c["pl_trop"],
                                   cl_trop=c["cl_trop"], soil=c["soil"], **spec.settings)  # fmt: skip
            decay = chem.decay(loss, spec.half_step(region, ndyn))
            s.lib.chemistry_region(zoom, s, region, decay[Z.scope(zoom, region)], (1,))

        return conv, {"sources": sources, "chemistry": chemistry}


def _reference_case(config, lm, seed, nt=1, physics=False, umax=40.0, lmax=None):
    """pydyn's Zoom, states and meteo for the synthetic case of pydyn_gb300.synth, and an
    interval runner: (zref, st, cst, phys, run_interval(t0, limits) -> (ndyn, n))."""
    _reference()
    sys.path.insert(0, str(HERE.parents[1]))
    from pydyn import redgrid as RG
    from pydyn import zoom as Z

    from pydyn_gb300 import synth

    zoom, met, fields = synth.case(config, lm, seed, nt, umax=umax)
    regions = []
    for g in zoom.region[1:]:
        kw = {k: getattr(g, k) for k in g._fields if k != "redgrid"}
        rg = None
        if g.redgrid is not None:
            rg = RG.RedGrid(g.im, g.jm, [b[0] + 1 for b in g.redgrid.bands], [b[1] for b in g.redgrid.bands])
        regions.append(Z.Region(**kw, redgrid=rg))
    zref = Z.Zoom(regions, lm, zoom.at, zoom.bt)
    st, cst = Z.ZoomState.zeros(zref, nt), Z.ZoomState.zeros(zref, nt)
    for r, f in fields.items():
        for name, a in f.items():
            st[r][name].data[...] = a
        cst[r]["dxyp"].data[...] = f["dxyp"]
    meteo = {r: [met.fluxes(r, k) for k in (0, 1)] for r in zref.regions()}

    def interp(s, t):
        a1, a2 = synth.weights(t)
        for r in zref.regions():
            (pu0, pv0), (pu1, pv1) = meteo[r]
            s[r]["pu"].data[...] = a1 * pu0 + a2 * pu1
            s[r]["pv"].data[...] = a1 * pv0 + a2 * pv1

    phys = None
    if physics:
        phys = _RefPhysics(zref, synth.Physics(zoom, met, seed, lm if lmax is None else lmax), fields)
        phys.init(st)

    def run_interval(t0, limits=True):
        for r in zref.regions():
            for name in ("m", "sp"):
                cst[r][name].data[...] = st[r][name].data
        ndyn, n, _ = Z.check_cfl_zoom(zref, cst, 3600, 1, 3600, lambda z, s, i, nd: interp(s, t0 + (i - 0.5) * nd))
        for k in range(n):
            interp(st, t0 + k * ndyn + ndyn / 2.0)
            Z.setup_massflow(zref, st, ndyn)
            kw = {}
            if phys is not None:
                conv, kw = phys.step(st, t0 + k * ndyn, ndyn)
            else:
                conv = {r: _no_convection(zref, r) for r in zref.regions()}
            Z.step(zref, st, conv, ndyn, limits=limits, inverse="crout", **kw)
        return ndyn, n

    return zref, st, cst, phys, run_interval


ADJOINT_CASE = {"config": "one", "lm": 4, "seed": 23, "lmax": 4}


def adjoint_goldens(nbasis=None, ny=2, seed=5):
    """The transposed reference operator on the `one` tree: pydyn's own interval (Check_CFL,
    Setup_MassFlow, Calc_Kzz, xyzvsc|csvzyx with convection, emission at zero flux and chemistry,
    limits off) is linear in the tracer moments; it is applied to every basis vector e_j of the
    interior (rm, rxm, rym, rzm) (or `nbasis` sampled ones) and dotted with `ny` seeded vectors
    y_k, which gives (A^T y_k)_j.  Also A delta for one seeded delta (the forward's own check)."""
    c = ADJOINT_CASE
    zref, st, _, phys, run_interval = _reference_case(c["config"], c["lm"], c["seed"], physics=True, lmax=c["lmax"])
    for r in zref.regions():
        phys.spec.region[r]["flux"][...] = 0.0
    g, lm = zref.g(1), c["lm"]
    names = ("rm", "rxm", "rym", "rzm")
    start = {k: v.data.copy() for k, v in st[1].items()}

    def apply(vec):
        for k, v in start.items():
            st[1][k].data[...] = v
        for w, name in enumerate(names):
            st[1][name].data[2 : g.im + 2, 2 : g.jm + 2, :, 0] = vec[w]
        run_interval(0.0, limits=False)
        return np.stack([st[1][name].data[2 : g.im + 2, 2 : g.jm + 2, :, 0].copy() for name in names])

    rng = np.random.default_rng([seed, 31337])
    shape = (4, g.im, g.jm, lm)
    ys = rng.random((ny, *shape)) + 0.5
    delta = rng.random(shape) * np.array([1.0, 0.3, 0.3, 0.3])[:, None, None, None]
    a_delta = apply(delta)
    size = int(np.prod(shape))
    idx = np.arange(size) if nbasis is None else np.sort(rng.choice(size, size=nbasis, replace=False))
    vals = np.zeros((ny, idx.size))
    for n, j in enumerate(idx):
        e = np.zeros(shape)
        e.flat[j] = 1.0
        out = apply(e)
        vals[:, n] = [float(np.dot(out.ravel(), y.ravel())) for y in ys]
    return {"adjoint": ({"y": ys, "delta": delta, "index": idx}, {"ATy": vals, "A_delta": a_delta}, dict(c))}


def reference_run(config, lm, seed, nsteps, nt=1, physics=False, keep=None, umax=40.0, lmax=None, kind="full"):
    """pydyn's own driver (zoom.check_cfl_zoom on a copy of m and sp, then setup_massflow and
    zoom.step, as pydyn forward.py:388-451 runs an interval of one step) on the synthetic case
    of pydyn_gb300.synth.  Returns [(ndyn, n, digest)] per interval; keep: a list that receives
    the full host state after each interval."""
    _reference()
    sys.path.insert(0, str(HERE.parents[1]))
    from pydyn import redgrid as RG
    from pydyn import zoom as Z

    from pydyn_gb300 import synth

    zoom, met, fields = synth.case(config, lm, seed, nt, umax=umax)
    regions = []
    for g in zoom.region[1:]:
        kw = {k: getattr(g, k) for k in g._fields if k != "redgrid"}
        rg = None
        if g.redgrid is not None:
            rg = RG.RedGrid(g.im, g.jm, [b[0] + 1 for b in g.redgrid.bands], [b[1] for b in g.redgrid.bands])
        regions.append(Z.Region(**kw, redgrid=rg))
    zref = Z.Zoom(regions, lm, zoom.at, zoom.bt)
    st, cst = Z.ZoomState.zeros(zref, nt), Z.ZoomState.zeros(zref, nt)
    for r, f in fields.items():
        for name, a in f.items():
            st[r][name].data[...] = a
        cst[r]["dxyp"].data[...] = f["dxyp"]
    meteo = {r: [met.fluxes(r, k) for k in (0, 1)] for r in zref.regions()}

    def interp(s, t):
        a1, a2 = synth.weights(t)
        for r in zref.regions():
            (pu0, pv0), (pu1, pv1) = meteo[r]
            s[r]["pu"].data[...] = a1 * pu0 + a2 * pu1
            s[r]["pv"].data[...] = a1 * pv0 + a2 * pv1

    phys = None
    if physics:
        phys = _RefPhysics(zref, synth.Physics(zoom, met, seed, lm if lmax is None else lmax, kind=kind), fields)
        phys.init(st)
    out, t = [], 0.0
    for _ in range(nsteps):
        for r in zref.regions():
            for name in ("m", "sp"):
                cst[r][name].data[...] = st[r][name].data
        t0 = t
        ndyn, n, _ = Z.check_cfl_zoom(zref, cst, 3600, 1, 3600, lambda z, s, i, nd: interp(s, t0 + (i - 0.5) * nd))
        for k in range(n):
            interp(st, t0 + k * ndyn + ndyn / 2.0)
            Z.setup_massflow(zref, st, ndyn)
            kw = {}
            if phys is not None:
                conv, kw = phys.step(st, t0 + k * ndyn, ndyn)
            else:
                conv = {r: _no_convection(zref, r) for r in zref.regions()}
            Z.step(zref, st, conv, ndyn, limits=True, inverse="crout", **kw)
        t = t0 + 3600.0
        host = {r: {name: st[r][name].data for name in STATE_FIELDS} for r in zref.regions()}
        out.append((ndyn, n, digest(host)))
        if keep is not None:
            keep.append({r: {k: v.copy() for k, v in f.items()} for r, f in host.items()})
    return out


def _no_convection(zoom, r):
    """convection over no level: the `v` operator of an advection-only run is then a no-op."""
    g = zoom.g(r)
    z = np.zeros((g.im, g.jm, 0))
    c = np.zeros((g.im, g.jm), dtype=np.int32)
    return {"entu": z, "detu": z, "entd": z, "detd": z, "dkg": z, "cloud_top": c, "cloud_lfs": c, "lmax": 0}


STEP_RUNS = {  # name: (tree, lm, seed, intervals, umax[, physics lmax, intervals the CPU tests run][, options])
    "config0": ("glb6x4", 25, 11, 24, 40.0),
    "config0-strong": ("glb6x4", 25, 12, 6, 160.0),
    "two": ("two", 5, 13, 6, 40.0),
    "two-strong": ("two", 5, 14, 6, 120.0),
    "two-reject": ("two", 5, 14, 4, 1000.0),  # Check_CFL halves ndyn on the child's tree
    "three": ("three", 4, 15, 4, 40.0),
    "config2-adv": ("glb3x2+nam1x1", 34, 31, 3, 40.0),
    "two-phys": ("two", 8, 21, 6, 40.0, 8, 6),
    "three-phys": ("three", 6, 22, 4, 40.0, 6, 4),
    "config1": ("glb3x2", 34, 41, 24, 40.0, 34, 1),  # one simulated day
    "config2": ("glb3x2+nam1x1", 34, 42, 168, 40.0, 34, 1),  # one simulated week
    "two-phys-nt3": ("two", 8, 24, 4, 40.0, 8, 2, {"nt": 3}),
    "config0-nt8": ("glb6x4", 25, 16, 3, 40.0, {"nt": 8}),
    "config1-nt12": ("glb3x2", 34, 43, 2, 40.0, 34, 1, {"nt": 12}),
    # pydyn's own GPU benchmark case: glb3x2 + a 72 x 44 child, convection over 26 levels on a given dkg
    "a100-case": ("glb3x2+nam72x44", 34, 51, 24, 40.0, 26, 1, {"kind": "convection"}),
}


def step_goldens(names=None):
    import time

    res = {}
    for name, spec in STEP_RUNS.items():
        if names and name not in names:
            continue
        opts = spec[-1] if isinstance(spec[-1], dict) else {}
        spec = spec[:-1] if opts else spec
        config, lm, seed, nsteps, umax = spec[:5]
        lmax = spec[5] if len(spec) > 5 else None
        nt, kind = opts.get("nt", 1), opts.get("kind", "full")
        t = time.perf_counter()
        runs = reference_run(config, lm, seed, nsteps, nt=nt, umax=umax, physics=lmax is not None, lmax=lmax,
                             kind=kind)  # fmt: skip
        res[name] = {"config": config, "lm": lm, "seed": seed, "umax": umax, "steps": [list(x) for x in runs],
                     "reference_seconds_per_interval": (time.perf_counter() - t) / nsteps}  # fmt: skip
        if nt != 1:
            res[name]["nt"] = nt
        if lmax is not None:
            res[name].update(physics=True if kind == "full" else kind, lmax=lmax, cpu_prefix=spec[6])
        print(name, runs[-1], res[name]["reference_seconds_per_interval"])
    return res


# ------------------------------------------------------------------ call traces of pydyn's driver
TRACE_TREES = {  # name: the regions' parameters (pydyn zoom.Region keywords) and lm
    "one": None, "two": None, "three": None, "glb6x4": None, "glb3x2+nam1x1": None, "glb3x2+nam72x44": None,
    "eur": ([{"name": "glb600x400", "im": 60, "jm": 45, "xcyc": 1, "touch_sp": 1, "touch_np": 1},
             {"name": "eur300x200", "im": 30, "jm": 36, "xbeg": -36, "xend": 54, "ybeg": 2, "yend": 74, "xref": 2,
              "yref": 2, "tref": 2, "parent": 1},
             {"name": "eur100x100", "im": 60, "jm": 54, "xbeg": -21, "xend": 39, "ybeg": 12, "yend": 66, "xref": 6,
              "yref": 4, "tref": 4, "parent": 2}], 3),
}  # fmt: skip
TRACE_RUNS = ("config0-strong", "two-reject")  # runs whose Check_CFL rejects steps


def trace_tree_regions(name):
    """(regions as keyword dicts, lm) of a traced tree: pydyn_gb300.synth's trees by name."""
    if TRACE_TREES[name] is not None:
        return TRACE_TREES[name]
    sys.path.insert(0, str(HERE.parents[1]))
    from pydyn_gb300 import synth

    zoom = synth.tree(name, 4)
    return [{k: getattr(g, k) for k in g._fields if k != "redgrid"} for g in zoom.region[1:]], 4


def _json_arg(a):
    if a is None or isinstance(a, (bool, int, float, str)):
        return a
    if isinstance(a, (np.integer,)):
        return int(a)
    if isinstance(a, (np.floating,)):
        return float(a)
    if isinstance(a, dict) and "lmax" in a:
        return "<conv>"
    raise TypeError(f"trace: argument {type(a)} not recorded")


MASS_ONLY = ("_dynamum_region1", "_dynamvm_region1", "_dynamwm", "_dynamum_child", "_dynamvm_child")


class _Trace:
    """A `lib` for pydyn's driver that records every body call as [name, *args after (zoom, st)]
    (save / restore / scale: after st), a kwargs dict last when given, a mass-only body's return
    as {"return": ok}, and for a context-manager body ["enter:<name>", ...] / ["exit:<name>"].
    `inner` (a real lib) does the work when given; else the mass-only bodies answer ok."""

    def __init__(self, inner=None):
        self.calls, self.inner = [], inner

    def __getattr__(self, name):
        inner = getattr(self.inner, name) if self.inner is not None else None
        rec = self

        def row(args, kw, tag):
            first = 1 if name in ("save", "restore", "scale") else 2
            out = [tag, *[[_json_arg(x) for x in a] if isinstance(a, tuple) else _json_arg(a) for a in args[first:]]]
            if kw:
                out.append({k: _json_arg(v) for k, v in kw.items()})
            return out

        if name in ("outer_x_faces_zeroed", "outer_y_faces_zeroed"):
            from contextlib import contextmanager

            @contextmanager
            def cm(*args, **kw):
                rec.calls.append(row(args, kw, "enter:" + name))
                if inner is None:
                    yield
                else:
                    with inner(*args, **kw):
                        yield
                rec.calls.append(["exit:" + name])

            return cm

        def call(*args, **kw):
            out = inner(*args, **kw) if inner is not None else (True if name in MASS_ONLY else None)
            r = row(args, kw, name)
            if name in MASS_ONLY:
                r.append({"return": bool(out)})
            rec.calls.append(r)
            return out

        return call


class _Bare:
    """A state for the recording lib alone: pydyn's driver reads nothing of it but `lib`."""

    def __init__(self, lib):
        self.lib = lib


def plan_traces():
    """pydyn's own driver (zoom.setup_massflow, zoom.step, zoom.check_cfl_zoom) on a recording
    lib, per traced tree: the calls the package's planner must reproduce."""
    _reference()
    from pydyn import zoom as Z

    out = {}
    for name in TRACE_TREES:
        regions, lm = trace_tree_regions(name)
        at, bt = np.linspace(2000.0, 0.0, lm + 1), np.linspace(1.0, 0.0, lm + 1)
        zref = Z.Zoom([Z.Region(**kw) for kw in regions], lm, at, bt)
        conv = {r: {"lmax": lm} for r in zref.regions()}
        res = {"regions": regions, "lm": lm}
        lib = _Trace()
        st = _Bare(lib)
        Z.setup_massflow(zref, st, 3600)
        res["massflow"], lib.calls = lib.calls, []

        def hook(kind):
            return lambda zoom, s, region: lib.calls.append([kind, region, zoom.status[region]])

        Z.step(zref, st, conv, 3600, sources=hook("sources"), chemistry=hook("chemistry"))
        res["step"], lib.calls = lib.calls, []
        Z.check_cfl_zoom(zref, st, 3600, 1, 3600)
        res["check_cfl"] = lib.calls
        out[name] = res
    return out


def run_traces(names=TRACE_RUNS):
    """pydyn's own driver over its real host bodies on the runs whose Check_CFL rejects steps,
    every body call recorded with the mass-only bodies' returns, plus ["interpolate", state,
    t] where the run sets the meteo of a time and ["interval", ndyn, n] at each interval's end:
    the sequence a device module must reproduce call for call."""
    out = {}
    for name in names:
        config, lm, seed, nsteps, umax = STEP_RUNS[name][:5]
        zref, st, cst, _, _ = _reference_case(config, lm, seed, umax=umax)
        from pydyn import zoom as Z

        from pydyn_gb300 import synth

        zoom, met, _ = synth.case(config, lm, seed, 1, umax=umax)
        meteo = {r: [met.fluxes(r, k) for k in (0, 1)] for r in zref.regions()}
        real = st.lib
        lib = _Trace(real)
        st.lib = cst.lib = lib

        def interp(s, t):
            lib.calls.append(["interpolate", "<main>" if s is st else "<cfl>", float(t)])
            a1, a2 = synth.weights(t)
            for r in zref.regions():
                (pu0, pv0), (pu1, pv1) = meteo[r]
                s[r]["pu"].data[...] = a1 * pu0 + a2 * pu1
                s[r]["pv"].data[...] = a1 * pv0 + a2 * pv1

        t = 0.0
        conv = {r: _no_convection(zref, r) for r in zref.regions()}
        for _ in range(nsteps):
            for r in zref.regions():
                for fname in ("m", "sp"):
                    cst[r][fname].data[...] = st[r][fname].data
            lib.calls.append(["copy_m_sp"])
            t0 = t
            ndyn, n, _ = Z.check_cfl_zoom(zref, cst, 3600, 1, 3600, lambda z, s, i, nd: interp(s, t0 + (i - 0.5) * nd))
            for k in range(n):
                interp(st, t0 + k * ndyn + ndyn / 2.0)
                Z.setup_massflow(zref, st, ndyn)
                Z.step(zref, st, conv, ndyn, limits=True, inverse="crout")
            lib.calls.append(["interval", ndyn, n])
            t = t0 + 3600.0
        st.lib = cst.lib = real
        out[name] = lib.calls
    return out


# ------------------------------------------------------------------ dump sets (pydyn.dump, pydyn.replay)
# name: (tree, lm, seed, tracers, ranks, umax) of a synthetic set written by oracle/dumpset.py;
# two-reject's winds make Check_CFL halve the step (two steps of 1800 s in the interval)
DUMP_SETS = {"two": ("two", 5, 3, 1, 1, 40.0), "one": ("one", 5, 4, 1, 1, 40.0), "two-ranks": ("two", 4, 6, 2, 2, 40.0),
             "two-reject": ("two", 5, 14, 1, 1, 1000.0)}
REPLAY_TAGS = ("x", "y", "z", "v", "s", "c", "cfl", "massflow", "m2phlb")


def parse_digest(events):
    """sha1 of a reader's view of a set: every event's identity, header, array bounds and types,
    and its arrays' values (row-major bytes), in sequence order."""
    import hashlib

    h = hashlib.sha1()
    for ev in events:
        meta = {k: list(v) if isinstance(v, tuple) else v for k, v in sorted(ev.meta.items())}
        h.update(json.dumps([ev.tag, ev.seq, ev.region, meta], sort_keys=True).encode())
        for name in sorted(ev.arrays):
            a = ev[name]
            h.update(json.dumps([name, list(a.lower), list(a.data.shape), str(a.data.dtype)]).encode())
            h.update(np.ascontiguousarray(a.data).tobytes())
    return h.hexdigest()


def write_dump_set(name, out):
    sys.path.insert(0, str(HERE.parents[1]))
    from oracle import dumpset

    tree, lm, seed, nt, ranks, umax = DUMP_SETS[name]
    return dumpset.write_set(out, tree, lm=lm, seed=seed, nt=nt, ranks=ranks, umax=umax), dumpset.digest(out)


def dump_goldens():
    """Per set: its sha1, the digest of pydyn's reader's view of it (merged ranks), and what
    pydyn's replay reports event by event -- with the Crout inverse (TM5 built without LAPACK,
    the device's path) and pydyn's libm routed through the package's gbmath."""
    import io
    import tempfile
    import types

    sys.modules.setdefault("netCDF4", types.SimpleNamespace(Dataset=None))  # pydyn.inputs imports it
    _reference()
    from pydyn import dump, ops, replay

    ops.use_libm(str(_gbmath()))
    out = {}
    for name in DUMP_SETS:
        with tempfile.TemporaryDirectory() as d:
            (ndyn, n), sha = write_dump_set(name, d)
            events = dump.load_events(d, merge=True)
            entry = {"sha1": sha, "ndyn": ndyn, "n": n, "events": len(events), "parse": parse_digest(events)}
            res = replay.replay(d, lapack="crout", tags=set(REPLAY_TAGS), out=io.StringIO())
            entry["results"] = [[ev.seq, kind, ev.region, [r["name"] for r in reports],
                                 all(r["equal"] for r in reports)] for ev, kind, reports, _ in res]  # fmt: skip
            entry["failures"] = [list(f) for f in res.failures]
            out[name] = entry
    return out


def save(cases, path):
    flat = {}
    for name, (ins, outs, meta) in cases.items():
        for k, v in ins.items():
            flat[f"{name}.in.{k}"] = np.asarray(v)
        for k, v in outs.items():
            flat[f"{name}.out.{k}"] = np.asarray(v)
        flat[f"{name}.meta"] = np.array(json.dumps(meta))
    np.savez_compressed(path, **flat)


def load(path):
    """{case: (inputs, outputs, meta)} from a fixture file (case names hold no dots)."""
    z = np.load(path)
    cases = {}
    for key in z.files:
        name, kind = key.split(".")[:2]
        slot = cases.setdefault(name, ({}, {}, {}))
        if kind == "meta":
            slot[2].update(json.loads(str(z[key])))
        else:
            slot[0 if kind == "in" else 1][key.split(".", 2)[2]] = z[key]
    return cases


if __name__ == "__main__":
    what = sys.argv[1:] or ["kernels"]
    if "kernels" in what:
        save(kernel_cases(), HERE / "kernels.npz")
        print("wrote", HERE / "kernels.npz")
    if "balance" in what:
        save(balance_cases(), HERE / "balance.npz")
        print("wrote", HERE / "balance.npz")
    if "adjoint" in what:
        save(adjoint_goldens(), HERE / "adjoint.npz")
        print("wrote", HERE / "adjoint.npz")
    if "traces" in what:
        path = HERE / "traces.json"
        path.write_text(json.dumps({"plans": plan_traces(), "runs": run_traces()}) + "\n")
        print("wrote", path)
    if "dumps" in what:
        path = HERE / "dumps.json"
        path.write_text(json.dumps(dump_goldens(), indent=1) + "\n")
        print("wrote", path)
    if "steps" in what:  # `steps [name ...]`: those runs only, the others kept
        path = HERE / "steps.json"
        old = json.loads(path.read_text()) if path.exists() else {}
        old.update(step_goldens([n for n in what if n in STEP_RUNS]))
        path.write_text(json.dumps(old, indent=1) + "\n")
        print("wrote", path)
