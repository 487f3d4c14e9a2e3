"""Run one golden kernel case (tests/golden/kernels.npz) on the oracle or on the device, so the
CPU tests (oracle vs reference fixtures) and the GPU tests (device vs the same fixtures) read the
same way.  Each runner returns ({name: output array}, error) with error None, "CFLError",
"ValueError" or "fail" (a Check_CFL rehearsal that exceeded its cap)."""

import numpy as np

TRACERS = ("rm", "rxm", "rym", "rzm")


def run_oracle(ins, meta):
    from oracle import kernels as O

    op = meta["op"]
    a = {k: np.array(v, dtype=np.float64 if v.dtype.kind == "f" else v.dtype) for k, v in ins.items()}
    try:
        if op in ("x", "y", "z", "xred"):
            q = [a[k] for k in TRACERS]
            if op == "x":
                O.advect_x(a["m"], *q, a["flux"])
            elif op == "xred":
                O.advect_x(a["m"], *q, a["flux"], clust=a["clust"])
            elif op == "y":
                O.advect_y(a["m"], *q, a["flux"])
            else:
                O.advect_z(a["m"], *q, a["flux"])
            return {k: a[k] for k in ("m", *TRACERS, "flux")}, None
        if op == "cflx":
            r = O.advect_x(a["m"], None, None, None, None, a["flux"], clust=a["clust"], max_nloop=10, mass_only=True)
        elif op == "cfly":
            r = O.advect_y(a["m"], None, None, None, None, a["flux"], max_nloop=1, mass_only=True)
        elif op == "cflz":
            r = O.advect_z(a["m"], None, None, None, None, a["flux"], iter_limit=1, mass_only=True)
        elif op == "fluxes":
            pu, pv, bt = a["pu"], a["pv"], a["bt"]
            im, jm, lm = pv.shape[0], pu.shape[1], pu.shape[2]
            am, bm, cm = np.zeros((im + 1, jm, lm)), np.zeros((im, jm + 1, lm)), np.zeros((im, jm, lm + 1))
            O.fluxes_from_meteo(pu, pv, bt, meta["dt"], am, bm, cm)
            return {"am": am, "bm": bm, "cm": cm}, None
        elif op == "m2phlb1":
            m = a["m"]
            sp, phlb = np.zeros(m.shape[:2]), np.zeros((*m.shape[:2], m.shape[2] + 1))
            O.m2phlb(m, sp, phlb, a["dxyp"], a["at"], a["bt"])
            return {"sp": sp, "phlb": phlb}, None
        elif op == "convec":
            q = [a[k] for k in TRACERS]
            O.convec(a["m"], *q, a["entu"], a["detu"], a["entd"], a["detd"], a["cloud_top"], a["cloud_lfs"], a["dkg"],
                     meta["dt"], meta["lmax"])  # fmt: skip
            return {k: a[k] for k in ("m", *TRACERS)}, None
        elif op == "kzz":
            surface = {k: a[f"surface.{k}"] for k in O.KZZ_SURFACE}
            dkg, pblh = O.calc_kzz(a["spm"], a["sp"], a["pu"], a["pv"], a["t"], a["q"], surface, a["at"], a["bt"],
                                   a["dxyp"], meta["lmax"], meta["dx"], meta["dy"], meta["ybeg"])  # fmt: skip
            return {"dkg": dkg, "pblh": pblh}, None
        elif op == "chem":
            kw = {k: meta[k] for k in ("oh_scale", "cl_scale", "o1d_scale", "soil_rate") if k in meta}
            extra = {k: a[k] for k in ("pl_trop", "cl_trop", "soil", "oh_factor") if k in a}
            loss, decay = O.loss_rates(a["temper"], a["phlb"], a["lat"], a["strat_press"], a["strat_oh"], a["strat_cl"],
                                       a["strat_od"], a["oh_3d"], **extra, **kw, dt=meta["dt"])  # fmt: skip
            return {"loss": loss, "decay": decay}, None
        else:
            raise KeyError(op)
        if r is None:
            return {}, "fail"
        return {"m": a["m"], "flux": a["flux"]}, None
    except O.CFLError:
        return {}, "CFLError"
    except ValueError:
        return {}, "ValueError"


def run_device(dev, ins, meta):
    from pydyn_gb300 import _native as N
    from pydyn_gb300 import kernels as K
    from pydyn_gb300.device import DevArray

    op = meta["op"]
    d = {k: DevArray.from_host(dev, np.ascontiguousarray(v)) for k, v in ins.items()}
    try:
        if op in ("x", "y", "z", "xred"):
            q = [d[k] for k in TRACERS]
            if op == "x":
                K.advect_x(d["m"], *q, d["flux"])
            elif op == "xred":
                K.advect_x(d["m"], *q, d["flux"], clust=d["clust"])
            elif op == "y":
                K.advect_y(d["m"], *q, d["flux"])
            else:
                K.advect_z(d["m"], *q, d["flux"])
            dev.sync()
            return {k: d[k].host() for k in ("m", *TRACERS, "flux")}, None
        if op in ("cflx", "cfly", "cflz"):
            dev.cfl_reset()
            if op == "cflx":
                K.cfl_x(d["m"], d["flux"], clust=d["clust"])
            elif op == "cfly":
                K.cfl_y(d["m"], d["flux"])
            else:
                K.cfl_z(d["m"], d["flux"])
            dev.sync()
            if dev.cfl_failed():
                return {}, "fail"
            return {"m": d["m"].host(), "flux": d["flux"].host()}, None
        if op == "fluxes":
            pu, pv = d["pu"], d["pv"]
            im, jm, lm = pv.shape[0], pu.shape[1], pu.shape[2]
            am = DevArray.zeros(dev, (0, im), (0, jm - 1), (0, lm - 1))
            bm = DevArray.zeros(dev, (0, im - 1), (0, jm), (0, lm - 1))
            cm = DevArray.zeros(dev, (0, im - 1), (0, jm - 1), (0, lm))
            K.fluxes_from_meteo(pu, pv, d["bt"], meta["dt"], am, bm, cm)
            dev.sync()
            return {"am": am.host(), "bm": bm.host(), "cm": cm.host()}, None
        if op == "m2phlb1":
            m = d["m"]
            im, jm, lm = m.shape
            sp = DevArray.zeros(dev, (0, im - 1), (0, jm - 1))
            phlb = DevArray.zeros(dev, (0, im - 1), (0, jm - 1), (0, lm))
            K.m2phlb(m, sp, phlb, d["dxyp"], d["at"], d["bt"])
            dev.sync()
            return {"sp": sp.host(), "phlb": phlb.host()}, None
        if op == "convec":
            im, jm = d["m"].shape[0], d["m"].shape[1]
            cols = DevArray.from_host(dev, np.array([(i, j) for i in range(im) for j in range(jm)], dtype=np.int32))
            q = [d[k] for k in TRACERS]
            K.convec(d["m"], *q, d["entu"], d["detu"], d["entd"], d["detd"], d["dkg"], d["cloud_top"], d["cloud_lfs"],
                     cols, meta["dt"], meta["lmax"])  # fmt: skip
            dev.sync()
            cols.free()
            return {k: d[k].host() for k in ("m", *TRACERS)}, None
        if op == "kzz":
            im, jm = d["t"].shape[0], d["t"].shape[1]
            dkg = DevArray.zeros(dev, (0, im - 1), (0, jm - 1), (0, meta["lmax"] - 1))
            pblh = DevArray.zeros(dev, (0, im - 1), (0, jm - 1))
            surface = [d[f"surface.{k}"] for k in K.KZZ_SURFACE]
            K.calc_kzz(d["spm"], d["sp"], d["pu"], d["pv"], d["t"], d["q"], surface, d["at"], d["bt"], d["dxyp"],
                       meta["lmax"], meta["dx"], meta["dy"], meta["ybeg"], dkg, pblh)  # fmt: skip
            dev.sync()
            out = {"dkg": dkg.host(), "pblh": pblh.host()}
            dkg.free()
            pblh.free()
            return out, None
        if op == "chem":
            im, jm, lm = d["temper"].shape
            loss = DevArray.zeros(dev, (0, im - 1), (0, jm - 1), (0, lm - 1), (0, 3))
            decay = DevArray.zeros(dev, (0, im - 1), (0, jm - 1), (0, lm - 1))
            kw = {k: meta[k] for k in ("oh_scale", "cl_scale", "o1d_scale", "soil_rate") if k in meta}
            K.loss_rates(d["temper"], d["phlb"], d["lat"], d, meta["dt"], loss=loss, decay=decay,
                         oh_factor=d.get("oh_factor"), **kw)  # fmt: skip
            dev.sync()
            out = {"loss": loss.host(), "decay": decay.host()}
            loss.free()
            decay.free()
            return out, None
        raise KeyError(op)
    except N.CFLError:
        return {}, "CFLError"
    except ValueError:
        return {}, "ValueError"
    finally:
        for v in d.values():
            v.free()
