"""ORACLE -- test infrastructure.  A synthetic dump set in the format of TM5's pydyn_dump module
(a header `e<seq:05d>_<tag>_r<region>_p<rank:03d>.meta` of `key = value` lines, arrays declared
as `array NAME = lb ub ...` / `iarray NAME = ...`, one raw Fortran-order `<prefix>_<NAME>.bin`
per array; pydyn dump.py:1-8), written from one read interval of the oracle on a small tree:

    cfl        one per region: the air mass and surface pressure Check_CFL started from, the
               meteo data pair, the read interval, and Check_CFL's (ndyn, n)
    massflow   one per region after Setup_MassFlow: m, pu, pv, am, bm, cm, the data pair and
               the step's interval
    bef_<op> / aft_<op>   the state around every operator of the step (x y z v s c), with
               the convection inputs in bef_v, one `emis` event per injection inside an s
               pair and the `chem` event (its inputs and loss rates) inside a c pair
    m2phlb     each region's air mass, surface pressure and half levels after the m2phlb that
               ends its pass

The model is the oracle (pydyn's algorithm restated, bitwise pydyn's), so every event must
replay bitwise.  Header keys and bounds are the ones pydyn's replay reads (replay.py:86-560,
dump.py:23-190); tests/golden/make_golden.py checks a set with pydyn's own reader and replay,
and the replay tests regenerate the same bytes here.  `ranks` > 1 writes the run as a
tracer-split parallel run would (dump.py:228-232): the tracer arrays in slabs, one file set
per rank."""

import hashlib
from datetime import datetime, timedelta
from pathlib import Path

import numpy as np

from pydyn_gb300 import synth

from . import driver as D
from . import kernels as O
from . import zoom as Z
from .forward import oracle_tree
from .physics import OraclePhysics
from .zoom import HostState

T0 = datetime(2000, 1, 1)  # the read interval's start and the first meteo instant
T2 = T0 + timedelta(hours=6)  # the second meteo instant
STATE = ("m", "rm", "rxm", "rym", "rzm", "am", "bm", "cm")
TRACER_ARRAYS = ("rm", "rxm", "rym", "rzm")
MOL_MASS, MOL_MASS_E, EFRAC, SEC_MONTH = 16.04, 12.01, 0.5, 31.0 * 86400.0


def interpol_fractions(t, t1, t2):
    """go_date InterpolFractions (pydyn balance.py:55-60): the weights of t1 and t2 at t."""
    ds, ds1 = (t2 - t1).total_seconds(), (t - t1).total_seconds()
    a2 = 0.5 if abs(ds) < np.finfo(float).tiny else ds1 / ds
    return 1.0 - a2, a2


def _date(t):
    return (t.year, t.month, t.day, t.hour, t.minute, t.second)


def _text(v):
    if isinstance(v, bool | np.bool_):
        return "T" if v else "F"
    if isinstance(v, int | np.integer):
        return str(int(v))
    if isinstance(v, float | np.floating):
        return repr(float(v))
    if isinstance(v, tuple):
        return " ".join(str(int(x)) for x in v)
    return str(v)


class Writer:
    """Events of one set, numbered in order; `ranks` > 1 splits the tracer arrays by rank."""

    def __init__(self, out, zoom, nt, ranks=1):
        self.dir, self.zoom, self.nt, self.ranks = Path(out), zoom, nt, ranks
        self.dir.mkdir(parents=True, exist_ok=True)
        self.seq = 0
        per = -(-nt // ranks)
        self.slabs = [(k * per, min(nt, (k + 1) * per)) for k in range(ranks)]

    def tree_meta(self, r):
        z, g = self.zoom, self.zoom.g(r)
        m = {"grid_name": g.name, "im": g.im, "jm": g.jm, "lm": z.lm, "xref": g.xref, "yref": g.yref,
             "zref": g.zref, "tref": g.tref, "parent": g.parent, "xcyc": g.xcyc, "touch_sp": g.touch_sp,
             "touch_np": g.touch_np, "splitorder": z.splitorderzoom[r], "status": z.status[r]}  # fmt: skip
        if z.children[r]:
            kids = tuple(z.children[r])
            m["children"] = kids if len(kids) > 1 else kids[0]
        if r > 1:
            m.update(ibeg=z.ibeg[r], iend=z.iend[r], jbeg=z.jbeg[r], jend=z.jend[r])
        rg = g.redgrid
        if rg is not None:
            jred = tuple(j + 1 for j, _, _ in rg.bands)
            clust = tuple(c for _, c, _ in rg.bands)
            m.update(grid_reduced=True, nred=len(jred), jred=jred if len(jred) > 1 else jred[0],
                     clustsize=clust if len(clust) > 1 else clust[0])  # fmt: skip
        else:
            m["grid_reduced"] = False
        return m

    def event(self, tag, region, meta, arrays, tracer=None):
        """arrays: {name: (data, lower)}; tracer: the global tracer number of a per-tracer event
        (written by the rank that holds it alone)."""
        self.seq += 1
        for rank, (t0, t1) in enumerate(self.slabs):
            if tracer is not None and not (t0 < tracer <= t1):
                continue
            head = {"tag": tag, "seq": self.seq, "region": region, **self.tree_meta(region), **meta}
            if self.ranks > 1:
                head.update(rank=rank, ntracet=self.nt)
                if "ch4_tracers" in head:
                    local = tuple(t - t0 for t in np.atleast_1d(head["ch4_tracers"]) if t0 < t <= t1)
                    head["ch4_tracers"] = local if len(local) != 1 else local[0]
            prefix = self.dir / f"e{self.seq:05d}_{tag}_r{region}_p{rank:03d}"
            lines = [f"{k} = {_text(v)}" for k, v in head.items()]
            for name, (data, lower) in arrays.items():
                data = np.asarray(data)
                lower = list(lower)
                if self.ranks > 1 and name in TRACER_ARRAYS:
                    data = data[..., t0:t1]
                bounds = " ".join(f"{lo} {lo + n - 1}" for lo, n in zip(lower, data.shape, strict=True))
                kind = "iarray" if data.dtype.kind in "iu" else "array"
                lines.append(f"{kind} {name} = {bounds}")
                dt = "<i4" if kind == "iarray" else "<f8"
                np.asarray(data, dtype=dt).ravel(order="F").tofile(f"{prefix}_{name}.bin")
            prefix.with_suffix(".meta").write_text("\n".join(lines) + "\n")


def _fa(fa):
    return (fa.data.copy(), fa.lower)


def _state(st, r, names=STATE):
    return {k: _fa(st[r][k]) for k in names}


class _Lib:
    """The oracle's bodies, with convec_region and the m2phlb bodies dumping around themselves."""

    def __init__(self, writer, ndyn):
        self.w, self.ndyn = writer, ndyn

    def __getattr__(self, name):
        return getattr(Z, name)

    def convec_region(self, zoom, st, region, conv, ndyn, inverse="crout"):
        lmax = conv["lmax"]
        ins = {k: (np.asarray(conv[k])[:, :, :lmax], (1, 1, 1)) for k in ("entu", "detu", "entd", "detd", "dkg")}
        ins.update({k: (np.asarray(conv[k], dtype=np.int32), (1, 1)) for k in ("cloud_top", "cloud_lfs")})
        self.w.event("bef_v", region, {"limits": True, "nconv": int(ndyn)}, {**_state(st, region), **ins})
        Z.convec_region(zoom, st, region, conv, ndyn, inverse)
        self.w.event("aft_v", region, {}, _state(st, region))

    def _m2phlb(self, fn, zoom, st, region):
        fn(zoom, st, region)
        self.w.event("m2phlb", region, {}, _state(st, region, ("m", "sp", "phlb")))

    def m2phlb(self, zoom, st, region):
        self._m2phlb(Z.m2phlb, zoom, st, region)

    def m2phlb1(self, zoom, st, region=1):
        self._m2phlb(Z.m2phlb1, zoom, st, region)


def write_set(out, config="two", lm=5, seed=3, nt=1, ranks=1, umax=40.0, ndyn=3600, nread=3600):
    """Write the set of one read interval of `config` into `out`; returns (ndyn, n) of its
    Check_CFL."""
    gen, met, fields = synth.case(config, lm, seed, nt, umax=umax)
    zoom = oracle_tree(gen)
    st, cst = HostState(zoom, nt), HostState(zoom, nt)
    st.load(fields)
    for r in zoom.regions():
        cst[r]["dxyp"].data[...] = fields[r]["dxyp"]
    spec = synth.Physics(gen, met, seed, lm, kind="full")
    phys = OraclePhysics(zoom, spec)
    phys.init(st)
    w = Writer(out, zoom, nt, ranks)
    pairs = {r: [met.fluxes(r, k) for k in (0, 1)] for r in zoom.regions()}
    const = {"at": (zoom.at, (1,)), "bt": (zoom.bt, (1,))}

    def pair_arrays(r):
        (pu1, pv1), (pu2, pv2) = pairs[r]
        lo_u, lo_v = st[r]["pu"].lower, st[r]["pv"].lower
        return {"pu1": (pu1, lo_u), "pu2": (pu2, lo_u), "pv1": (pv1, lo_v), "pv2": (pv2, lo_v)}

    def interpolate(s, t):
        a1, a2 = interpol_fractions(t, T0, T2)
        for r in zoom.regions():
            (pu1, pv1), (pu2, pv2) = pairs[r]
            s[r]["pu"].data[...] = a1 * pu1 + a2 * pu2
            s[r]["pv"].data[...] = a1 * pv1 + a2 * pv2

    # ---- Check_CFL from the interval's start
    for r in zoom.regions():
        for name in ("m", "sp"):
            cst[r][name].data[...] = st[r][name].data
    start = {r: _state(cst, r, ("m", "sp", "dxyp")) for r in zoom.regions()}
    ndyn_out, n_out, _ = D.check_cfl_zoom(zoom, cst, ndyn, nread // ndyn, nread,
                                          lambda z, s, i, nd: interpolate(s, T0 + timedelta(seconds=(i - 0.5) * nd)))
    for r in zoom.regions():
        meta = {"tread1": _date(T0), "tread2": _date(T0 + timedelta(seconds=nread)), "pu_t1": _date(T0),
                "pu_t2": _date(T2), "ndyn_in": ndyn, "n_in": nread // ndyn, "nread": nread, "ndyn_out": ndyn_out,
                "n_out": n_out}  # fmt: skip
        w.event("cfl", r, meta, {**start[r], **pair_arrays(r), **const})

    # ---- the steps
    for k in range(n_out):
        tr1 = T0 + timedelta(seconds=k * ndyn_out)
        tr2 = tr1 + timedelta(seconds=ndyn_out)
        interpolate(st, tr1 + (tr2 - tr1) / 2)
        D.setup_massflow(zoom, st, ndyn_out)
        for r in zoom.regions():
            meta = {"tr1": _date(tr1), "tr2": _date(tr2), "pu_t1": _date(T0), "pu_t2": _date(T2), "ndyn": ndyn_out}
            w.event("massflow", r, meta, {**_state(st, r, ("m", "pu", "pv", "am", "bm", "cm", "dxyp")),
                                          **pair_arrays(r), **const})  # fmt: skip
        conv, _ = phys.step(st, (tr1 - T0).total_seconds(), ndyn_out)
        _step(zoom, st, w, spec, conv, ndyn_out)
    return ndyn_out, n_out


def _step(zoom, st, w, spec, conv, ndyn):
    lib = _Lib(w, ndyn)
    saved_ops = dict(D.OPERATORS)

    def dumped(op, fn):
        def run(z, s, region, limits=True, stats=None):
            w.event(f"bef_{op}", region, {"limits": bool(limits)}, _state(s, region))
            fn(z, s, region, limits, stats=stats)
            w.event(f"aft_{op}", region, {}, _state(s, region))

        return run

    def sources(z, s, region):
        g = z.g(region)
        w.event("bef_s", region, {"limits": True}, _state(s, region))
        emis = spec.region[region]["flux"] * s[region]["dxyp"].data[None, :]
        m2dt = (float(ndyn) / (2 * g.tref)) / SEC_MONTH
        x = ((emis * m2dt) * (MOL_MASS / MOL_MASS_E)) * EFRAC  # emis.inject (pydyn emis.py:52-54)
        meta = {"month2dt": m2dt, "mol_mass": MOL_MASS, "mol_mass_e": MOL_MASS_E, "efrac": EFRAC, "l_level": 1,
                "i_tracer": 1}  # fmt: skip
        w.event("emis", region, meta, {"emis": (emis, (1, 1))}, tracer=1)
        Z.sources_region(z, s, region, [(x, 1, 1)])
        w.event("aft_s", region, {}, _state(s, region))

    def chemistry(z, s, region):
        g, R = z.g(region), spec.region[region]
        c, lm = R["chem"], z.lm
        si, sj = z.scope(region)
        w.event("bef_c", region, {"limits": True}, _state(s, region))
        phlb = s[region]["phlb"][1 : g.im, 1 : g.jm, 1 : lm + 1]
        dt = spec.half_step(region, ndyn)
        loss, decay = O.loss_rates(R["kzz"]["t"][si, sj], phlb[si, sj], c["lat"][sj], c["strat_press"][sj],
                                   c["strat_oh"][sj], c["strat_cl"][sj], c["strat_od"][sj], c["oh_3d"][si, sj],
                                   pl_trop=c["pl_trop"][si, sj], cl_trop=c["cl_trop"][si, sj], soil=c["soil"][si, sj],
                                   dt=dt, **spec.settings)  # fmt: skip
        meta = {"dt_sec": dt, "isotopes": False, "ch4_tracers": 1, "trop_cl_sink": True, "soil_sink": True,
                **{k: float(v) for k, v in spec.settings.items()}}  # fmt: skip
        arrays = {"temper": (R["kzz"]["t"], (1, 1, 1)), "phlb": _fa(s[region]["phlb"]), "lat": (c["lat"], (1,)),
                  "oh_3d": (c["oh_3d"], (1, 1, 1)), "pl_trop": (c["pl_trop"], (1, 1, 1)),
                  "cl_trop": (c["cl_trop"], (1, 1, 1)), "soil": (c["soil"], (1, 1)), "loss": (loss, (1, 1, 1, 1))}
        arrays.update({f"strat_{k}": (c[f"strat_{k}"], (1, 1)) for k in ("press", "oh", "cl", "od")})
        w.event("chem", region, meta, arrays)
        Z.chemistry_region(z, s, region, decay, (1,))
        w.event("aft_c", region, {}, _state(s, region))

    st_lib = st.lib
    try:
        for op, fn in saved_ops.items():
            D.OPERATORS[op] = dumped(op, fn)
        st.lib = lib
        D.step(zoom, st, conv, ndyn, limits=True, sources=sources, chemistry=chemistry)
    finally:
        D.OPERATORS.update(saved_ops)
        st.lib = st_lib


def digest(out):
    """sha1 over the set's file names and bytes, in name order."""
    h = hashlib.sha1()
    for p in sorted(Path(out).iterdir()):
        h.update(p.name.encode())
        h.update(p.read_bytes())
    return h.hexdigest()
