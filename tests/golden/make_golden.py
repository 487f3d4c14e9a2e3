"""Make the golden fixtures of tests/golden/ from the reference itself.

Run where the pydyn reference is importable (its checkout is on PYDYN_REFERENCE, default
/root/reference); the fixtures it writes are what the tests compare the oracle and the device
against on machines that do not have the reference:

    python tests/golden/make_golden.py kernels     -> tests/golden/kernels.npz

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

REF = Path(os.environ.get("PYDYN_REFERENCE", "/root/reference"))
HERE = Path(__file__).resolve().parent


def _reference():
    sys.path.insert(0, str(REF))
    import pydyn  # noqa: F401

    return pydyn


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
