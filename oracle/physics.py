"""ORACLE -- test infrastructure.  The physics of a step on the host, as pydyn_gb300.physics runs
it on the device and the golden fixtures' pydyn run composes it: Calc_Kzz of every region after
Setup_MassFlow (spm the meteo's at the step's middle, sp the region's at its start), then `v`,
`s`, `c` on the owned columns with dt = ndyn / (2 tref) -- the C oracle's calc_kzz, convec and
loss_rates, NumPy for the emission and the decay's application."""

from pydyn_gb300 import synth

from . import kernels as O

N_OPERATORS = 6


class OraclePhysics:
    def __init__(self, zoom, spec):
        """zoom: the oracle's tree; spec: the physics inputs of pydyn_gb300.synth.Physics."""
        self.spec = spec
        self.zoom = zoom

    def init(self, st):
        """sp and phlb of every region from its initial air mass."""
        for r in self.zoom.regions():
            if r == 1:
                st.lib.m2phlb1(self.zoom, st, 1)
            else:
                st.lib.m2phlb(self.zoom, st, r)

    def step(self, st, t0, ndyn):
        """(conv, driver kwargs) of the step from t0, after Setup_MassFlow."""
        spec, zoom = self.spec, self.zoom
        if spec.kind == "convection":  # pydyn's GPU benchmark inputs: convection on a given dkg alone
            return {r: {**spec.region[r]["conv"], "dkg": spec.region[r]["dkg"], "lmax": spec.lmax}
                    for r in zoom.regions()}, {}  # fmt: skip
        a1, a2 = synth.weights(t0 + ndyn / 2.0)
        conv = {}
        for r in zoom.regions():
            g, R, f = zoom.g(r), spec.region[r], st[r]
            k = R["kzz"]
            spm = a1 * k["spm"][0] + a2 * k["spm"][1]
            dx, dy = (g.xend - g.xbeg) / g.im, (g.yend - g.ybeg) / g.jm
            dkg, _ = O.calc_kzz(spm, f["sp"][1 : g.im, 1 : g.jm, 1], f["pu"].data, f["pv"].data, k["t"], k["q"],
                                k["surface"], zoom.at, zoom.bt, f["dxyp"].data, spec.lmax, dx, dy, float(g.ybeg))  # fmt: skip
            conv[r] = {**R["conv"], "dkg": dkg, "lmax": spec.lmax}

        def sources(zoom, s, region):
            x = spec.region[region]["flux"] * s[region]["dxyp"].data[None, :] * spec.half_step(region, ndyn)
            s.lib.sources_region(zoom, s, region, [(x, 1, 1)])

        def chemistry(zoom, s, region):
            g, R = zoom.g(region), spec.region[region]
            h = zoom.status[region] // N_OPERATORS
            c = R["chem"]
            phlb = s[region]["phlb"][1 : g.im, 1 : g.jm, 1 : zoom.lm + 1]
            _, decay = O.loss_rates(R["kzz"]["t"], phlb, c["lat"], c["strat_press"], c["strat_oh"], c["strat_cl"],
                                    c["strat_od"], c["oh_3d"], pl_trop=c["pl_trop"], cl_trop=c["cl_trop"],
                                    soil=c["soil"], dt=spec.half_step(region, ndyn),
                                    oh_factor=spec.factors(region, t0, ndyn)[h], **spec.settings)  # fmt: skip
            s.lib.chemistry_region(zoom, s, region, decay[zoom.scope(region)], (1,))

        return conv, {"sources": sources, "chemistry": chemistry}
