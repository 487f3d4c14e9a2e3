"""The device against the oracle body by body through whole intervals of the production trees
(glb6x4, glb3x2, glb3x2 + nam1x1): the package's planned sequence (pydyn_gb300.plan) issues every
body on both, and after each every state array of every region must be bitwise equal; a failure
names the first body that diverged."""

import pytest
from lockstep import LockState


def _interval(zoom, lock, cst_lock, t0, weights_dev, orc):
    from pydyn_gb300 import plan as P

    def interpolate(z, s, i, ndyn):
        t = t0 + (i - 0.5) * ndyn
        weights_dev(s.dev_st, t)
        orc.interpolate(s.orc_st, t)

    ndyn, n, _ = P.check_cfl(zoom, cst_lock, 3600, 1, 3600, interpolate)
    for k in range(n):
        t = t0 + k * ndyn + ndyn / 2.0
        weights_dev(lock.dev_st, t)
        orc.interpolate(lock.orc_st, t)
        lock.compare("interpolation")
        P.setup_massflow(zoom, lock, ndyn)
        P.step(zoom, lock, None, ndyn, limits=True)
    return ndyn, n


@pytest.mark.gpu
@pytest.mark.parametrize(("config", "lm", "seed"), [("glb6x4", 25, 11), ("two", 5, 13), ("three", 4, 15),
                                                    ("glb3x2", 34, 21), ("glb3x2+nam1x1", 34, 31)])  # fmt: skip
def test_lockstep_interval(dev, config, lm, seed):
    from oracle.forward import OracleRun

    from pydyn_gb300.forward import Forward

    fw = Forward(dev, config, lm, seed)
    orc = OracleRun(config, lm, seed)
    lock = LockState(fw.st, orc.st)
    cst = LockState(fw.cfl_st, orc.cst)
    lock.compare("start")
    for r in fw.zoom.regions():
        for name in ("m", "sp"):
            fw.cfl_st[r][name].assign(fw.st[r][name])
            orc.cst[r][name].data[...] = orc.st[r][name].data

    def weights_dev(st, t):
        fw.put_weights(t)
        fw.interpolate(st)

    for k in range(2):
        got = _interval(fw.zoom, lock, cst, k * 3600.0, weights_dev, orc)
        assert got == (3600, 1), f"interval {k}: Check_CFL chose {got}"
        for r in fw.zoom.regions():
            for name in ("m", "sp"):
                fw.cfl_st[r][name].assign(fw.st[r][name])
                orc.cst[r][name].data[...] = orc.st[r][name].data
    fw.close()
