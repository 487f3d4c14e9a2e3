"""The adjoint of the dynamic step: the CH4 surface-flux gradient of a run.

Scope: one global region (glb3x2, glb6x4, the small `one`), one tracer, unlimited slopes
(`limits=False`), convection with Kzz diffusion folded in, emission, and chemistry at fixed OH.
With the limiter off every tracer operator of a step is linear in the tracer moments, for an air
mass and fluxes that do not depend on the tracers.  The operators are x, y and z advection,
convection, and chemistry (a per-cell decay).  Emission adds flux x area x dt.  The state after
any number of steps is therefore affine in the flux, and the cost

    J = sum over samples (cell, hour) of (rm(cell, end of hour) - obs)^2

is quadratic in it.

Gradient by checkpointing.  The forward pass keeps the whole state at the start of every
`every`-th interval.  The backward pass takes the segments last to first.  For each segment it
restores the segment's checkpoint and recomputes the segment's intervals with a tape on.  The
tape is a body layer over the region's bodies.  It copies the air mass and fluxes each tracer
operator is given, the sub-cycle counts that the device returns, the convection inverses and
the chemistry inputs.  Then the transposed operators run over the tape in reverse on the tracer
adjoints: `gb_adjoint_x / _y / _z / _convec / _sources`, and chemistry applied to the adjoints
itself, since it is diagonal.  The sample residuals 2 (rm - obs) are added where their hour
ends.  Every recomputation is bitwise the forward's: the same kernels on the same inputs, the
convection inverse remade on each step's first `v` as the forward made it.

`FluxGradient` is behind `torch.autograd.Function` (`CH4FluxCost`): forward(flux) -> J,
backward -> dJ / dflux, for a flux tensor on the GPU (float64, (im, jm)).  PyTorch is only this
wrapper: the run, the tape and the adjoint are the library's kernels."""

import numpy as np

from . import kernels as K
from .device import DevArray
from .state import TRACERS

N_OPERATORS = 6


def _copy(a):
    """A contiguous device copy of a section, with its bounds."""
    out = DevArray.zeros(a.dev, *((lo, lo + n - 1) for lo, n in zip(a.lower, a.shape, strict=True)), dtype=a.dtype)
    out.assign(a)
    return out


class TapingLib:
    """The region's bodies with a tape: each tracer operator's inputs are copied before it runs
    (and the sub-cycle counts after), then the body runs unchanged."""

    def __init__(self, lib, tape):
        self._lib, self._tape = lib, tape

    def __getattr__(self, name):
        return getattr(self._lib, name)

    def _dynamu_region1(self, zoom, st, js, je, limits, stats, max_nloop=50):
        g, f, lm = zoom.g(1), st[1], zoom.lm
        self._tape.append(("x", _copy(f["m"][1 : g.im, 1 : g.jm, 1:lm]), _copy(f["am"][0 : g.im, 1 : g.jm, 1:lm]),
                           max_nloop))  # fmt: skip
        self._lib._dynamu_region1(zoom, st, js, je, limits, stats, max_nloop)

    def _dynamv_region1(self, zoom, st, limits, stats, max_nloop=10):
        g, f, lm = zoom.g(1), st[1], zoom.lm
        m = f["m"][1 : g.im, 1 : g.jm, 1:lm]
        bm = f["bm"][1 : g.im, 1 : g.jm + 1, 1:lm]
        nloop = DevArray.zeros(st.dev, (0, lm - 1), dtype=np.int32)
        self._tape.append(("y", _copy(m), _copy(bm), nloop))
        q = [f[name][1 : g.im, 1 : g.jm, 1:lm] for name in TRACERS]
        K.advect_y(m, *q, bm, bm_full=f["bm"], bm_full_l0=1, limits=limits, max_nloop=max_nloop, nloop=nloop)

    def _dynamw_region1(self, zoom, st, limits, stats, iter_limit=15):
        g, f, lm = zoom.g(1), st[1], zoom.lm
        m = f["m"][1 : g.im, 1 : g.jm, 1:lm]
        n = DevArray.zeros(st.dev, (0, 0), dtype=np.int32)
        self._tape.append(("z", _copy(m), _copy(f["cm"][1 : g.im, 1 : g.jm, 0:lm]), n))
        self._lib._dynamw_region1(zoom, st, limits, stats, iter_limit)
        K.advect_z_last(m, n)

    def convec_region(self, zoom, st, region, conv, ndyn, inverse="crout"):
        self._lib.convec_region(zoom, st, region, conv, ndyn, inverse)
        d = conv.r[region]
        if d["ncol"]:
            self._tape.append(("v", _copy(d["cache"][0]), d["cols"], conv.lmax))


class FluxGradient:
    """J and dJ / dflux of a single-region run with physics (pydyn_gb300.forward.Forward made
    with limits=False, physics=True) over `hours` one-hour intervals from its present state.
    samples: (hour 1..hours, i, j, l) 0-based interior cells; obs: their observed tracer mass."""

    def __init__(self, fw, hours, samples, obs, every=6, graph=True):
        if fw.zoom.nregions != 1 or fw.physics is None or fw.limits:
            raise ValueError("FluxGradient: one region, physics on, limits off")
        self.fw, self.hours, self.every, self.graph = fw, int(hours), int(every), bool(graph)
        self.samples = np.asarray(samples, dtype=np.int64).reshape(-1, 4)
        self.obs = np.asarray(obs, dtype=np.float64).reshape(-1)
        if self.samples.shape[0] != self.obs.shape[0]:
            raise ValueError("FluxGradient: one observation per sample")
        if self.samples.size and (self.samples[:, 0].min() < 1 or self.samples[:, 0].max() > self.hours):
            raise ValueError("FluxGradient: sample hours are 1..hours")
        self.d = fw.physics.r[1]
        self.start = self._checkpoint()  # every evaluation starts here
        self.checkpoints = {}
        self.rm_at = {}
        self.intervals = 0

    # -------------------------------------------------------------- state
    def _checkpoint(self):
        st = self.fw.st[1]
        return {"t": self.fw.t, "fields": {k: _copy(a) for k, a in st.items()}}

    def _restore(self, ck):
        st = self.fw.st[1]
        for k, a in ck["fields"].items():
            st[k].assign(a)
        self.fw.t = ck["t"]

    def _free(self, ck):
        for a in ck["fields"].values():
            a.free()

    def set_flux(self, flux):
        """The region's CH4 surface flux (kg m-2 s-1, (im, jm)) from a host array or DevArray."""
        if isinstance(flux, DevArray):
            self.d["flux"].assign(flux)
        else:
            self.d["flux"].upload(np.ascontiguousarray(flux, dtype=np.float64))

    def _rm(self):
        g, lm = self.fw.zoom.g(1), self.fw.zoom.lm
        return self.fw.st[1]["rm"][1 : g.im, 1 : g.jm, 1:lm, 1]

    def _sample(self, hour):
        rows = np.flatnonzero(self.samples[:, 0] == hour)
        if rows.size == 0:
            return rows, np.zeros(0)
        rm = self._rm()
        vals = np.array([rm[i + 1 : i + 1, j + 1 : j + 1, l + 1 : l + 1].host().reshape(-1)[0]
                         for _, i, j, l in self.samples[rows].tolist()])  # fmt: skip
        return rows, vals

    # -------------------------------------------------------------- forward
    def cost(self, flux=None):
        """J from the starting state; keeps the checkpoints and the sampled values."""
        if flux is not None:
            self.set_flux(flux)
        for ck in self.checkpoints.values():
            self._free(ck)
        self.checkpoints, self.rm_at = {}, {}
        self._restore(self.start)
        J = 0.0
        for h in range(1, self.hours + 1):
            if (h - 1) % self.every == 0:
                self.checkpoints[h - 1] = self._checkpoint()
            self.fw.interval(graph=self.graph)  # replayed as the captured interval; the taped
            rows, vals = self._sample(h)  # recomputation runs the same kernels eagerly
            self.rm_at[h] = (rows, vals)
            r = vals - self.obs[rows]
            J += float(np.dot(r, r))
        self.fw.dev.sync()
        return J

    # -------------------------------------------------------------- backward
    def _taped_interval(self):
        fw, tape = self.fw, []
        phys = fw.physics
        src, chem = phys.sources, phys.chemistry

        def sources(zoom, st, region):
            tape.append(("s", phys.spec.half_step(region, phys.ndyn)))
            src(zoom, st, region)

        def chemistry(zoom, st, region):
            g, d = zoom.g(region), phys.r[region]
            h = zoom.status[region] // N_OPERATORS
            tape.append(("c", _copy(st[region]["phlb"][1 : g.im, 1 : g.jm, 1 : zoom.lm + 1]), _copy(d["factors"][h]),
                         phys.spec.half_step(region, phys.ndyn)))  # fmt: skip
            chem(zoom, st, region)

        old = fw.st.lib
        fw.st.lib = TapingLib(old, tape)
        phys.sources, phys.chemistry = sources, chemistry
        try:
            fw.interval(graph=False)
        finally:
            fw.st.lib = old
            del phys.sources, phys.chemistry  # the class's methods again
        return tape

    def _adjoint_op(self, op, qb, grad, free=True):
        d, zoom, st = self.d, self.fw.zoom, self.fw.st
        kind = op[0]
        if kind == "x":
            from .zoom import _clust

            K.adjoint_x(op[1], *qb, op[2], clust=_clust(st, 1), max_nloop=op[3])
        elif kind == "y":
            K.adjoint_y(op[1], *qb, op[2], op[3])
        elif kind == "z":
            K.adjoint_z(op[1], *qb, op[2], op[3])
        elif kind == "v":
            K.adjoint_convec(*qb, op[1], op[2], op[3])
        elif kind == "s":
            from .physics import LEVEL

            K.adjoint_sources(qb[0], qb[3], grad, d["cols"], LEVEL, d["dxyp"], op[1])
        elif kind == "c":
            from .physics import CH4_TRACERS

            phys = self.fw.physics
            K.chemistry(d["t"], op[1], d["chem"]["lat"], d["chem"], op[3], d["cols"], CH4_TRACERS, *qb,
                        oh_factor=op[2], krates=d["krates"], **phys.spec.settings)  # fmt: skip
        else:
            raise ValueError(f"adjoint: unknown taped operator {kind!r}")
        if free:  # the taped copies are given back as the sweep passes them
            for a in op[1:]:
                if isinstance(a, DevArray) and a is not d["cols"]:
                    a.free()

    def interval_pair(self, x, ys):
        """A x and A^T y for the linear map A of one interval from the present state at zero
        flux: x and every y of ys are (4, im, jm, lm) host arrays of (rm, rxm, rym, rzm) on the
        interior.  The run is left after the interval, the flux at zero."""
        fw = self.fw
        g, lm = fw.zoom.g(1), fw.zoom.lm
        self.set_flux(np.zeros((g.im, g.jm)))
        for w, name in enumerate(TRACERS):
            fw.st[1][name][1 : g.im, 1 : g.jm, 1:lm, 1:1].upload(np.asarray(x[w])[..., None])
        tape = self._taped_interval()
        ax = np.stack([fw.st[1][name][1 : g.im, 1 : g.jm, 1:lm, 1].host() for name in TRACERS])
        grad = DevArray.zeros(fw.dev, (0, g.im - 1), (0, g.jm - 1))
        out = []
        for y in ys:
            qb = [DevArray.from_host(fw.dev, np.asarray(y[w])[..., None], lower=(1, 1, 1, 1)) for w in range(4)]
            for op in reversed(tape):
                self._adjoint_op(op, qb, grad, free=False)
            out.append(np.stack([q.host()[..., 0] for q in qb]))
            for q in qb:
                q.free()
        for op in tape:
            for a in op[1:]:
                if isinstance(a, DevArray) and a is not self.d["cols"]:
                    a.free()
        grad.free()
        return ax, out

    def gradient(self):
        """dJ / dflux (a DevArray (im, jm)) of the last cost() evaluation."""
        if not self.checkpoints:
            raise RuntimeError("FluxGradient: cost() first")
        fw, dev = self.fw, self.fw.dev
        g, lm = fw.zoom.g(1), fw.zoom.lm
        grad = DevArray.zeros(dev, (0, g.im - 1), (0, g.jm - 1))
        qb = [DevArray.zeros(dev, (1, g.im), (1, g.jm), (1, lm), (1, 1)) for _ in TRACERS]
        starts = sorted(self.checkpoints)
        for s0 in reversed(starts):
            s1 = min(s0 + self.every, self.hours)
            self._restore(self.checkpoints[s0])
            tapes = [self._taped_interval() for _ in range(s0, s1)]
            for h in range(s1, s0, -1):  # hour h ends interval h - 1 (0-based)
                rows, vals = self.rm_at[h]
                if rows.size:
                    resid = 2.0 * (vals - self.obs[rows])
                    for (_, i, j, l), v in zip(self.samples[rows].tolist(), resid.tolist(), strict=True):
                        cell = qb[0][i + 1 : i + 1, j + 1 : j + 1, l + 1 : l + 1, 1:1]
                        cell.upload(cell.host() + v)
                for op in reversed(tapes[h - 1 - s0]):
                    self._adjoint_op(op, qb, grad)
        dev.sync()
        self._restore(self.start)  # the run is left at its start, the tapes given back
        for a in qb:
            a.free()
        return grad

    def close(self):
        for ck in self.checkpoints.values():
            self._free(ck)
        self.checkpoints = {}
        self._free(self.start)


def make_samples(zoom, hours, n=500, seed=0):
    """n seeded (hour, i, j, l) samples over the region's interior cells and hours 1..hours."""
    g, lm = zoom.g(1), zoom.lm
    rng = np.random.default_rng([seed, 7717])
    return np.stack([rng.integers(1, hours + 1, n), rng.integers(0, g.im, n), rng.integers(0, g.jm, n),
                     rng.integers(0, lm, n)], axis=1)  # fmt: skip


def _torch_function():
    import torch

    class CH4FluxCost(torch.autograd.Function):
        """J(flux) of a FluxGradient, with its adjoint as the backward."""

        @staticmethod
        def forward(ctx, flux, problem):
            ctx.problem = problem
            J = problem.cost(flux.detach().to("cpu", torch.float64).numpy())
            return torch.tensor(J, dtype=torch.float64, device=flux.device)

        @staticmethod
        def backward(ctx, gJ):
            grad = ctx.problem.gradient()
            out = torch.from_numpy(grad.host()).to(gJ.device) * gJ
            grad.free()
            return out, None

    return CH4FluxCost


def ch4_flux_cost(flux, problem):
    """J(flux) as a differentiable torch scalar: `ch4_flux_cost(flux, problem).backward()` fills
    flux.grad with dJ / dflux from the adjoint."""
    return _torch_function().apply(flux, problem)
