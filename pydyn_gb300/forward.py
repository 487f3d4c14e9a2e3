"""The dynamic step as a run performs it, on the device (pydyn forward.py:388-451, Forward._carry
and Forward._step, recomposed for a region tree): for every read interval, Check_CFL rehearses
the interval's steps on a copy of the air mass and decides ndyn; then each step interpolates
the meteo fluxes to its middle, runs Setup_MassFlow, (with physics) Calc_Kzz, and the operator
sequence with sources and chemistry at each half step.

A step never waits for the device.  `interval(graph=True)` replays the interval (Check_CFL +
one step at ndyn = nread) as one captured CUDA graph; the step runs speculatively next to the
rehearsal, from a device copy of the state taken at the interval's start, and the host reads
the rehearsal's one flag after the replay -- if it failed, the state is put back and the
interval is redone uncaptured with ndyn reduced, as Check_CFL decides.

The meteo of a configuration (pydyn_gb300.synth) is two flux instants per region, six hours
apart; a step at time t interpolates them with weights held in device memory, so the captured
graph serves every step."""

import numpy as np

from . import _native as N
from . import plan as P
from . import synth
from .device import DevArray, Device
from .schedule import ScheduledLib, Scheduler, scheduled_physics, spreadable
from .state import TRACERS, ZoomState
from .synth import weights

SPECULATED = ("m", *TRACERS, "sp", "phlb")
# stream priorities of the captured interval's side contexts, in steps above the device's least
# (the run's own stream and the Check_CFL rehearsal stay at the least): a child's chain of small
# kernels is the interval's critical path, each region's Calc_Kzz gates its first convection, and
# the rehearsal has the most slack -- measured on glb3x2+nam1x1, 6.49 -> 6.42 ms per interval
CHILD_PRIORITY = 3
KZZ_PRIORITY = 1
FAR_PRIORITY = 0  # region 1's physics on its far segment (slack until the parent's m2phlb1)
MAIN_PRIORITY = 0  # the run's own stream (region 1's bodies on the edge segment)
CFL_PRIORITY = 0  # the Check_CFL rehearsal's context


class Forward:
    """A configuration's run on one device: the state, the Check_CFL copy, the meteo instants."""

    def __init__(self, dev, config="glb6x4", lm=25, seed=0, nt=1, ndyn=3600, nread=3600, limits=True, physics=False,
                 umax=40.0, lmax=None, wind_scale=1.0, physics_seed=None):  # fmt: skip
        """physics: True (or "full") with convection (Kzz folded in), emission and CH4 chemistry
        over lmax levels (default lm), on the inputs of pydyn_gb300.synth.Physics drawn from
        physics_seed (default seed); "convection": convection alone on a given dkg, the inputs of
        pydyn's own GPU benchmark; False: advection only.  wind_scale multiplies the meteo's winds."""
        self.dev = dev
        self.zoom, self.met, fields = synth.case(config, lm, seed, nt, umax=umax, wind_scale=wind_scale)
        self.st = ZoomState.from_host(dev, self.zoom, fields)
        self.cfl_st = ZoomState.zeros(dev, self.zoom, nt)
        for r in self.zoom.regions():
            self.cfl_st[r]["dxyp"].assign(self.st[r]["dxyp"])
        self.ndyn_max, self.nread, self.limits = ndyn, nread, limits
        self.t = 0.0
        self.meteo = {}
        for r in self.zoom.regions():
            pair = [self.met.fluxes(r, k) for k in (0, 1)]
            self.meteo[r] = [(DevArray.from_host(dev, pu), DevArray.from_host(dev, pv)) for pu, pv in pair]
        self.w = DevArray.zeros(dev, (0, 1))
        self.physics = None
        if physics:
            from .physics import Physics

            pseed = seed if physics_seed is None else physics_seed
            kind = "full" if physics is True else physics
            spec = synth.Physics(self.zoom, self.met, pseed, lm if lmax is None else lmax, kind=kind)
            self.physics = Physics(dev, self.zoom, spec, {r: self.st[r]["dxyp"] for r in self.zoom.regions()})
            self.physics.init_state(self.st)
        self.graphs = {}
        self.last = {}
        self.aux = None  # the captured interval's side contexts, one per region (a child's share of the step)
        self.prep = None  # the captured interval's Calc_Kzz contexts, one per region (with physics)
        self.aux_cfl = None  # the captured interval's rehearsal context
        self._replays, self._side_per_replay = 0, 0

    # -------------------------------------------------------------- meteo
    def put_weights(self, t):
        self.w.upload(np.array(weights(t)))

    def interp_into(self, dst, a, b):
        """dst = w1 a + w2 b with the device-held weights of the step."""
        _interp(dst, a, b, self.w)

    def put_step_inputs(self, t0, ndyn):
        """The step's time-dependent inputs into device memory: the meteo weights at its middle
        and the physics' OH factors of its half steps."""
        self.put_weights(t0 + ndyn / 2.0)
        if self.physics is not None:
            self.physics.put_factors(t0, ndyn)

    def interpolate(self, st):
        """pu, pv of every region from the meteo instants with the device-held weights."""
        for r in self.zoom.regions():
            (pu0, pv0), (pu1, pv1) = self.meteo[r]
            _interp(st[r]["pu"], pu0, pu1, self.w)
            _interp(st[r]["pv"], pv0, pv1, self.w)

    # -------------------------------------------------------------- Check_CFL, the step
    def _rehearse(self, st, i, n, ndyn):
        P.rehearse_step(self.zoom, st, ndyn)

    def check_cfl(self, t0):
        """Check_CFL on the copy of m and sp (Forward._carry); (ndyn, n, iterations)."""
        for r in self.zoom.regions():
            for name in ("m", "sp"):
                self.cfl_st[r][name].assign(self.st[r][name])

        def interpolate(zoom, st, i, ndyn):
            self.put_weights(t0 + (i - 0.5) * ndyn)
            self.interpolate(st)

        return P.check_cfl(self.zoom, self.cfl_st, self.ndyn_max, self.nread // self.ndyn_max, self.nread,
                           interpolate)  # fmt: skip

    def step(self, t0, ndyn):
        """One step from t0 (Forward._step): meteo at the middle, Setup_MassFlow, the sequence."""
        self.put_step_inputs(t0, ndyn)
        self.enqueue_step(ndyn)

    def enqueue_step(self, ndyn):
        st = self.st
        self.interpolate(st)
        P.setup_massflow(self.zoom, st, ndyn)
        kw = {"limits": self.limits}
        conv = None
        if self.physics is not None:
            conv, kw2 = self.physics.prepare(self, ndyn)
            kw.update(kw2)
        P.step(self.zoom, st, conv, ndyn, **kw)

    def interval(self, graph=False):
        """One read interval: Check_CFL, then its steps.  Returns (ndyn, n)."""
        t0 = self.t
        if graph:
            return self._interval_graph(t0)
        ndyn, n, _ = self.check_cfl(t0)
        for s in range(n):
            self.step(t0 + s * ndyn, ndyn)
        self.dev.sync()
        self.t = t0 + self.nread
        return ndyn, n

    # -------------------------------------------------------------- the captured interval
    def _enqueue_interval(self):
        """Check_CFL's rehearsal of one step at ndyn = nread and that step, speculatively: the
        step never reads the rehearsal's outcome (the host reads its flag after the replay), so
        the rehearsal runs on its own context -- its own Check_CFL flag, search counters and
        scratch -- beside the step, on the copies of m and sp taken at the interval's start.
        With physics each region's Calc_Kzz and rate constants also run on a side context from
        after Setup_MassFlow to the region's first convection, which is the first to read them.
        Every kernel gets the inputs of the sequential order; only the overlap is new."""
        zoom, cst, st = self.zoom, self.cfl_st, self.st
        lib = st.lib
        # the speculation's backup and the rehearsal's m and sp: one launch of every copy
        table, n, most = self._prologue
        N.check(self.dev.L.gb_copy_many(self.dev.h, table.ptr, n, most), "gb_copy_many")
        fork = self.dev.event()
        fork.record()
        self.aux_cfl.wait(fork)
        with self.dev.redirect(self.aux_cfl):
            self._enqueue_rehearsal()
        rehearsed = self.aux_cfl.event()
        rehearsed.record()
        self.interpolate(st)
        # Setup_MassFlow first: it rebuilds a parent's mass over a child's footprint and with it
        # the parent's sp (m2phlb), which Calc_Kzz reads
        P.setup_massflow(zoom, st, self.nread)
        kw = {"limits": self.limits}
        conv = None
        joins = []
        forked = None
        sides = (self.prep or []) + (self.aux or [])
        if self.physics is not None:
            self.physics.prepare_step(self.nread)
        if sides:  # the side contexts start from the step's own setup
            forked = self.dev.event()
            forked.record()
            for aux in sides:
                aux.wait(forked)
        if self.physics is not None:
            if self.prep:
                # each region's Calc_Kzz on a stream of its own: beside the region's advection
                # too, which a child runs on its own side context
                for r, prep in zip(zoom.regions(), self.prep, strict=True):
                    with self.dev.redirect(prep):
                        self.physics.prepare_region(self, r)
                    joins.append(prep.event())
                    joins[-1].record()
                # a region's side stream joins at the region's first convection (dkg; the rate
                # constants follow in chemistry).  Until then the step's advection and exchange
                # run beside it: they read and write none of Calc_Kzz's arrays (sp, pu, pv, t, q
                # in; dkg, krates out) -- sp changes only in m2phlb after the region's first v
                self.physics.pending = {r: (self.dev, j) for r, j in zip(zoom.regions(), joins, strict=True)}
            conv, kw2 = self.physics.driver_args()
            kw.update(kw2)
        sched = None
        if self.aux is not None and zoom.nregions > 1 and spreadable(zoom):
            # the step's bodies spread over one stream per region (pydyn_gb300.schedule)
            # region 1's own side context (its bodies run on the run's stream) takes its physics
            # on the far segment
            sched = Scheduler(self.dev, {r: aux for r, aux in zip(zoom.regions(), self.aux, strict=True) if r != 1},
                              far=self.aux[0] if self.physics is not None else None)
            for name in ("sources", "chemistry"):
                if name in kw:
                    kw[name] = scheduled_physics(sched, kw[name], name)
            st.lib = ScheduledLib(lib, sched)
        try:
            P.step(zoom, st, conv, self.nread, **kw)
        finally:
            st.lib = lib
        if sched is not None:
            sched.join()
        if self.physics is not None:
            self.physics.join_all()
        for aux in sides:  # every side stream is joined before the capture ends
            done = aux.event()
            done.record()
            self.dev.wait(done)
            joins.append(done)
        self.dev.wait(rehearsed)
        self._fork_events = (fork, rehearsed, forked, joins, sched.keep if sched else None)  # alive until the capture ends

    def _enqueue_rehearsal(self):
        """Check_CFL's rehearsal of one step on the copy (save, which clears the flag, meteo, the
        mass-only operators, restore), enqueued on whatever context the device points to."""
        cst, lib = self.cfl_st, self.st.lib
        lib.save(cst, "check_cfl", ("m", "am", "bm", "cm"))
        self.interpolate(cst)
        self._rehearse(cst, 1, 1, self.nread)
        lib.restore(cst, "check_cfl")

    def _interval_graph(self, t0):
        if self.nread // self.ndyn_max != 1:
            raise NotImplementedError("the captured interval is one step at ndyn = nread")
        if "interval" not in self.graphs:
            # the first interval runs uncaptured: every device constant and scratch array the
            # bodies create lazily exists before capture (allocation is not capturable)
            out = self.interval(graph=False)
            self.capture_interval()
            return out
        self.enqueue_interval_async(t0)
        return self.settle_interval(t0)

    def capture_interval(self):
        """(Re)capture the interval graph with the context's current launch shapes; the run has
        made one uncaptured interval before (its lazily made device arrays exist)."""
        if not hasattr(self, "_spec"):
            self._spec = {(r, k): DevArray.zeros(self.dev, *((lo, lo + n - 1) for lo, n in
                                                         zip(a.lower, a.shape, strict=True)))
                          for r in self.zoom.regions() for k, a in self.st[r].items() if k in SPECULATED}  # fmt: skip
            pairs = [(self._spec[(r, k)], self.st[r][k]) for r in self.zoom.regions() for k in SPECULATED]
            pairs += [(self.cfl_st[r][k], self.st[r][k]) for r in self.zoom.regions() for k in ("m", "sp")]
            for dst, src in pairs:  # whole arrays of one layout: flat copies
                if not (dst.contiguous() and src.contiguous() and dst.shape == src.shape and dst.dtype == src.dtype):
                    raise RuntimeError("capture_interval: a speculated array is not a whole contiguous array")
            self._prologue = copy_table(self.dev, pairs)
        self.st.lib.save(self.cfl_st, "check_cfl", ("m", "am", "bm", "cm"))
        if self.aux_cfl is None:
            # the captured interval's side contexts, their work spaces and scratch sized by one
            # uncaptured run of what they will run (harmless: the rehearsal's copy is refilled at
            # every interval's start, and every step recomputes what Calc_Kzz writes)
            self.dev.sync()
            if MAIN_PRIORITY:
                self.dev.set_priority(MAIN_PRIORITY)
            self.aux_cfl = Device(self.dev.ordinal)
            with self.dev.redirect(self.aux_cfl):
                self._enqueue_rehearsal()
            self.aux_cfl.sync()
            if CFL_PRIORITY:
                self.aux_cfl.set_priority(CFL_PRIORITY)
            if self.physics is not None and self.physics.full:
                # one per region for Calc_Kzz, its work space sized by an uncaptured run of it
                self.prep = [Device(self.dev.ordinal) for _ in self.zoom.regions()]
                for r, prep in zip(self.zoom.regions(), self.prep, strict=True):
                    with self.dev.redirect(prep):
                        self.physics.prepare_region(self, r)
                    prep.set_priority(KZZ_PRIORITY)
                    prep.sync()
            if self.zoom.nregions > 1 and spreadable(self.zoom):
                # one per region for a child's share of the step, its work space as large as the
                # run's own grew in its uncaptured interval.  Its streams get the highest
                # priority (CHILD_PRIORITY): the block scheduler then serves a child's chain before
                # the wide kernels beside it
                self.aux = [Device(self.dev.ordinal) for _ in self.zoom.regions()]
                for r, aux in zip(self.zoom.regions(), self.aux, strict=True):
                    aux.reserve_work(self.dev.work_size())
                    aux.set_priority(CHILD_PRIORITY if r != 1 else FAR_PRIORITY)
                    aux.sync()
        self.dev.sync()
        # the side contexts launch with the run's own shapes (gb_tune_set), re-read at every
        # capture: a tuner that changes the run's shapes re-captures
        shapes = self.dev.tuning()
        for side in (self.prep or []) + (self.aux or []) + ([self.aux_cfl] if self.aux_cfl is not None else []):
            side.tune(**shapes)
        self.graphs.pop("interval", None)
        side0 = self._side_launches()
        with self.dev.capture() as g:
            self._enqueue_interval()
        self.graphs["interval"] = g
        self._side_per_replay = self._side_launches() - side0  # the side branches' kernels

    def rehearsal_failed(self):
        """Whether the last captured interval's rehearsal rejected ndyn = nread (waits for the
        replay)."""
        self.dev.sync_stream()
        return (self.aux_cfl or self.dev).cfl_failed()

    def settle_interval(self, t0):
        """After a launched interval: read the rehearsal's flag; if Check_CFL rejected ndyn =
        nread, put the state back and redo the interval uncaptured.  Returns (ndyn, n)."""
        self.dev.sync_stream()  # the replay, the side contexts' branches included
        failed = self.aux_cfl.cfl_failed()  # the rehearsal's flag, on its context
        for aux in (self.prep or []) + (self.aux or []):
            aux.sync()  # errors of the side contexts' kernels (Calc_Kzz, a child's) are raised here
        if failed:  # the speculation was wrong: back to the interval's start
            for (r, k), a in self._spec.items():
                self.st[r][k].assign(a)
            self.dev.discard_status()  # the speculative step's own errors are not the run's
            self.t = t0
            return self.interval(graph=False)
        self.dev.sync()
        self.t = t0 + self.nread
        return self.nread, 1

    def close(self):
        """Give the device memory of both states, the meteo and the graphs back."""
        self.graphs.clear()
        for s in (self.st, self.cfl_st):
            s.free()
        for pairs in self.meteo.values():
            for pu, pv in pairs:
                pu.free()
                pv.free()
        for a in getattr(self, "_spec", {}).values():
            a.free()
        if hasattr(self, "_prologue"):
            self._prologue[0].free()
        if self.physics is not None:
            self.physics.free()
        self.w.free()
        for aux in (self.prep or []) + (self.aux or []) + ([self.aux_cfl] if self.aux_cfl is not None else []):
            aux.close()
        self.prep, self.aux, self.aux_cfl = None, None, None

    def _side_launches(self):
        side = (self.prep or []) + (self.aux or []) + ([self.aux_cfl] if self.aux_cfl is not None else [])
        return sum(aux.launches() for aux in side)

    def launches(self):
        """Kernels launched so far by the run's contexts, the captured side branches' included
        (a replay counts the main context's captured kernels there, the side ones here)."""
        return self.dev.launches() + self._side_launches() + self._replays * self._side_per_replay

    def enqueue_interval_async(self, t0):
        """The captured interval, launched without any host read (the benchmark's timed loop;
        the rehearsal flag is read once after the loop)."""
        self.put_step_inputs(t0, self.nread)
        self.graphs["interval"].launch()
        self._replays += 1


def copy_table(dev, pairs):
    """gb_copy_many's table of whole-array copies [(dst, src) DevArrays]: (device table, n, the
    largest byte count).  Every copy moves whole 8-byte elements: a count that is not a multiple
    of 8, or an empty copy, is refused here, since the kernel copies 8 bytes at a time."""
    rows = []
    for dst, src in pairs:
        nbytes = src.size * src.dtype.itemsize
        if nbytes <= 0 or nbytes % 8 or dst.size * dst.dtype.itemsize < nbytes:
            raise ValueError(f"copy_table: a copy of {nbytes} bytes into {dst.size * dst.dtype.itemsize} "
                             "(8-byte elements, non-empty, the destination at least as large)")  # fmt: skip
        rows.append((dst.ptr, src.ptr, nbytes))
    if len(rows) > 65535:
        raise ValueError("copy_table: at most 65535 copies in one launch")
    return DevArray.from_host(dev, np.array(rows, dtype=np.uint64)), len(rows), max(b for _, _, b in rows)


def _interp(dst, a, b, w):
    import ctypes

    L = dst.dev.L
    from . import _native as N

    vd, va, vb = dst.view(), a.view(), b.view()
    N.check(L.gb_interp(dst.dev.h, ctypes.byref(vd), ctypes.byref(va), ctypes.byref(vb), w.ptr), "gb_interp")
