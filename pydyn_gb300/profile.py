"""Per-body device time of one eagerly enqueued interval: every body the driver calls through
`st.lib` is bracketed by CUDA events on the context's stream (pydyn's CudaBackend
profile_begin/end has the same role, gpu/backend.py:634-651).  And the timeline of a captured
interval: the GPU's timer stamped at each body's start and end on the stream it runs on
(`timeline`)."""

import functools
from collections import defaultdict

from . import zoom as Z


class BodyProfiler:
    """Wrap the lib's bodies with event pairs while active; report {name: [ms per call]}."""

    WRAPPED = ("_dynamu_region1", "_dynamv_region1", "_dynamw_region1", "_dynamu_child", "_dynamv_child",
               "_dynamw_child", "_dynamum_region1", "_dynamvm_region1", "_dynamwm", "_dynamum_child",
               "_dynamvm_child", "dynam0", "m2phlb1", "m2phlb", "convec_region", "sources_region",
               "chemistry_region", "put_xedges", "put_yedges", "mix_edges", "update_parent", "_coarsen_block",
               "coarsen_ambm", "_uncompress_xedges", "_uncompress_yedges", "save", "restore")  # fmt: skip

    # a run's physics object: its per-step preparation (Calc_Kzz) and its `s` / `c` callbacks
    PHYSICS = {"prepare": "calc_kzz", "sources": "sources_region", "chemistry": "chemistry_region"}

    def __init__(self, dev, physics=None):
        self.dev = dev
        self.physics = physics
        self.pairs = defaultdict(list)
        self.launches = defaultdict(int)
        self._saved = {}

    def __enter__(self):
        for name in self.WRAPPED:
            f = getattr(Z, name, None)
            if f is None or name in self._saved:
                continue
            self._saved[name] = f
            setattr(Z, name, self._wrap(name, f))
        if self.physics is not None:
            for attr, name in self.PHYSICS.items():
                setattr(self.physics, attr, self._wrap(name, getattr(self.physics, attr)))
        return self

    def __exit__(self, *exc):
        for name, f in self._saved.items():
            setattr(Z, name, f)
        self._saved.clear()
        if self.physics is not None:
            for attr in self.PHYSICS:
                self.physics.__dict__.pop(attr, None)
        return False

    def _wrap(self, name, f):
        dev = self.dev

        @functools.wraps(f)
        def call(*a, **k):
            e0, e1 = dev.event(), dev.event()
            n0 = dev.launches()
            e0.record()
            out = f(*a, **k)
            e1.record()
            if name.endswith("region1"):  # region 1's bodies take no region argument
                region = 1
            else:
                region = a[2] if len(a) > 2 and isinstance(a[2], int) and not isinstance(a[2], bool) else None
            key = name if region is None else f"{name}@{region}"
            self.pairs[key].append((e0, e1))
            self.launches[key] += dev.launches() - n0
            return out

        return call

    def report(self):
        """{body: (calls, total ms, kernel launches)}."""
        self.dev.sync()
        out = {}
        for name, pairs in self.pairs.items():
            ms = [a.elapsed_ms(b) for a, b in pairs]
            out[name] = (len(ms), sum(ms), self.launches[name])
        return out


class Timeline:
    """Stamps of the GPU's global timer (gb_stamp) at the start and end of a captured interval's
    parts, each on the stream the part runs on: the scheduler's region bodies, the Check_CFL
    rehearsal, each region's Calc_Kzz, Setup_MassFlow and the interval's ends."""

    def __init__(self, fw, slots=8192):
        import numpy as np

        from .device import DevArray

        self.fw, self.dev = fw, fw.dev
        self.buf = DevArray.zeros(fw.dev, (0, slots - 1), dtype=np.int64)
        self.slots = slots
        self.marks = []  # slot -> (stream, part, "b" | "e")
        self._saved = []

    def _stream(self):
        fw, h = self.fw, self.dev.h
        if h == self._main:
            return "main"
        if fw.aux_cfl is not None and h == fw.aux_cfl.h:
            return "rehearsal"
        for kind, ctxs in (("kzz", fw.prep), ("region", fw.aux)):
            for r, c in zip(fw.zoom.regions(), ctxs or (), strict=False):
                if h == c.h:
                    return f"{kind}{r}"
        return "other"

    def stamp(self, part, kind):
        from . import _native as N

        slot = len(self.marks)
        if slot >= self.slots:
            raise RuntimeError("Timeline: out of slots")
        self.marks.append((self._stream(), part, kind))
        N.check(self.dev.L.gb_stamp(self.dev.h, self.buf.ptr, slot), "gb_stamp")

    def _bracket(self, owner, attr, part_of):
        f = getattr(owner, attr)
        tl = self

        @functools.wraps(f)
        def call(*a, **k):
            part = part_of(*a, **k)
            tl.stamp(part, "b")
            out = f(*a, **k)
            tl.stamp(part, "e")
            return out

        self._saved.append((owner, attr, f))
        setattr(owner, attr, call)

    def __enter__(self):
        from contextlib import contextmanager

        from . import forward as F
        from . import physics as P
        from . import plan as PL
        from . import schedule as S

        self._main = self.dev.h
        tl = self
        body = S.Scheduler.body

        @contextmanager
        def stamped(sched, name, region):
            with body(sched, name, region):
                tl.stamp(f"{name}@{region}", "b")
                yield
                tl.stamp(f"{name}@{region}", "e")

        self._saved.append((S.Scheduler, "body", body))
        S.Scheduler.body = stamped
        self._bracket(F.Forward, "_enqueue_rehearsal", lambda *a, **k: "check_cfl")
        self._bracket(P.Physics, "prepare_region", lambda self_, fwd, r: f"calc_kzz@{r}")
        self._bracket(PL, "setup_massflow", lambda *a, **k: "setup_massflow")
        self._bracket(F.Forward, "_enqueue_interval", lambda *a, **k: "interval")
        return self

    def __exit__(self, *exc):
        for owner, attr, f in reversed(self._saved):
            setattr(owner, attr, f)
        self._saved.clear()
        return False

    def report(self):
        """[(stream, part, start us, end us)] of the last replay, from the interval's first stamp."""
        t = self.buf.host()[: len(self.marks)]
        t0 = int(t.min())
        open_, rows = {}, []
        for (stream, part, kind), v in zip(self.marks, t, strict=True):
            key = (stream, part)
            if kind == "b":
                open_.setdefault(key, []).append(int(v))
            elif open_.get(key):
                b = open_[key].pop(0)
                rows.append((stream, part, (b - t0) / 1e3, (int(v) - t0) / 1e3))
        return sorted(rows, key=lambda r: r[2])


def timeline(fw, replays=5):
    """The timeline of the run's captured interval: capture it with stamps, replay it, and return
    Timeline.report() of the last replay."""
    if "interval" not in fw.graphs:
        fw.interval(graph=True)
    with Timeline(fw) as tl:
        fw.capture_interval()
    for _ in range(replays):
        fw.enqueue_interval_async(fw.t)
        fw.settle_interval(fw.t)
    rows = tl.report()
    fw.capture_interval()  # the interval without stamps again
    tl.buf.free()
    return rows


def main(argv=None):
    """One eagerly enqueued interval of a configuration -- every kernel launched once, no graph,
    no pinned copies -- for a launch list under a profiler:

        python -m pydyn_gb300.profile --config glb3x2+nam1x1 --levels 34 --intervals 1

    With --fp64-rates it measures the GPU's FP64 issue rates instead (the step's compute ceiling);
    with --timeline it prints the timeline of the captured interval's streams.
    """
    import argparse
    import sys
    from pathlib import Path

    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    ap = argparse.ArgumentParser(description=main.__doc__.split("\n")[0])
    ap.add_argument("--config", default="glb3x2+nam1x1")
    ap.add_argument("--levels", type=int, default=34)
    ap.add_argument("--seed", type=int, default=42)
    ap.add_argument("--intervals", type=int, default=1)
    ap.add_argument("--physics", default="1",
                    help="1: convection, Kzz, emission, chemistry; convection: convection alone on a given dkg "
                         "(pydyn's GPU benchmark inputs); 0: advection")  # fmt: skip
    ap.add_argument("--lmax", type=int, default=None)
    ap.add_argument("--fp64-rates", action="store_true", help="measure the FP64 issue rates and exit")
    ap.add_argument("--timeline", action="store_true", help="the captured interval's timeline per stream")
    a = ap.parse_args(argv)
    from __graft_entry__ import build

    build()
    from .device import Device
    from .forward import Forward

    dev = Device(0)
    if a.fp64_rates:
        for name, rate in dev.fp64_rates().items():
            print(f"{name}: {rate:.1f} G instructions/s")
        dev.close()
        return
    physics = {"1": True, "0": False}.get(a.physics, a.physics)
    fw = Forward(dev, a.config, a.levels, a.seed, physics=physics, lmax=a.lmax)
    if a.timeline:
        for _ in range(3):
            fw.interval(graph=True)
        rows = timeline(fw)
        end = max(r[3] for r in rows)
        print(f"captured interval of {a.config}: {end:.1f} us from its first stamp to its last")
        print(f"{'stream':10s} {'part':34s} {'start us':>9s} {'end us':>9s} {'us':>8s}")
        for stream, part, b, e in rows:
            print(f"{stream:10s} {part[:34]:34s} {b:9.1f} {e:9.1f} {e - b:8.1f}")
        busy = defaultdict(float)
        for stream, part, b, e in rows:
            if part != "interval":
                busy[stream] += e - b
        print("busy per stream (us, parts summed):", {k: round(v, 1) for k, v in sorted(busy.items())})
        fw.close()
        dev.close()
        return
    n0 = dev.launches()
    for _ in range(a.intervals):
        fw.interval(graph=False)
    dev.sync()
    print(f"{a.intervals} interval(s) of {a.config}: {dev.launches() - n0} kernel launches")
    fw.close()
    dev.close()


if __name__ == "__main__":
    main()
