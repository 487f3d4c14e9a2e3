"""The bodies of a captured step spread over one stream per region, ordered by what they touch.

Every body of a step belongs to a region (its region argument).  Region 1's bodies stay on the
run's own stream; each child's go to the child's side context (its own stream, work space,
scratch and status word).  Every body declares which parts of the state it reads and writes:

    p_far    region 1's owned columns outside every child's footprint
    p_edge   region 1's owned columns inside a footprint (under a child's edge ring)
    p_core   region 1's columns under a child's scope (not owned)
    c_in     a child's scope: its owned columns, fluxes, pressures, physics arrays
    c_ring   a child's edge ring inside its interior (xr / yr cells wide)
    c_halo   a child's halo cells

put_xedges / put_yedges of region 1 read the parent around and at a footprint's edge and write
the child's halo and edge ring; update_parent writes the whole footprint (p_edge, p_core).
Region 1's physics runs as two bodies, one per segment of its owned columns (far, edge): the
far segment shares nothing with a child's pass.

A body waits for the last writer of every part it reads, and for the last writer and every
reader since of every part it writes, when those ran on another stream (recorded events), as
the sequential order would have them.  Each stream keeps its own order.  So every body sees the
inputs of the sequential order, and the results are bitwise those of the sequential step.  What
runs side by side is what touches disjoint parts.  In the parent's first half, its convection,
emission and chemistry on the far segment run beside the child's whole first pass.  In the
second half, the child's chemistry, emission and convection (its scope) run beside the parent's
advection.

Only trees whose children are leaves are spread (a grandchild makes region 2 both a parent and
a child); others keep the sequential order on one stream."""

from contextlib import contextmanager

PARENT_ALL = frozenset({"p_far", "p_edge", "p_core"})
REGION1_BODIES = ("_dynamu_region1", "_dynamv_region1", "_dynamw_region1", "m2phlb1")  # no region argument
CHILD_ALL = frozenset({"c_in", "c_ring", "c_halo"})
PHYSICS = ("convec_region", "sources", "chemistry")


def spreadable(zoom):
    """Whether a tree's bodies can be spread: every region below region 1 is a leaf."""
    return all(not zoom.children[r] for r in zoom.regions() if r != 1)


def parts(name, region):
    """(reads, writes) of a body of `region`, as parts of the state."""
    if region == 1 and name in ("outer_x_faces_zeroed", "outer_y_faces_zeroed"):
        return set(), set()  # region 1 has no outer faces to zero
    body, _, seg = name.partition(":")
    if region == 1:
        if body in PHYSICS:
            own = {"far": {"p_far"}, "edge": {"p_edge"}}.get(seg, {"p_far", "p_edge"})
            return own, own
        if body in ("put_xedges", "put_yedges"):  # the parent at a footprint -> the child's halo and ring
            return PARENT_ALL, {"c_halo", "c_ring"}
        return PARENT_ALL, PARENT_ALL  # advection, m2phlb1
    if body in PHYSICS:
        return {"c_in"}, {"c_in"}
    if body == "update_parent":  # the child's block sums -> the parent's footprint
        return CHILD_ALL, {"p_edge", "p_core"}
    return CHILD_ALL, CHILD_ALL  # advection, the edge exchanges within the child, m2phlb


class Scheduler:
    """The dependency tracker of one captured step: `streams` maps a region to the Device its
    bodies run on (None: the run's own); `far`, when given, is the Device region 1's physics on
    its far segment runs on (it shares nothing with a child, so it need not wait in the run's
    stream behind the edge segment's bodies, which wait for update_parent)."""

    def __init__(self, dev, streams, far=None):
        self.dev, self.streams, self.far = dev, streams, far
        self.writer = {}  # part -> (stream key, sequence number, event)
        self.readers = {}  # part -> [(stream key, sequence number, event)]
        self.seq = 0
        self.waited = {}  # (stream key, other stream key) -> the latest sequence number waited for
        self.last = {}  # stream key -> its last event
        self.keep = []  # the events, alive until the capture ends

    def _key(self, name, region):
        if region == 1 and self.far is not None and name.endswith(":far") and name.partition(":")[0] in PHYSICS:
            return "far"
        return region if self.streams.get(region) is not None else 1

    def _device(self, key):
        return self.far if key == "far" else (self.streams.get(key) if key != 1 else None)

    @contextmanager
    def body(self, name, region):
        """Run a body's enqueues inside this block on the region's stream, after its waits."""
        key = self._key(name, region)
        reads, writes = parts(name, region)
        waits = []
        for p in reads | writes:
            w = self.writer.get(p)
            if w is not None:
                waits.append(w)
        for p in writes:
            waits.extend(self.readers.get(p, []))
        latest = {}  # another stream -> its latest event to wait for (a stream's events are ordered)
        for k, n, ev in waits:
            if k != key and n > self.waited.get((key, k), 0) and (k not in latest or n > latest[k][0]):
                latest[k] = (n, ev)
        for k, (n, _) in latest.items():
            self.waited[(key, k)] = n
        side = self._device(key)
        ctx = self.dev.redirect(side) if side is not None else _nothing()
        with ctx:
            for _, ev in latest.values():
                self.dev.wait(ev)
            yield
            ev = self.dev.event()
            ev.record()
        self.seq += 1
        entry = (key, self.seq, ev)
        self.keep.append(ev)
        self.last[key] = ev
        for p in writes:
            self.writer[p] = entry
            self.readers[p] = []
        for p in reads - writes:
            self.readers.setdefault(p, []).append(entry)

    def join(self):
        """The run's own stream waits for every other stream's last body (the far segment's
        included)."""
        for k, ev in self.last.items():
            if k != 1:
                self.dev.wait(ev)


@contextmanager
def _nothing():
    yield


class ScheduledLib:
    """The region bodies of `lib` run through a Scheduler (bodies, and the context managers
    that bracket an advection)."""

    def __init__(self, lib, sched):
        self._lib, self._sched = lib, sched

    def __getattr__(self, name):
        f = getattr(self._lib, name)
        if not callable(f) or name.startswith("__"):
            return f
        sched = self._sched

        if name in ("outer_x_faces_zeroed", "outer_y_faces_zeroed"):

            @contextmanager
            def bracket(zoom, st, region, *a, **k):
                with sched.body(name, region):
                    cm = f(zoom, st, region, *a, **k)
                    cm.__enter__()
                try:
                    yield
                finally:
                    with sched.body(name, region):
                        cm.__exit__(None, None, None)

            return bracket

        if name in REGION1_BODIES:

            def body1(zoom, st, *a, **k):
                with sched.body(name, 1):
                    return f(zoom, st, *a, **k)

            return body1

        if name == "convec_region":

            def convec(zoom, st, region, conv, *a, **k):
                segs = conv.segment_names(region) if region == 1 else []
                if len(segs) < 2:
                    with sched.body(name, region):
                        return f(zoom, st, region, conv, *a, **k)
                for seg in segs:  # one body per segment of region 1's owned columns
                    with sched.body(f"{name}:{seg}", region), conv.only_segment(seg):
                        f(zoom, st, region, conv, *a, **k)
                return None

            return convec

        def body(zoom, st, region, *a, **k):
            with sched.body(name, region):
                return f(zoom, st, region, *a, **k)

        return body


def scheduled_physics(sched, fn, name):
    """A physics callback (sources, chemistry: a bound method of the run's Physics) through the
    Scheduler, one body per segment of region 1's owned columns."""
    phys = fn.__self__

    def call(zoom, st, region):
        segs = phys.segment_names(region) if region == 1 else []
        if len(segs) < 2:
            with sched.body(name, region):
                return fn(zoom, st, region)
        for seg in segs:
            with sched.body(f"{name}:{seg}", region), phys.only_segment(seg):
                fn(zoom, st, region)
        return None

    return call
