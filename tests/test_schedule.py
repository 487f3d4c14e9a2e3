"""The region scheduler's dependency tracking (pydyn_gb300.schedule), on the host with a fake
device that records which stream each event is recorded on and which stream waits for it."""

from contextlib import contextmanager

import pytest

from pydyn_gb300 import schedule as S


class FakeEvent:
    def __init__(self, dev):
        self.dev, self.stream = dev, None

    def record(self):
        self.stream = self.dev.current
        self.dev.log.append(("record", self.stream, id(self)))


class FakeDev:
    def __init__(self):
        self.current, self.log = "main", []

    def event(self):
        return FakeEvent(self)

    def wait(self, ev):
        self.log.append(("wait", self.current, ev.stream))

    @contextmanager
    def redirect(self, other):
        old, self.current = self.current, other
        try:
            yield other
        finally:
            self.current = old


def _run(bodies, far=None):
    dev = FakeDev()
    sched = S.Scheduler(dev, {2: "child"}, far=far)
    waits = []
    for name, region in bodies:
        n0 = len(dev.log)
        with sched.body(name, region):
            pass
        waits.append([e for e in dev.log[n0:] if e[0] == "wait"])
    return waits


def test_parts_follow_the_kernels():
    assert S.parts("put_xedges", 1) == (S.PARENT_ALL, {"c_halo", "c_ring"})
    assert S.parts("update_parent", 2) == (S.CHILD_ALL, {"p_edge", "p_core"})
    assert S.parts("convec_region:far", 1) == ({"p_far"}, {"p_far"})
    assert S.parts("chemistry:edge", 1) == ({"p_edge"}, {"p_edge"})
    assert S.parts("chemistry", 2) == ({"c_in"}, {"c_in"})
    assert S.parts("outer_x_faces_zeroed", 1) == (set(), set())


def test_far_physics_beside_the_child_edge_after_it():
    waits = _run([
        ("_dynamu_region1", 1),       # 0: the parent's advection
        ("put_xedges", 1),            # 1: the parent -> the child's halo and ring
        ("_dynamu_child", 2),         # 2: the child waits for the edges
        ("update_parent", 2),         # 3: the child's sums -> the footprint
        ("convec_region:far", 1),     # 4: beside the child
        ("convec_region:edge", 1),    # 5: after update_parent
        ("put_xedges", 1),            # 6: after the child's last use of its halo and ring
        ("m2phlb1", 1),               # 7: the whole parent, after update_parent
    ])  # fmt: skip
    assert waits[2] == [("wait", "child", "main")]  # after the parent's advection and edges
    assert waits[3] == []  # the child's stream waited for those already (at 2)
    assert waits[4] == []
    assert waits[5] == [("wait", "main", "child")]  # after update_parent, the child's last body
    assert waits[6] == []  # implied by 5
    assert waits[7] == []


def test_child_physics_beside_the_parent_advection():
    waits = _run([
        ("update_parent", 2),
        ("_dynamw_region1", 1),       # the parent's z: waits for update_parent
        ("put_yedges", 1),            # writes the child's halo and ring
        ("chemistry", 2),             # the child's scope: nothing to wait for
        ("convec_region", 2),
        ("_dynamw_child", 2),         # the child's advection: waits for put_yedges
    ])  # fmt: skip
    assert waits[1] == [("wait", "main", "child")]
    assert waits[3] == [] and waits[4] == []
    assert waits[5] == [("wait", "child", "main")]


def test_far_segment_physics_on_its_own_stream():
    waits = _run([
        ("_dynamw_region1", 1),       # 0: the parent's z on the run's stream
        ("convec_region:far", 1),     # 1: on the far stream, after the parent's z
        ("convec_region:edge", 1),    # 2: the run's stream, nothing new to wait for
        ("chemistry:far", 1),         # 3: the far stream's own order
        ("update_parent", 2),         # 4: the child writes the footprint (edge, core)
        ("chemistry:edge", 1),        # 5: after update_parent
        ("m2phlb1", 1),               # 6: the whole parent: after the far stream's last body
    ], far="far")  # fmt: skip
    assert waits[1] == [("wait", "far", "main")]
    assert waits[2] == [] and waits[3] == []
    assert waits[4] == [("wait", "child", "main")]  # the edge segment's readers on the run's stream
    assert waits[5] == [("wait", "main", "child")]
    assert waits[6] == [("wait", "main", "far")]


def test_spreadable_trees():
    from pydyn_gb300 import synth

    assert S.spreadable(synth.tree("two", 4))
    assert S.spreadable(synth.tree("glb3x2+nam1x1", 4))
    assert not S.spreadable(synth.tree("three", 4))


@pytest.mark.gpu
def test_timeline_of_a_spread_interval(built):
    """The captured interval's timeline: the region bodies on their streams, inside the interval,
    and the interval graph itself unchanged afterwards (its digest still the run's)."""
    from pydyn_gb300.device import Device
    from pydyn_gb300.forward import Forward
    from pydyn_gb300.profile import timeline

    dev = Device(0)
    fw = Forward(dev, "two", 8, seed=3, physics=True, lmax=8)
    for _ in range(2):
        fw.interval(graph=True)
    rows = timeline(fw, replays=2)
    streams = {s for s, _, _, _ in rows}
    assert {"main", "region2", "rehearsal", "kzz1", "kzz2"} <= streams
    (b0, e0), = [(b, e) for s, p, b, e in rows if p == "interval"]
    assert b0 == 0.0 and all(b0 <= b <= e <= e0 for _, p, b, e in rows)
    assert any(p.startswith("convec_region") and s == "region2" for s, p, _, _ in rows)
    fw.interval(graph=True)  # the recaptured interval still runs
    fw.close()
    dev.close()
