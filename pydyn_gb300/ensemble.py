"""A batched ensemble of independent runs on one GPU.

The production mix is 256 members: 128 glb6x4, 96 glb3x2 and 32 glb3x2 + nam1x1 trees, all with
physics, each member with its own seed for a wind scaling in [0.9, 1.1] and for its physics
inputs (CH4 flux, convection, Kzz and chemistry fields).  The members of a class share the
class's flow (its meteo seed), scaled.

Every member is a plain run (pydyn_gb300.forward.Forward) on its own context: its own stream,
status word, work space and captured interval graph (one CUDA graph per member and time step).
A step launches the graphs of all members without waiting.  The members are spread over
`width` lanes, longest first (each member's cost is its class's measured step time); a lane is
a chain of members whose launches wait on the previous member's event, so `width` members are
in flight at any time and the GPU packs the CTAs of their kernels side by side: the small
members' latency-bound kernels fill the SMs that the large members' leave idle.  Then the host
reads each member's Check_CFL flag and, for any member whose rehearsal rejected ndyn = nread,
puts the state back and redoes that member's interval uncaptured -- what its solo run does.

Each member launches exactly the kernels of its solo run on its own data, in the same order on
its own stream, so it is bitwise its solo run (the tests check that).  The width and each
class's launch shapes come from the autotuner (pydyn_gb300.tune).

Lanes beyond the device's hardware queues serialise behind one another: a process that runs an
ensemble sets CUDA_DEVICE_MAX_CONNECTIONS (up to 32) before its first CUDA call."""

from dataclasses import dataclass

import numpy as np

from .device import Device
from .forward import Forward
from .synth import ENSEMBLE_CLASSES as CLASSES
from .synth import ENSEMBLE_MIX as MIX


@dataclass(frozen=True)
class MemberSpec:
    """One member: its class, tree and levels, the class's meteo seed, its own physics seed and
    wind scale."""

    index: int
    cls: str
    tree: str
    lm: int
    lmax: int
    physics: bool
    seed: int
    member_seed: int
    wind_scale: float

    def forward(self, dev):
        """The member's run on a device context: the same construction as its solo run."""
        return Forward(dev, self.tree, self.lm, seed=self.seed, physics=self.physics,
                       lmax=self.lmax if self.physics else None, wind_scale=self.wind_scale,
                       physics_seed=self.member_seed)  # fmt: skip


def member_specs(mix=MIX, seed=2024, physics=True, classes=None):
    """The members of a mix ((class, count), ...), numbered in order; the wind scales and the
    members' seeds are drawn from `seed`."""
    classes = CLASSES if classes is None else classes
    rng = np.random.default_rng([seed, 15485863])
    out = []
    for cls, count in mix:
        tree, lm, lmax, cseed = classes[cls]
        for _ in range(count):
            k = len(out)
            scale = 0.9 + 0.2 * float(rng.random())
            out.append(MemberSpec(k, cls, tree, lm, lmax, physics, cseed, seed * 1_000_003 + k, scale))
    return out


def lanes_for(costs, width):
    """Members (by cost) onto `width` lanes, longest first onto the least loaded lane; each
    lane lists its members in launch order."""
    width = max(1, min(width, len(costs)))
    order = sorted(range(len(costs)), key=lambda k: (-costs[k], k))
    load = [0.0] * width
    lanes = [[] for _ in range(width)]
    for k in order:
        j = min(range(width), key=lambda q: (load[q], q))
        lanes[j].append(k)
        load[j] += costs[k]
    return [lane for lane in lanes if lane]


class Ensemble:
    """The members of `specs`, each on its own context of `device`; `shapes` maps a class to
    its launch shapes ({name: value}, pydyn_gb300.device.Device.tune)."""

    def __init__(self, specs, device=0, width=None, shapes=None, costs=None):
        self.specs = list(specs)
        self.devs, self.runs = [], []
        shapes = shapes or {}
        for s in self.specs:
            dev = Device(device)
            if s.cls in shapes:
                dev.tune(**shapes[s.cls])
            self.devs.append(dev)
            self.runs.append(s.forward(dev))
        self.events = [dev.event() for dev in self.devs]
        self.costs = costs or {}
        self.set_width(width or len(self.specs))
        self.t = 0.0
        self.captured = False
        self.redone = 0  # member intervals redone uncaptured after a rejected rehearsal

    def cost(self, k):
        """Member k's relative cost: its class's measured step time, else its cell count."""
        s = self.specs[k]
        if s.cls in self.costs:
            return float(self.costs[s.cls])
        z = self.runs[k].zoom
        return float(sum(z.g(r).im * z.g(r).jm * z.g(r).tref for r in z.regions()) * z.lm)

    def set_width(self, width):
        self.width = max(1, min(int(width), len(self.specs)))
        self.lanes = lanes_for([self.cost(k) for k in range(len(self.specs))], self.width)

    def capture(self):
        """Each member's first interval, uncaptured, and the capture of its interval graph."""
        for fw in self.runs:
            fw.interval(graph=True)
        self.t = self.runs[0].t
        self.captured = True

    def launch(self, before=None, after=None):
        """Every member's captured interval from the ensemble's time, no host wait.  before(k)
        and after(k) enqueue a member's own copies around its graph (the end-to-end path)."""
        t0 = self.t
        for lane in self.lanes:
            prev = None
            for k in lane:
                fw = self.runs[k]
                # the step's inputs go up while the member's stream is idle (an upload from a
                # host temporary waits for its stream), then the stream waits for the lane
                fw.put_step_inputs(t0, fw.nread)
                if prev is not None:
                    self.devs[k].wait(self.events[prev])
                if before is not None:
                    before(k)
                fw.graphs["interval"].launch()
                fw._replays += 1
                if after is not None:
                    after(k)
                self.events[k].record()
                prev = k

    def settle(self):
        """After launch(): every member's Check_CFL verdict; rejected members redo their
        interval uncaptured.  Advances the ensemble's time."""
        t0 = self.t
        for fw in self.runs:
            if fw.settle_interval(t0) != (fw.nread, 1):
                self.redone += 1
        self.t = t0 + self.runs[0].nread

    def step(self, before=None, after=None):
        """One read interval of every member, all in flight together (the batched step)."""
        if not self.captured:
            self.capture()
            return
        self.launch(before, after)
        self.settle()

    def step_looped(self):
        """The same interval as the plain step looped over the members: each member's graph
        launched and finished before the next one starts."""
        if not self.captured:
            self.capture()
            return
        t0 = self.t
        for fw in self.runs:
            fw.enqueue_interval_async(t0)
            if fw.settle_interval(t0) != (fw.nread, 1):
                self.redone += 1
        self.t = t0 + self.runs[0].nread

    def sync(self):
        for dev in self.devs:
            dev.sync()

    def close(self):
        for fw in self.runs:
            fw.close()
        self.runs.clear()
        self.events.clear()
        for dev in self.devs:
            dev.close()
        self.devs.clear()
