"""Per-body device time of one eagerly enqueued interval: every body the driver calls through
`st.lib` is bracketed by CUDA events on the context's stream (pydyn's CudaBackend
profile_begin/end has the same role, gpu/backend.py:634-651)."""

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
            region = a[2] if len(a) > 2 and isinstance(a[2], int) else (1 if name.endswith("region1") else None)
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


def main(argv=None):
    """One eagerly enqueued interval of a configuration -- every kernel launched once, no graph,
    no pinned copies -- for a launch list under a profiler:

        python -m pydyn_gb300.profile --config glb3x2+nam1x1 --levels 34 --intervals 1

    With --fp64-rates it measures the GPU's FP64 issue rates instead (the step's compute ceiling).
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
    ap.add_argument("--physics", type=int, default=1, help="1: convection, Kzz, emission, chemistry; 0: advection")
    ap.add_argument("--lmax", type=int, default=None)
    ap.add_argument("--fp64-rates", action="store_true", help="measure the FP64 issue rates and exit")
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
    fw = Forward(dev, a.config, a.levels, a.seed, physics=bool(a.physics), lmax=a.lmax)
    n0 = dev.launches()
    for _ in range(a.intervals):
        fw.interval(graph=False)
    dev.sync()
    print(f"{a.intervals} interval(s) of {a.config}: {dev.launches() - n0} kernel launches")
    fw.close()
    dev.close()


if __name__ == "__main__":
    main()
