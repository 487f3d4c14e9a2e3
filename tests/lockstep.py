"""Run the package's operator sequence on the device and on the oracle side by side, comparing
every state array of every region after every body the driver calls, so a divergence is named
by the first body that produced it.  Test infrastructure (the oracle is the checker)."""

import numpy as np

STATE_FIELDS = ("m", "rm", "rxm", "rym", "rzm", "am", "bm", "cm", "pu", "pv", "sp", "phlb")


class Divergence(AssertionError):
    pass


def _bits(a):
    return np.ascontiguousarray(a, dtype="<f8").view(np.int64)


class LockState:
    """A pair (device ZoomState, oracle HostState); `lib` dispatches each body to both."""

    def __init__(self, dev_st, orc_st, fields=STATE_FIELDS, log=None):
        self.dev_st, self.orc_st, self.fields = dev_st, orc_st, fields
        self.zoom = dev_st.zoom
        self.nt = dev_st.nt
        self.log = log if log is not None else []
        self.lib = _Lib(self)

    def compare(self, where):
        for r in self.zoom.regions():
            for name in self.fields:
                d = self.dev_st[r][name].host()
                o = self.orc_st[r][name].data
                diff = _bits(d) != _bits(o)
                if diff.any():
                    idx = tuple(int(i) for i in np.argwhere(diff)[0])
                    raise Divergence(f"after {where}: region {r} {name}: {int(diff.sum())} values differ, first at "
                                     f"data index {idx}: device {d[idx]!r} oracle {o[idx]!r}")  # fmt: skip


class _Ctx:
    def __init__(self, a, b, lock, name):
        self.a, self.b, self.lock, self.name = a, b, lock, name

    def __enter__(self):
        self.a.__enter__()
        self.b.__enter__()
        self.lock.compare(self.name + " (enter)")
        return self

    def __exit__(self, *exc):
        self.a.__exit__(*exc)
        self.b.__exit__(*exc)
        if exc[0] is None:
            self.lock.compare(self.name + " (exit)")
        return False


class _Lib:
    def __init__(self, lock):
        self._lock = lock

    def __getattr__(self, name):
        lock = self._lock
        dev_f = getattr(lock.dev_st.lib, name)
        orc_f = getattr(lock.orc_st.lib, name)

        def call(*args, **kw):
            dargs = [lock.dev_st if a is lock else a for a in args]
            oargs = [lock.orc_st if a is lock else a for a in args]
            if name in ("outer_x_faces_zeroed", "outer_y_faces_zeroed"):
                return _Ctx(dev_f(*dargs, **kw), orc_f(*oargs, **kw), lock, name)
            d = dev_f(*dargs, **kw)
            o = orc_f(*oargs, **kw)
            lock.log.append(name)
            if name == "cfl_all_ok":
                if d != o:
                    raise Divergence(f"Check_CFL outcome: device {d} oracle {o}")
                return d
            lock.compare(f"{name}{tuple(a for a in args[2:] if isinstance(a, (int, float, str)))}")
            return d

        return call
