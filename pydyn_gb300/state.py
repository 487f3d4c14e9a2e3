"""Every region's state on the device, its arrays with the Fortran bounds TM5 declares them
with, as pydyn's ZoomState holds them on the host (pydyn zoom/state.py:13-50, layout.py:26-36):

    m (-1:im+2, -1:jm+2, 1:lm)        rm rxm rym rzm (-1:im+2, -1:jm+2, 1:lm, 1:nt)
    am bm cm (0:im+1, 0:jm+1, 0:lm+1) pu (0:im, 1:jm, 1:lm)   pv (1:im, 1:jm+1, 1:lm)
    sp (-1:im+2, -1:jm+2, 1:1)        phlb (-1:im+2, -1:jm+2, 1:lm+1)   dxyp (1:jm)

C-order on the device, so the level (and tracer) index is the fastest: a (j, l) row of x and an
(i, l) column of y are read by consecutive threads at consecutive addresses, and a z column is
contiguous.  `lib` is the module of bodies the driver calls: pydyn_gb300.zoom."""

import numpy as np

from .device import DevArray
from .layout import FIELDS, TRACERS, bounds  # noqa: F401  (re-exported)


class ZoomState:
    """Every region's device arrays: `st[r][name]` is a DevArray with its Fortran bounds."""

    def __init__(self, dev, zoom, fields, nt, lib=None):
        if lib is None:
            from . import zoom as lib
        self.dev, self.zoom, self.fields, self.lib = dev, zoom, fields, lib
        self._nt = nt
        self.saved = {}
        self.consts = {}  # per-region device constants (cluster sizes, at, bt, ...)

    @classmethod
    def zeros(cls, dev, zoom, nt):
        lm = zoom.lm
        fields = {}
        for r in zoom.regions():
            g = zoom.g(r)
            fields[r] = {name: DevArray.zeros(dev, *bounds(name, g.im, g.jm, lm, nt)) for name in FIELDS}
        return cls(dev, zoom, fields, nt)

    @classmethod
    def from_host(cls, dev, zoom, host_fields):
        """A device copy of host arrays: host_fields[r][name] are NumPy arrays in the declared
        shapes (FView .data arrays of a pydyn ZoomState, for instance)."""
        nt = host_fields[1]["rm"].shape[3]
        st = cls.zeros(dev, zoom, nt)
        st.upload(host_fields)
        return st

    def upload(self, host_fields):
        for r, f in host_fields.items():
            for name, arr in f.items():
                if name in self.fields[r]:
                    self.fields[r][name].upload(np.asarray(arr, dtype=np.float64))

    def host(self):
        """{r: {name: NumPy array}} of the whole state (a download)."""
        return {r: {name: a.host() for name, a in f.items()} for r, f in self.fields.items()}

    def __getitem__(self, r):
        return self.fields[r]

    @property
    def nt(self):
        return self._nt

    def copy(self):
        out = ZoomState.zeros(self.dev, self.zoom, self.nt)
        out.lib = self.lib
        for r, f in self.fields.items():
            for name, a in f.items():
                out.fields[r][name].assign(a)
        return out

    def const(self, r, key, make):
        """A per-region device constant, made once by make() -> NumPy array."""
        k = (r, key)
        if k not in self.consts:
            self.consts[k] = DevArray.from_host(self.dev, np.ascontiguousarray(make()))
        return self.consts[k]

    def free(self):
        for f in self.fields.values():
            for a in f.values():
                a.free()
        for a in self.consts.values():
            for x in a if isinstance(a, tuple) else (a,):
                if isinstance(x, DevArray):
                    x.free()
        for d in self.saved.values():
            for a in d.values():
                a.free()
