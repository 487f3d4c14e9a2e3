"""Pinned host buffers for the end-to-end path: a run's per-step inputs go to the device and its
results come back with asynchronous copies on the context's stream."""

import ctypes

import numpy as np

from . import _native as N
from .device import DevArray


class PinnedArray:
    """A float64 NumPy array in page-locked host memory."""

    def __init__(self, shape):
        self.shape = tuple(shape)
        self.nbytes = int(np.prod(self.shape)) * 8
        p = ctypes.c_void_p()
        N.check(N.lib().gb_host_alloc(self.nbytes, ctypes.byref(p)), "gb_host_alloc")
        self.p = p.value
        buf = (ctypes.c_double * int(np.prod(self.shape))).from_address(self.p)
        self.array = np.frombuffer(buf, dtype=np.float64).reshape(self.shape)
        self._staging = None

    @classmethod
    def empty(cls, shape):
        return cls(shape)

    @classmethod
    def copy_of(cls, a):
        out = cls(np.shape(a))
        out.array[...] = a
        return out

    def to_device(self, dev, dst):
        """dst (a contiguous DevArray of the same size) <- this buffer, asynchronously."""
        if not dst.contiguous() or dst.size * 8 != self.nbytes:
            raise ValueError("PinnedArray.to_device: a contiguous destination of the same size")
        N.check(dev.L.gb_put(dev.h, dst.ptr, self.p, self.nbytes), "gb_put")

    def from_device(self, dev, src):
        """This buffer <- src (a DevArray view of the same extents), asynchronously; strided
        views are first gathered on the device into a contiguous staging array."""
        if src.size * 8 != self.nbytes:
            raise ValueError("PinnedArray.from_device: extents differ")
        if not src.contiguous():
            if self._staging is None:
                self._staging = DevArray.zeros(dev, *((0, n - 1) for n in src.shape))
            self._staging.assign(src)
            src = self._staging
        N.check(dev.L.gb_get_async(dev.h, self.p, src.ptr, self.nbytes), "gb_get_async")

    def __del__(self):
        try:
            N.lib().gb_host_free(self.p)
        except Exception:
            pass
