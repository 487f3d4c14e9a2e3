"""The device context and device arrays addressed with Fortran bounds.

`Device` owns one libgbdyn context (one CUDA stream).  `DevArray` is the device counterpart of
pydyn's FView (pydyn dump.py:63-95): a float64 (or int32) array whose sections are taken with
the inclusive Fortran bounds it was declared with, `a[0:im, 1:jm, 1:lm]`, and are views --
pointer, extents and element strides -- that the kernels take as they are."""

import ctypes
from contextlib import contextmanager

import numpy as np

from . import _native as N


class Device:
    """One GPU context: memory, the stream every operator is enqueued on, graphs, events."""

    def __init__(self, device=0):
        L = N.lib()
        h = ctypes.c_void_p()
        N.check(L.gb_create(device, ctypes.byref(h)), "gb_create")
        self.h = h
        self.L = L
        self.ordinal = device
        self._owned = []
        self.capturing = False  # inside capture(): nothing may read the device back

    def close(self):
        if self.h:
            for p in self._owned:
                self.L.gb_free(self.h, p)
            self._owned.clear()
            self.L.gb_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -------------------------------------------------------------- memory
    def alloc(self, nbytes):
        p = ctypes.c_void_p()
        N.check(self.L.gb_alloc(self.h, nbytes, ctypes.byref(p)), "gb_alloc")
        self._owned.append(p.value)
        return p.value

    def put_bytes(self, dptr, host):
        host = np.ascontiguousarray(host)
        N.check(self.L.gb_put(self.h, dptr, host.ctypes.data, host.nbytes), "gb_put")
        self.sync_stream()  # the host buffer may be a temporary

    def get_bytes(self, dptr, nbytes, dtype):
        out = np.empty(nbytes // np.dtype(dtype).itemsize, dtype=dtype)
        N.check(self.L.gb_get(self.h, out.ctypes.data, dptr, nbytes), "gb_get")
        return out

    def sync_stream(self):
        N.check(self.L.gb_stream_sync(self.h), "gb_stream_sync")

    def sync(self):
        """Wait for the stream; raise what the device reported (CFLError, ValueError, ...)."""
        rc = self.L.gb_sync(self.h)
        N.check(rc, "device")

    def discard_status(self):
        """Wait for the stream and clear the device status word without raising (the errors of
        work that is being thrown away, a failed speculation's)."""
        self.L.gb_sync(self.h)

    def launches(self):
        return int(self.L.gb_launches(self.h))

    # -------------------------------------------------------------- graphs and events
    @contextmanager
    def capture(self):
        """Capture everything enqueued in the block into a Graph (yielded, filled on exit)."""
        g = Graph(self)
        N.check(self.L.gb_capture_begin(self.h), "gb_capture_begin")
        self.capturing = True
        try:
            yield g
        finally:
            self.capturing = False
            p = ctypes.c_void_p()
            N.check(self.L.gb_capture_end(self.h, ctypes.byref(p)), "gb_capture_end")
            g.p = p.value

    def event(self):
        return Event(self)

    def wait(self, event):
        """Work enqueued here from now on waits for `event` (recorded on any context's stream)."""
        N.check(self.L.gb_stream_wait(self.h, event.p), "gb_stream_wait")

    @contextmanager
    def redirect(self, other):
        """Inside the block, work enqueued through this device (its arrays' operators) goes to
        `other`'s context instead: its stream, work space and status word."""
        h = self.h
        self.h = other.h
        try:
            yield other
        finally:
            self.h = h

    # -------------------------------------------------------------- Check_CFL flag
    def cfl_reset(self):
        N.check(self.L.gb_cfl_reset(self.h), "gb_cfl_reset")

    def cfl_failed(self):
        f = ctypes.c_int()
        N.check(self.L.gb_cfl_failed(self.h, ctypes.byref(f)), "gb_cfl_failed")
        return bool(f.value)

    # -------------------------------------------------------------- work space
    def work_size(self):
        return int(self.L.gb_work_size(self.h))

    def set_priority(self, rank):
        """The context's streams at `rank` steps above the device's least priority (gb_stream_priority);
        outside a capture."""
        N.check(self.L.gb_stream_priority(self.h, int(rank)), "gb_stream_priority")

    def reserve_work(self, nbytes):
        """At least nbytes of work space (outside a capture)."""
        N.check(self.L.gb_work_reserve(self.h, int(nbytes)), "gb_work_reserve")

    # -------------------------------------------------------------- launch shapes
    def name(self):
        """The GPU's name, compute capability and SM count."""
        buf = ctypes.create_string_buffer(256)
        N.check(self.L.gb_device_name(self.h, buf, 256), "gb_device_name")
        return buf.value.decode()

    def tuning(self):
        """{name: value} of the context's launch shapes (gb_tune_get)."""
        out = {}
        for name, key in N.TUNE_KEYS.items():
            v = ctypes.c_int()
            N.check(self.L.gb_tune_get(self.h, key, ctypes.byref(v)), "gb_tune_get")
            out[name] = v.value
        return out

    def tune(self, **shapes):
        """Set launch shapes by name (gb_tune_set); results do not depend on them."""
        for name, value in shapes.items():
            N.check(self.L.gb_tune_set(self.h, N.TUNE_KEYS[name], int(value)), f"gb_tune_set({name}={value})")

    # -------------------------------------------------------------- FP64 ceiling
    def fp64_rates(self):
        """Measured FP64 issue rates of the device in G instructions/s: multiply + add pairs,
        fused multiply-adds, correctly rounded divisions; and the same pair with the add on the
        integer pipe (add_ip, counted as two instructions) and the integer-corrected division
        (div_ip, divisions/s)."""
        out = {}
        for kind, name in enumerate(("dmul_dadd", "dfma", "ddiv", "dmul_add_ip", "div_ip")):
            r = ctypes.c_double()
            N.check(self.L.gb_fp64_rate(self.h, kind, ctypes.byref(r)), "gb_fp64_rate")
            out[name] = r.value / 1e9
        return out


class Graph:
    def __init__(self, dev):
        self.dev, self.p = dev, None

    def launch(self):
        N.check(self.dev.L.gb_graph_launch(self.dev.h, self.p), "gb_graph_launch")

    def __del__(self):
        if self.p:
            try:
                self.dev.L.gb_graph_destroy(self.p)
            except Exception:
                pass


class Event:
    def __init__(self, dev):
        self.dev = dev
        p = ctypes.c_void_p()
        N.check(dev.L.gb_event_create(ctypes.byref(p)), "gb_event_create")
        self.p = p.value

    def record(self):
        N.check(self.dev.L.gb_event_record(self.dev.h, self.p), "gb_event_record")

    def synchronize(self):
        """Wait on the host until the work before the last record has completed."""
        N.check(self.dev.L.gb_event_sync(self.p), "gb_event_sync")

    def elapsed_ms(self, later):
        ms = ctypes.c_float()
        N.check(self.dev.L.gb_event_elapsed_ms(self.p, later.p, ctypes.byref(ms)), "gb_event_elapsed_ms")
        return float(ms.value)

    def __del__(self):
        try:
            self.dev.L.gb_event_destroy(self.p)
        except Exception:
            pass


class DevArray:
    """A device array with Fortran lower bounds; sections are views (writes go through)."""

    def __init__(self, dev, base, offset, shape, strides, lower, dtype):
        self.dev, self.base, self.offset = dev, base, offset
        self.shape, self.strides, self.lower = tuple(shape), tuple(strides), tuple(lower)
        self.dtype = np.dtype(dtype)

    # -------------------------------------------------------------- construction
    @classmethod
    def zeros(cls, dev, *bounds, dtype=np.float64):
        """`DevArray.zeros(dev, (-1, im + 2), (-1, jm + 2), (1, lm))`: (lower, upper) pairs."""
        shape = tuple(hi - lo + 1 for lo, hi in bounds)
        n = int(np.prod(shape)) if shape else 1
        base = dev.alloc(max(n, 1) * np.dtype(dtype).itemsize)
        strides = _c_strides(shape)
        return cls(dev, base, 0, shape, strides, [lo for lo, _ in bounds], dtype)

    @classmethod
    def from_host(cls, dev, arr, lower=None, dtype=None):
        arr = np.ascontiguousarray(arr, dtype=dtype if dtype is not None else arr.dtype)
        lower = (0,) * arr.ndim if lower is None else tuple(lower)
        out = cls.zeros(dev, *((lo, lo + n - 1) for lo, n in zip(lower, arr.shape, strict=True)), dtype=arr.dtype)
        dev.put_bytes(out.ptr, arr)
        return out

    # -------------------------------------------------------------- addressing
    @property
    def ptr(self):
        return self.base + self.offset * self.dtype.itemsize

    @property
    def ndim(self):
        return len(self.shape)

    @property
    def upper(self):
        return tuple(lo + n - 1 for lo, n in zip(self.lower, self.shape, strict=True))

    @property
    def size(self):
        return int(np.prod(self.shape)) if self.shape else 1

    def contiguous(self):
        return self.strides == _c_strides(self.shape)

    def __getitem__(self, item):
        """Inclusive Fortran section; an int index drops its axis; trailing axes whole."""
        if not isinstance(item, tuple):
            item = (item,)
        off, shape, strides, lower = self.offset, [], [], []
        for ax in range(self.ndim):
            lo, n, st = self.lower[ax], self.shape[ax], self.strides[ax]
            ix = item[ax] if ax < len(item) else slice(None)
            if isinstance(ix, slice):
                if ix.step not in (None, 1):
                    raise IndexError("DevArray: strided Fortran sections are not supported")
                a = lo if ix.start is None else ix.start
                b = lo + n - 1 if ix.stop is None else ix.stop
                if a < lo or b > lo + n - 1 or b < a - 1:
                    raise IndexError(f"DevArray: section {a}:{b} outside {lo}:{lo + n - 1}")
                off += (a - lo) * st
                shape.append(b - a + 1)
                strides.append(st)
                lower.append(a)
            else:
                if not lo <= ix <= lo + n - 1:
                    raise IndexError(f"DevArray: index {ix} outside {lo}:{lo + n - 1}")
                off += (ix - lo) * st
        return DevArray(self.dev, self.base, off, shape, strides, lower, self.dtype)

    def view(self):
        """The gb_view of this array (rank <= 4)."""
        if self.ndim > 4:
            raise ValueError("DevArray.view: rank > 4")
        v = N.GBView()
        v.p = self.ptr
        for k in range(4):
            v.n[k] = self.shape[k] if k < self.ndim else 1
            v.s[k] = self.strides[k] if k < self.ndim else 0
        return v

    def reshape_axes(self, shape, strides, lower=None):
        """A view with explicit extents and element strides over the same memory."""
        lower = (0,) * len(shape) if lower is None else lower
        return DevArray(self.dev, self.base, self.offset, shape, strides, lower, self.dtype)

    # -------------------------------------------------------------- host transfer (tests, setup)
    def host(self):
        """Download to a NumPy array (a copy)."""
        if self.contiguous():
            return self.dev.get_bytes(self.ptr, self.size * self.dtype.itemsize, self.dtype).reshape(self.shape)
        tmp = DevArray.zeros(self.dev, *((0, n - 1) for n in self.shape), dtype=self.dtype)
        tmp.assign(self)
        out = tmp.host()
        tmp.free()
        return out

    def upload(self, arr):
        arr = np.ascontiguousarray(np.broadcast_to(np.asarray(arr, dtype=self.dtype), self.shape))
        if self.contiguous():
            self.dev.put_bytes(self.ptr, arr)
            return
        tmp = DevArray.from_host(self.dev, arr)
        self.assign(tmp)
        tmp.free()

    def free(self):
        if self.offset == 0 and self.base in self.dev._owned:
            self.dev._owned.remove(self.base)
            self.dev.L.gb_free(self.dev.h, self.base)

    # -------------------------------------------------------------- box statements
    def _box(self, op, a=None, b=None, x=0.0, y=0.0):
        if self.dtype != np.float64:
            raise TypeError("box statements are float64")
        va = a.view() if a is not None else None
        vb = b.view() if b is not None else None
        vd = self.view()
        N.check(self.dev.L.gb_box(self.dev.h, op, ctypes.byref(vd), None if va is None else ctypes.byref(va),
                                  None if vb is None else ctypes.byref(vb), float(x), float(y)), "gb_box")  # fmt: skip

    def assign(self, src):
        """self[...] = src (same extents).  Two contiguous arrays of one layout are one device copy
        (stream-ordered, capturable); other sections go through the box kernel."""
        _same(self, src)
        nbytes = self.size * self.dtype.itemsize
        if self.contiguous() and src.contiguous() and self.dtype == src.dtype:
            if self.ptr == src.ptr:
                return
            if self.ptr + nbytes <= src.ptr or src.ptr + nbytes <= self.ptr:  # disjoint
                N.check(self.dev.L.gb_copy_d2d(self.dev.h, self.ptr, src.ptr, nbytes), "gb_copy_d2d")
                return
        self._box(0, src)

    def fill(self, x):
        self._box(3, x=x)

    def scaled(self, src, x):
        """self[...] = src * x."""
        _same(self, src)
        self._box(1, src, x=x)

    def divided(self, src, x):
        """self[...] = src / x."""
        _same(self, src)
        self._box(2, src, x=x)

    def binary(self, op, a, b):
        """self[...] = a (+ - * /) b, op one of '+-*/'."""
        _same(self, a)
        _same(self, b)
        self._box({"+": 4, "-": 5, "*": 6, "/": 7}[op], a, b)

    def progressive(self, src, n):
        """self[...] = src * (n - 1) / n (ops.progressive)."""
        _same(self, src)
        self._box(8, src, x=float(n - 1), y=float(n))

    def interpolate(self, a, b, alfa1, alfa2):
        """self[...] = alfa1 a + alfa2 b (balance.time_interpolation)."""
        _same(self, a)
        _same(self, b)
        self._box(9, a, b, x=alfa1, y=alfa2)

    def seqsum_of(self, src, axis, post_mul=1.0):
        """self = seqsum of src over `axis`; self has src's extents with that axis of length 1."""
        vd, vs = self.view(), src.view()
        N.check(self.dev.L.gb_seqsum(self.dev.h, ctypes.byref(vd), ctypes.byref(vs), axis, float(post_mul)),
                "gb_seqsum")

    def expand_axis(self, axis):
        """A view with a length-1 axis inserted at `axis` (stride 0)."""
        shape = list(self.shape)
        strides = list(self.strides)
        lower = list(self.lower)
        shape.insert(axis, 1)
        strides.insert(axis, 0)
        lower.insert(axis, 0)
        return DevArray(self.dev, self.base, self.offset, shape, strides, lower, self.dtype)

    def __repr__(self):
        b = ", ".join(f"{lo}:{lo + n - 1}" for lo, n in zip(self.lower, self.shape, strict=True))
        return f"DevArray({b})"


def _c_strides(shape):
    st, acc = [], 1
    for n in reversed(shape):
        st.append(acc)
        acc *= n
    return tuple(reversed(st))


def _same(a, b):
    if tuple(a.shape) != tuple(b.shape):
        raise ValueError(f"extents differ: {a.shape} vs {b.shape}")


def views(*arrays):
    """ctypes byref gb_views of DevArrays (None stays None)."""
    out = []
    for a in arrays:
        out.append(None if a is None else ctypes.byref(a.view()))
    return out
