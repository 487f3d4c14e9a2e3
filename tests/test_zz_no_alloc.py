"""gb_advect_y_noalloc, the y advection whose per-layer scratch is a fixed array in the library,
against gb_advect_y on the same inputs: two calls in a row (the second over different fluxes,
so its counts overwrite the first's), every array bitwise, the per-layer counts equal.  This
file is collected after every other, so that the entry point also runs after them."""

import ctypes

import numpy as np
import pytest
from conftest import assert_bitwise

TRACERS = ("rm", "rxm", "rym", "rzm")
MAX_LEVELS = 1024  # GB_NOALLOC_MAX_LEVELS


def _inputs(rng, im, jm, lm, nt, cfl):
    """Masses ~1e9, tracers with slopes, and closed columns of meridional flux (polar faces 0)
    moving each column towards a seeded target: Courant numbers up to about cfl."""
    m = 1e9 * rng.uniform(0.8, 1.2, (im, jm, lm))
    rm = m[..., None] * rng.uniform(0.5, 1.5, (im, jm, lm, nt)) * 1e-6
    f = {"m": m, "rm": rm}
    for k in TRACERS[1:]:
        f[k] = 0.3 * rm * rng.uniform(-1, 1, rm.shape)
    target = m * (1.0 + min(0.6 * cfl, 0.9) * rng.uniform(-1, 1, m.shape))
    target *= m.sum(axis=1, keepdims=True) / target.sum(axis=1, keepdims=True)
    bm = np.concatenate([np.zeros((im, 1, lm)), np.cumsum(m - target, axis=1)], axis=1)
    bm[:, jm] = 0.0
    f["bm"] = bm
    return f


def _run(dev, name, host, nloop):
    """One call of the entry point `name` on device copies of `host`; returns their host copies."""
    from pydyn_gb300 import _native as N
    from pydyn_gb300.device import DevArray, views

    d = {k: DevArray.from_host(dev, v) for k, v in host.items()}
    L = N.lib()
    rc = getattr(L, name)(dev.h, *views(d["m"], *(d[q] for q in TRACERS), d["bm"], None), 0, 1, 10, nloop.ptr)
    N.check(rc, name)
    dev.sync()
    out = {k: v.host() for k, v in d.items()}
    for v in d.values():
        v.free()
    return out


@pytest.mark.gpu
def test_noalloc_y_equals_advect_y_on_two_calls_in_a_row(dev):
    from pydyn_gb300.device import DevArray

    rng = np.random.default_rng(2024)
    im, jm, lm, nt = 40, 30, 12, 2
    first, second = _inputs(rng, im, jm, lm, nt, 0.9), _inputs(rng, im, jm, lm, nt, 0.3)
    counts = {}
    for name in ("gb_advect_y", "gb_advect_y_noalloc"):
        n1 = DevArray.zeros(dev, (0, lm - 1), dtype=np.int32)
        n2 = DevArray.zeros(dev, (0, lm - 1), dtype=np.int32)
        counts[name] = (_run(dev, name, first, n1), _run(dev, name, second, n2), n1.host(), n2.host())
        n1.free()
        n2.free()
    want, got = counts["gb_advect_y"], counts["gb_advect_y_noalloc"]
    for call in (0, 1):
        for k in ("m", *TRACERS, "bm"):
            assert_bitwise(got[call][k], want[call][k], f"call {call + 1}: {k}")
    np.testing.assert_array_equal(got[2], want[2])
    np.testing.assert_array_equal(got[3], want[3])
    assert want[2].max() > 1 and not np.array_equal(want[2], want[3])  # the two calls' counts differ


@pytest.mark.gpu
def test_noalloc_y_rejects_more_levels_than_its_array(dev):
    """A call over more levels than the fixed array holds returns GB_EARG before any launch."""
    from pydyn_gb300 import _native as N
    from pydyn_gb300.device import DevArray, views

    im, jm, lm = 2, 3, MAX_LEVELS + 1
    a = {"m": DevArray.zeros(dev, (0, im - 1), (0, jm - 1), (0, lm - 1)),
         "bm": DevArray.zeros(dev, (0, im - 1), (0, jm), (0, lm - 1))}  # fmt: skip
    for q in TRACERS:
        a[q] = DevArray.zeros(dev, (0, im - 1), (0, jm - 1), (0, lm - 1), (0, 0))
    before = dev.launches()
    rc = N.lib().gb_advect_y_noalloc(dev.h, *views(a["m"], *(a[q] for q in TRACERS), a["bm"], None), 0, 1, 10,
                                     ctypes.c_void_p())  # fmt: skip
    assert rc == N.GB_EARG
    assert "1025 levels" in N.last_error()
    assert dev.launches() == before
    for v in a.values():
        v.free()


def _scratch(dev):
    """The context's int32 scratch as (device pointer, length)."""
    from pydyn_gb300 import _native as N

    p, n = ctypes.c_void_p(), ctypes.c_size_t()
    N.check(N.lib().gb_scratch_info(dev.h, ctypes.byref(p), ctypes.byref(n)), "gb_scratch_info")
    return p.value, n.value


@pytest.mark.gpu
def test_noalloc_y_leaves_the_context_scratch_and_device_memory_alone(dev):
    """The entry point exists for callers that cannot allocate: its calls take no device memory
    (the free memory is the same before and after calls past the first) and keep their counts
    out of the context's scratch (a pattern written there is intact after them)."""
    torch = pytest.importorskip("torch")
    from pydyn_gb300 import _native as N
    from pydyn_gb300.device import DevArray

    rng = np.random.default_rng(7)
    im, jm, lm, nt = 24, 20, 10, 1
    host = _inputs(rng, im, jm, lm, nt, 0.8)
    n1 = DevArray.zeros(dev, (0, lm - 1), dtype=np.int32)
    _run(dev, "gb_advect_y_noalloc", host, n1)  # the first call looks the fixed array's address up
    ptr, n = _scratch(dev)
    pattern = (np.arange(n, dtype=np.int64) * 2654435761 % 2**31).astype(np.int32)
    N.check(N.lib().gb_put(dev.h, ptr, pattern.ctypes.data, pattern.nbytes), "gb_put")
    dev.sync()
    free0, _ = torch.cuda.mem_get_info(0)
    for _ in range(3):
        _run(dev, "gb_advect_y_noalloc", host, n1)
    free1, _ = torch.cuda.mem_get_info(0)
    back = np.empty_like(pattern)
    N.check(N.lib().gb_get(dev.h, back.ctypes.data, ptr, back.nbytes), "gb_get")
    dev.sync()
    np.testing.assert_array_equal(back, pattern)
    # _run's own device copies of the inputs come and go through the caching of the test's
    # DevArrays; the entry point itself must not leave the free memory lower
    assert free1 >= free0
    n1.free()
