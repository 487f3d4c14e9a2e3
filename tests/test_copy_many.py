"""gb_copy_many, the captured interval's batched device-to-device copies, on its own: copies of
very different sizes in one launch land bitwise with the bytes after each destination
untouched; no copy, or no bytes, launch nothing; malformed arguments are refused.  And its
table builder's checks on the host."""

import numpy as np
import pytest


class _Fake:
    """An array as the table builder sees it: a pointer, an element count and a dtype."""

    def __init__(self, ptr, size, dtype):
        self.ptr, self.size, self.dtype = ptr, size, np.dtype(dtype)


@pytest.mark.parametrize(("src", "dst"), [((1, "f4"), (4, "f4")), ((0, "f8"), (1, "f8")), ((4, "f8"), (3, "f8"))])
def test_copy_table_refuses_what_the_kernel_cannot_copy(src, dst):
    """Byte counts not a multiple of 8, empty copies and short destinations: ValueError."""
    from pydyn_gb300.forward import copy_table

    with pytest.raises(ValueError, match="copy_table"):
        copy_table(None, [(_Fake(64, *dst), _Fake(128, *src))])


@pytest.mark.gpu
def test_copy_many_copies_each_row_and_nothing_past_it(dev):
    from pydyn_gb300 import _native as N
    from pydyn_gb300.device import DevArray
    from pydyn_gb300.forward import copy_table

    rng = np.random.default_rng(12)
    sizes = (1, 517, 131072 + 3)  # elements: far shorter than the longest, odd counts, many grid rows
    srcs = [DevArray.from_host(dev, rng.standard_normal(k)) for k in sizes]
    pad = 64
    sentinel = -7.25
    dsts = [DevArray.from_host(dev, np.full(k + pad, sentinel)) for k in sizes]
    views = [d[0 : k - 1] for d, k in zip(dsts, sizes, strict=True)]
    table, n, most = copy_table(dev, list(zip(views, srcs, strict=True)))
    assert (n, most) == (3, 8 * sizes[-1])
    before = dev.launches()
    N.check(N.lib().gb_copy_many(dev.h, table.ptr, n, most), "gb_copy_many")
    dev.sync()
    assert dev.launches() - before == 1
    for s, d, k in zip(srcs, dsts, sizes, strict=True):
        got = d.host()
        np.testing.assert_array_equal(got[:k].view(np.int64), s.host().view(np.int64))
        assert (got[k:] == sentinel).all(), "bytes past a destination changed"
    # nothing to copy: no launch
    for args in ((table.ptr, 0, most), (table.ptr, n, 0)):
        before = dev.launches()
        assert N.lib().gb_copy_many(dev.h, *args) == N.GB_OK
        assert dev.launches() == before
    # malformed: a byte bound not a multiple of 8, a negative or too large count, no table
    for args in ((table.ptr, n, most - 4), (table.ptr, -1, most), (table.ptr, 65536, most), (None, n, most)):
        assert N.lib().gb_copy_many(dev.h, *args) == N.GB_EARG
    for a in (*srcs, *dsts, table):
        a.free()
