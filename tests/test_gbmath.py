"""The package's host math library (libgbmath.so, the host build of csrc/gbmath.h) against the C
library: within 1 ulp on the arguments the dynamic step's Kzz and chemistry pass (and wider
ranges), C99 special values; the device build equals the host build bit for bit (GPU test)."""

import math

import numpy as np
import pytest

from conftest import bits


def ulps(a, b):
    def ordered(x):
        i = np.asarray(x, dtype="<f8").view(np.int64)
        return np.where(i < 0, np.iinfo(np.int64).min - i, i)

    return np.abs(ordered(a) - ordered(b))


def _cases(rng):
    return {
        "exp": [(x,) for x in np.concatenate([rng.uniform(-700, 700, 4000), rng.uniform(-2, 2, 4000),
                                             rng.uniform(-1e-8, 1e-8, 500)])],
        "log": [(x,) for x in np.concatenate([np.exp(rng.uniform(-700, 700, 4000)), rng.uniform(0.5, 2.0, 4000),
                                             1.0 + rng.uniform(-1e-7, 1e-7, 500), [5e-320, 1e-310]])],
        "pow": [(x, y) for x, y in zip(rng.uniform(0.1, 10, 4000), rng.uniform(-5, 5, 4000), strict=True)]
        + [(x, 1.0 / 3.0) for x in rng.uniform(1e-6, 1e3, 2000)]
        + [(x, 1.37) for x in rng.uniform(0.6, 1.1, 2000)]
        + [(x, 0.2857) for x in rng.uniform(0.01, 100.0, 2000)]
        + [(x, y) for x, y in zip(rng.uniform(0.99, 1.01, 1000), rng.uniform(-3e3, 3e3, 1000), strict=True)],
        "cos": [(x,) for x in np.concatenate([rng.uniform(-1.6, 1.6, 4000), rng.uniform(-100, 100, 2000)])],
        "sin": [(x,) for x in np.concatenate([rng.uniform(-1.6, 1.6, 4000), rng.uniform(-100, 100, 2000)])],
    }


@pytest.mark.parametrize("name", ["exp", "log", "pow", "cos", "sin"])
def test_within_one_ulp_of_the_c_library(built, name):
    from pydyn_gb300 import _native as N

    f = getattr(N.mathlib(), name)
    rng = np.random.default_rng(7)
    args = _cases(rng)[name]
    ours = np.array([f(*a) for a in args])
    theirs = np.array([getattr(math, name)(*a) for a in args])
    d = ulps(ours, theirs)
    assert d.max() <= 1, f"{name}: {d.max()} ulp at {args[int(d.argmax())]}"


def test_special_values(built):
    from pydyn_gb300 import _native as N

    L = N.mathlib()
    inf, nan = math.inf, math.nan
    assert L.exp(0.0) == 1.0 and L.exp(-inf) == 0.0 and L.exp(inf) == inf and L.exp(800.0) == inf
    assert L.exp(-800.0) == 0.0 and math.isnan(L.exp(nan))
    assert L.log(1.0) == 0.0 and L.log(0.0) == -inf and math.isnan(L.log(-1.0)) and L.log(inf) == inf
    assert L.pow(1.0, nan) == 1.0 and L.pow(2.0, 0.0) == 1.0 and L.pow(-8.0, 1.0 / 3.0) != L.pow(-8.0, 1.0 / 3.0)
    assert L.pow(-2.0, 3.0) == -8.0 and L.pow(0.0, -1.0) == inf and L.pow(4.0, 0.5) == 2.0
    assert L.pow(2.0, -1075.0) == 0.0 and L.pow(2.0, 1024.0) == inf and L.pow(2.0, -1074.0) == 5e-324
    assert L.cos(0.0) == 1.0 and L.sin(0.0) == 0.0 and bits(L.sin(-0.0)) == bits(-0.0)


@pytest.mark.gpu
def test_device_math_equals_host_math(dev):
    from pydyn_gb300 import _native as N
    from pydyn_gb300.device import DevArray

    L = N.mathlib()
    rng = np.random.default_rng(11)
    for op, name in enumerate(("exp", "log", "pow", "cos", "sin")):
        args = _cases(rng)[name]
        x = np.array([a[0] for a in args])
        y = np.array([a[1] if len(a) > 1 else 0.0 for a in args])
        dx, dy = DevArray.from_host(dev, x), DevArray.from_host(dev, y)
        out = DevArray.zeros(dev, (0, len(x) - 1))
        N.check(dev.L.gb_math_eval(dev.h, op, dx.ptr, dy.ptr, out.ptr, len(x)), "gb_math_eval")
        got = out.host()
        want = np.array([getattr(L, name)(*a) for a in args])
        assert (bits(got) == bits(want)).all(), name
        for a in (dx, dy, out):
            a.free()


def _division_cases(rng):
    """(a, d) pairs: random magnitudes over the whole range, quotients a hair off a rounding
    midpoint, significands of all ones, and every kind of special value."""
    n = 200_000
    sig = lambda k: 1.0 + rng.integers(0, 2**52, k) / 2.0**52  # noqa: E731
    a = sig(n) * np.exp2(rng.integers(-1074, 1023, n).astype(float)) * rng.choice([-1.0, 1.0], n)
    d = sig(n) * np.exp2(rng.integers(-1074, 1023, n).astype(float)) * rng.choice([-1.0, 1.0], n)
    a2 = sig(n) * np.exp2(rng.integers(-40, 40, n).astype(float))
    d2 = sig(n) * np.exp2(rng.integers(-40, 40, n).astype(float))
    q = sig(n)
    d3 = sig(n)
    a3 = d3 * (q + 2.0**-53)  # the product rounded: a quotient next to a midpoint
    special = np.array([0.0, -0.0, 5e-324, -5e-324, 2.2250738585072014e-308, 1.7976931348623157e308, np.inf,
                        -np.inf, np.nan, 1.0, -1.0, 2.0 - 2.0**-52, 1.0 + 2.0**-52, 3.0, 0.1, 2.0**-1000,
                        2.0**1000, 2.0**-960, 2.0**1001, 2.0**-1001])  # fmt: skip
    sa, sd = np.meshgrid(special, special)
    return np.concatenate([a, a2, a3, sa.ravel()]), np.concatenate([d, d2, d3, sd.ravel()])


@pytest.mark.gpu
def test_shared_reciprocal_division_is_the_division(dev):
    """div_by_recip equals the hardware division bit for bit (NaNs included), and both equal the
    host's IEEE division wherever the quotient is not a NaN."""
    from pydyn_gb300 import _native as N
    from pydyn_gb300.device import DevArray

    a, d = _division_cases(np.random.default_rng(5))
    da, dd = DevArray.from_host(dev, a), DevArray.from_host(dev, d)
    outs = []
    for op in (5, 6):
        out = DevArray.zeros(dev, (0, len(a) - 1))
        N.check(dev.L.gb_math_eval(dev.h, op, da.ptr, dd.ptr, out.ptr, len(a)), "gb_math_eval")
        outs.append(out.host())
        out.free()
    fast, hw = outs
    assert (bits(fast) == bits(hw)).all()
    with np.errstate(all="ignore"):
        want = a / d
    ok = ~np.isnan(want)
    assert (bits(fast[ok]) == bits(want[ok])).all() and np.isnan(fast[~ok]).all()
    for x in (da, dd):
        x.free()


def _eval(dev, op, a, b):
    from pydyn_gb300 import _native as N
    from pydyn_gb300.device import DevArray

    da, db = DevArray.from_host(dev, a), DevArray.from_host(dev, b)
    out = DevArray.zeros(dev, (0, len(a) - 1))
    N.check(dev.L.gb_math_eval(dev.h, op, da.ptr, db.ptr, out.ptr, len(a)), "gb_math_eval")
    got = out.host()
    for x in (da, db, out):
        x.free()
    return got


@pytest.mark.gpu
def test_integer_corrected_division_is_the_division(dev):
    """div_ip (an FP32 reciprocal seed, one FMA correction, the exact integer residual) equals the
    hardware division bit for bit, NaNs included, over the whole range and at the edges of its
    fast path: divisors at the ends of [2^-125, 2^125], significands at a binade's edges, exact
    quotients."""
    rng = np.random.default_rng(7)
    a, d = _division_cases(rng)
    n = 100_000
    sig = lambda k: 1.0 + rng.integers(0, 2**52, k) / 2.0**52  # noqa: E731
    edge = np.concatenate([1.0 + np.arange(0, 4096) / 2.0**52, 2.0 - np.arange(1, 4097) / 2.0**52])
    d_edge = np.resize(edge, n) * np.exp2(rng.integers(-130, 130, n).astype(float))
    a_edge = sig(n) * np.exp2(rng.integers(-60, 60, n).astype(float)) * rng.choice([-1.0, 1.0], n)
    d_exact = sig(n)
    a_exact = d_exact * rng.integers(1, 2**20, n).astype(float)
    a = np.concatenate([a, a_edge, a_exact])
    d = np.concatenate([d, d_edge, d_exact])
    got, hw = _eval(dev, 7, a, d), _eval(dev, 6, a, d)
    assert (bits(got) == bits(hw)).all()
    with np.errstate(all="ignore"):
        want = a / d
    ok = ~np.isnan(want)
    assert (bits(got[ok]) == bits(want[ok])).all() and np.isnan(got[~ok]).all()


def _sum_cases(rng):
    """(a, b) pairs for a + b: like signs at every exponent gap from 0 to 70, zeros of both signs
    beside normal and subnormal numbers, subnormals, all-ones significands (carries), short
    significands (ties), opposite signs, and every kind of special value."""
    n = 100_000
    sig = lambda k: 1.0 + rng.integers(0, 2**52, k) / 2.0**52  # noqa: E731
    e = rng.integers(-900, 900, n).astype(float)
    s = rng.choice([-1.0, 1.0], n)
    a1 = sig(n) * np.exp2(e) * s
    b1 = sig(n) * np.exp2(e - rng.integers(0, 71, n)) * s
    a2 = sig(n) * np.exp2(rng.integers(-1074, 1023, n).astype(float)) * rng.choice([-1.0, 1.0], n)
    b2 = rng.choice([0.0, -0.0], n)
    a3 = rng.integers(1, 2**52, n) * 5e-324 * rng.choice([-1.0, 1.0], n)
    b3 = sig(n) * np.exp2(rng.integers(-1022, -1000, n).astype(float)) * np.sign(a3)
    ones = 2.0 - 2.0**-52
    a4 = ones * np.exp2(e) * s
    b4 = (2.0 - rng.integers(1, 8, n) * 2.0**-52) * np.exp2(e - rng.integers(0, 8, n)) * s
    short = lambda k: np.round(sig(k) * 2.0**rng.integers(0, 30, k)) / 2.0**rng.integers(0, 30, k)  # noqa: E731
    a5 = short(n) * np.exp2(e) * s
    b5 = short(n) * np.exp2(e - rng.integers(0, 60, n)) * s
    a6 = sig(n) * np.exp2(e) * s
    b6 = -sig(n) * np.exp2(e - rng.integers(0, 60, n)) * s
    special = np.array([0.0, -0.0, 5e-324, -5e-324, 2.2250738585072014e-308, 1.7976931348623157e308,
                        8.98846567431158e307, np.inf, -np.inf, np.nan, 1.0, -1.0, 2.0 - 2.0**-52])
    sa, sb = np.meshgrid(special, special)
    a = np.concatenate([a1, a2, a3, a4, a5, a6, sa.ravel()])
    b = np.concatenate([b1, b2, b3, b4, b5, b6, sb.ravel()])
    return np.concatenate([a, b]), np.concatenate([b, a])


@pytest.mark.gpu
def test_integer_pipe_sum_is_the_sum(dev):
    """add_ip / sub_ip equal IEEE a + b / a - b bit for bit (the host's, round to nearest even),
    a NaN where it is a NaN: the integer path (like signs, zeros) and the FP64 fallback alike."""
    a, b = _sum_cases(np.random.default_rng(13))
    with np.errstate(all="ignore"):
        want_add, want_sub = a + b, a - b
    for op, want in ((8, want_add), (9, want_sub)):
        got = _eval(dev, op, a, b)
        ok = ~np.isnan(want)
        assert (bits(got[ok]) == bits(want[ok])).all() and np.isnan(got[~ok]).all(), op


@pytest.mark.gpu
def test_integer_corrected_root_is_the_root(dev):
    """sqrt_ip (a correctly rounded FP32 seed, one Newton step, the exact integer residual) equals
    the hardware square root and IEEE sqrt bit for bit: over the whole range, exact squares and
    their neighbours, significands at a binade's edges, zeros, negatives, subnormals, specials."""
    rng = np.random.default_rng(17)
    n = 200_000
    sig = lambda k: 1.0 + rng.integers(0, 2**52, k) / 2.0**52  # noqa: E731
    x1 = sig(n) * np.exp2(rng.integers(-1022, 1024, n).astype(float))
    s = sig(n) * np.exp2(rng.integers(-200, 200, n).astype(float))
    sq = s * s
    x2 = np.concatenate([sq, np.nextafter(sq, 0.0), np.nextafter(sq, np.inf)])
    x3 = (rng.integers(1, 2**26, n).astype(float)) ** 2
    edge = np.concatenate([1.0 + np.arange(0, 4096) / 2.0**52, 2.0 - np.arange(1, 4097) / 2.0**52])
    x4 = np.resize(edge, n) * np.exp2(rng.integers(-300, 300, n).astype(float))
    special = np.array([0.0, -0.0, 5e-324, 2.2250738585072014e-308, 1.7976931348623157e308, np.inf, -np.inf,
                        np.nan, -1.0, 1.0, 4.0, 2.0, 0.25, -5e-324])
    x = np.concatenate([x1, x2, x3, x4, special])
    got, hw = _eval(dev, 10, x, x), _eval(dev, 11, x, x)
    assert (bits(got) == bits(hw)).all()
    with np.errstate(all="ignore"):
        want = np.sqrt(x)
    ok = ~np.isnan(want)
    assert (bits(got[ok]) == bits(want[ok])).all() and np.isnan(got[~ok]).all()


@pytest.mark.gpu
def test_fp64_rates(dev):
    """The rate probe's five kinds run and report positive rates."""
    r = dev.fp64_rates()
    assert set(r) == {"dmul_dadd", "dfma", "ddiv", "dmul_add_ip", "div_ip"}
    assert all(v > 0.0 for v in r.values())


@pytest.mark.gpu
def test_flag_arithmetic_is_the_statements(dev):
    """Calc_Kzz's flag arithmetic on the integer pipe equals the FP64 statements bit for bit (NaNs
    as NaNs), signed zeros, infinities and NaNs included: jq x + (1 - jq) y at jq = 1.0 and +0.0
    (blend01), +0.0 x (mul01), and jqif(x, y) = nint(0.5 + sign(0.5, x - y)) (jqif_ip)."""
    rng = np.random.default_rng(23)
    special = np.array([0.0, -0.0, 5e-324, -5e-324, 1.0, -1.0, 0.3, -0.3, 1.7976931348623157e308,
                        -1.7976931348623157e308, np.inf, -np.inf, np.nan, 2.2250738585072014e-308])
    sa, sb = np.meshgrid(special, special)
    n = 100_000
    a = np.concatenate([sa.ravel(), rng.standard_normal(n) * np.exp2(rng.integers(-60, 60, n).astype(float)),
                        rng.choice(special, n)])
    b = np.concatenate([sb.ravel(), rng.standard_normal(n) * np.exp2(rng.integers(-60, 60, n).astype(float)),
                        rng.choice(special, n)])
    with np.errstate(all="ignore"):
        want = {12: 1.0 * a + (1.0 - 1.0) * b, 13: 0.0 * a + (1.0 - 0.0) * b, 14: 0.0 * a,
                15: np.where(np.signbit(a - b), 0.0, 1.0)}
    for op, w in want.items():
        got = _eval(dev, op, a, b)
        ok = ~np.isnan(w)
        if op == 15:  # the sign of a NaN difference is the hardware's; compare the finite operands
            ok = np.isfinite(a) & np.isfinite(b)
        assert (bits(got[ok]) == bits(w[ok])).all() and np.isnan(got[~ok & np.isnan(w)]).all(), op
