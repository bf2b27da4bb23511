"""Bit-exactness of the integer-pipe binary64 operations (csrc/fm_softfp.cuh)
against the host's IEEE arithmetic, on the CPU: the header is compiled as
plain C++ (the same source the kernels inline) into a temporary library.

Inputs: random significands over wide exponent ranges, the special values
(signed zeros, subnormals, infinities, NaN), operands whose quotient lies
right at a binade boundary (x = d * 2^k and neighbours), and products that are
exact ties (one factor with a short significand), which exercise the
round-half-even branch.
"""
import ctypes
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "native" / "softfp_check.cpp"


def _build(tmp_path_factory, name, defines=()):
    out = tmp_path_factory.mktemp("softfp") / name
    subprocess.run(["g++", "-O2", "-ffp-contract=off", "-shared", "-fPIC", *defines, "-o",
                    str(out), str(SRC)], check=True)
    L = ctypes.CDLL(str(out))
    dp = ctypes.POINTER(ctypes.c_double)
    L.softfp_div_const.argtypes = [dp, ctypes.c_long, ctypes.c_double, dp]
    L.softfp_mul_const.argtypes = [dp, ctypes.c_long, ctypes.c_double, dp]
    L.softfp_mul.argtypes = [dp, dp, ctypes.c_long, dp]
    L.softfp_scale_pow2.argtypes = [dp, ctypes.c_long, ctypes.c_int, dp]
    L.softfp_div.argtypes = [dp, dp, ctypes.c_long, dp]
    L.softfp_max.argtypes = [dp, dp, ctypes.c_long, dp]
    L.softfp_min.argtypes = [dp, dp, ctypes.c_long, dp]
    L.softfp_le_zero.argtypes = [dp, ctypes.c_long, ctypes.POINTER(ctypes.c_ubyte)]
    L.softfp_cmp.argtypes = [dp, dp, ctypes.c_long, ctypes.POINTER(ctypes.c_ubyte)]
    fp = ctypes.POINTER(ctypes.c_float)
    L.softfp_f2d.argtypes = [fp, ctypes.c_long, dp]
    L.softfp_d2f.argtypes = [dp, ctypes.c_long, fp]
    up = ctypes.POINTER(ctypes.c_ulonglong)
    L.softfp_recip115.argtypes = [up, ctypes.c_long, up]
    L.softfp_div_reciprocal_words.argtypes = [ctypes.c_double, ctypes.POINTER(ctypes.c_uint),
                                              ctypes.POINTER(ctypes.c_uint)]
    return L


@pytest.fixture(scope="module", params=["full", "fast_only"])
def lib(tmp_path_factory, request):
    """The full operations, and the fast path alone: with FM_SOFT_SLOW_SENTINEL
    the slow path returns a marked NaN, so the fast path is checked on every
    input it accepts (and must accept every normal-range case)."""
    if request.param == "full":
        return _build(tmp_path_factory, "libsoftfp_full.so")
    return _build(tmp_path_factory, "libsoftfp_fast.so", ["-DFM_SOFT_SLOW_SENTINEL"])


SENTINEL = np.uint64(0x7ff8dead0000beef)


def _p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def random_doubles(rng, n, emin=-60, emax=60):
    """Random signs, uniformly random 52-bit fractions, exponents in [emin, emax]."""
    frac = rng.integers(0, 1 << 52, n, dtype=np.uint64)
    e = rng.integers(emin + 1023, emax + 1024, n).astype(np.uint64)
    s = rng.integers(0, 2, n).astype(np.uint64)
    return ((s << np.uint64(63)) | (e << np.uint64(52)) | frac).view(np.float64)


SPECIALS = np.array([0.0, -0.0, 5e-324, -5e-324, 2.2250738585072014e-308 / 3, 1e-310,
                     2.2250738585072014e-308, -2.2250738585072014e-308, 1.7976931348623157e308,
                     -1.7976931348623157e308, np.inf, -np.inf, np.nan, 1.0, -1.0, 0.5, 2.0,
                     1e-300, 1e300, 3e-308, 4e-308, 1e308])


def same_bits(a, b, normal_inputs):
    """Bitwise equality; slow-path sentinels are accepted only where an input
    lies outside the normal range or the result is not a normal number."""
    a64, b64 = a.view(np.uint64), b.view(np.uint64)
    nan = np.isnan(a) & np.isnan(b) & (a64 != SENTINEL)
    eq = (a64 == b64) | nan
    fast_case = normal_inputs & (np.abs(b) >= 2.2250738585072014e-308) & np.isfinite(b)
    slow_ok = (a64 == SENTINEL) & ~fast_case
    good = eq | slow_ok
    return np.all(good), np.flatnonzero(~good)


def normal(v):
    a = np.abs(v)
    return ((a >= 2.2250738585072014e-308) & np.isfinite(a)) | (a == 0)


def neighbours(v):
    """v and its next-up/next-down binary64 neighbours."""
    return np.concatenate([v, np.nextafter(v, np.inf), np.nextafter(v, -np.inf)])


DIVISORS = [0.01, 1.0 / 256, 0.1, 3.0, 0.7, 1.0, 0.5, 1.5, 0.001, 7.0e-6, 2.0 ** -40,
            2.0 ** 40 * 0.999, 0.0078125 * 1.0000000000000002]


@pytest.mark.parametrize("d", DIVISORS)
def test_div_const_matches_ieee(lib, d):
    rng = np.random.default_rng(int(d * 1e6) + 17)
    parts = [random_doubles(rng, 400_000), random_doubles(rng, 50_000, -1022, 1023),
             SPECIALS, neighbours(d * 2.0 ** np.arange(-30, 31)),
             neighbours(np.ldexp(d, np.arange(-1074, 1020, 7)))]
    x = np.concatenate(parts)
    with np.errstate(all="ignore"):
        want = x / d
    got = np.empty_like(x)
    lib.softfp_div_const(_p(x), x.size, d, _p(got))
    ok, bad = same_bits(got, want, normal(x))
    assert ok, (d, x[bad[:5]], got[bad[:5]], want[bad[:5]])


@pytest.mark.parametrize("y", [0.5, 2e-5, 1e-5, 0.04, 0.1, 0.06 + 0.04, 1.0, -3.0, 1.5,
                               1.0000000000000002, 1e300, 1e-300])
def test_mul_const_matches_ieee(lib, y):
    rng = np.random.default_rng(abs(hash(y)) % (1 << 31))
    short = (rng.integers(1, 1 << 12, 50_000) * 2.0 ** rng.integers(-30, 30, 50_000))
    x = np.concatenate([random_doubles(rng, 400_000), random_doubles(rng, 50_000, -1022, 1023),
                        SPECIALS, short, neighbours(1.0 / np.array([y]))])
    with np.errstate(all="ignore"):
        want = x * y
    got = np.empty_like(x)
    lib.softfp_mul_const(_p(x), x.size, y, _p(got))
    ok, bad = same_bits(got, want, normal(x))
    assert ok, (y, x[bad[:5]], got[bad[:5]], want[bad[:5]])


def test_mul_matches_ieee(lib):
    rng = np.random.default_rng(5)
    n = 1_000_000
    x = random_doubles(rng, n)
    y = random_doubles(rng, n)
    # exact ties: one factor with a short odd significand
    k = 200_000
    y[:k] = rng.integers(1, 1 << 10, k) * 2.0 ** rng.integers(-20, 20, k)
    # binade edges: y = (2^53 - j) / 2^52 style factors around 1 and 2
    y[k:k + 1000] = np.nextafter(1.0, 0.0)
    y[k + 1000:k + 2000] = np.nextafter(2.0, 0.0)
    # wide exponents (underflow / overflow to the slow path) and the specials
    xs = np.concatenate([x, random_doubles(rng, 100_000, -1022, 1023),
                         np.repeat(SPECIALS, SPECIALS.size)])
    ys = np.concatenate([y, random_doubles(rng, 100_000, -1022, 1023),
                         np.tile(SPECIALS, SPECIALS.size)])
    with np.errstate(all="ignore"):
        want = xs * ys
    got = np.empty_like(xs)
    lib.softfp_mul(_p(xs), _p(ys), xs.size, _p(got))
    ok, bad = same_bits(got, want, normal(xs) & normal(ys))
    assert ok, (xs[bad[:5]], ys[bad[:5]], got[bad[:5]], want[bad[:5]])


@pytest.mark.parametrize("k", [-1, 1, 3, -4, 10, -10, 62, -62, 0])
def test_scale_pow2_matches_ieee(lib, k):
    rng = np.random.default_rng(k + 100)
    x = np.concatenate([random_doubles(rng, 200_000), random_doubles(rng, 50_000, -1022, 1023),
                        SPECIALS, np.ldexp(1.0, np.arange(-1074, 1024))])
    with np.errstate(all="ignore"):
        want = x * (2.0 ** k)
    got = np.empty_like(x)
    lib.softfp_scale_pow2(_p(x), x.size, k, _p(got))
    ok, bad = same_bits(got, want, normal(x))
    assert ok, (k, x[bad[:5]], got[bad[:5]], want[bad[:5]])


def _ceil_recip115(md):
    """ceil(2^115 / md) in Python integers."""
    return [-((-(1 << 115)) // int(m)) for m in md]


def test_recip115_is_exact(lib):
    """The run-time reciprocal (binary32 seed, two fixed-point Newton steps,
    exact correction) equals ceil(2^115/md) for every significand tried: random
    ones, both ends of the binade, and the neighbourhoods of powers of two and
    of the points where the binary32 seed changes."""
    rng = np.random.default_rng(115)
    lo, hi = 1 << 52, 1 << 53
    md = [int(v) for v in rng.integers(lo, hi, 200_000, dtype=np.uint64)]
    md += list(range(lo, lo + 2000)) + list(range(hi - 2000, hi))
    for t in rng.integers(1 << 23, 1 << 24, 300):       # seed boundaries: top 24 bits change
        base = int(t) << 29
        md += [base - 1, base, base + 1, base + (1 << 28), base + (1 << 29) - 1]
    for k in range(1, 53):                               # 2^52 (1 + 2^-k) and neighbours
        m = lo + (lo >> k)
        md += [m - 1, m, m + 1]
    md = [m for m in md if lo <= m < hi]
    a = np.array(md, dtype=np.uint64)
    out = np.empty_like(a)
    lib.softfp_recip115(a.ctypes.data_as(ctypes.POINTER(ctypes.c_ulonglong)), a.size,
                        out.ctypes.data_as(ctypes.POINTER(ctypes.c_ulonglong)))
    want = np.array(_ceil_recip115(md), dtype=np.uint64)
    bad = np.flatnonzero(out != want)
    assert bad.size == 0, (a[bad[:5]], out[bad[:5]], want[bad[:5]])
    # the host-prepared constant (long division) gives the same words
    for d in (0.01, 3.0, 1.0, 0.7, 12.0 / 256):
        rh, rl = ctypes.c_uint(), ctypes.c_uint()
        lib.softfp_div_reciprocal_words(d, ctypes.byref(rh), ctypes.byref(rl))
        m = (int(np.float64(d).view(np.uint64)) & ((1 << 52) - 1)) | (1 << 52)
        assert (rh.value << 32) | rl.value == _ceil_recip115([m])[0]


def test_div_matches_ieee(lib):
    """x / y with both operands varying: random operands over wide and full
    exponent ranges, both signs, quotients at binade boundaries (x = y * 2^k
    and neighbours), and every pair of the special values."""
    rng = np.random.default_rng(23)
    n = 600_000
    x = random_doubles(rng, n)
    y = random_doubles(rng, n)
    k = 100_000
    t = y[:k] * 2.0 ** rng.integers(-10, 10, k)
    step = rng.integers(-1, 2, k)
    x[:k] = np.where(step > 0, np.nextafter(t, np.inf), np.where(step < 0, np.nextafter(t, -np.inf), t))
    xs = np.concatenate([x, random_doubles(rng, 100_000, -1022, 1023),
                         np.repeat(SPECIALS, SPECIALS.size)])
    ys = np.concatenate([y, random_doubles(rng, 100_000, -1022, 1023),
                         np.tile(SPECIALS, SPECIALS.size)])
    with np.errstate(all="ignore"):
        want = xs / ys
    got = np.empty_like(xs)
    lib.softfp_div(_p(xs), _p(ys), xs.size, _p(got))
    ok, bad = same_bits(got, want, normal(xs) & normal(ys) & (ys != 0))
    assert ok, (xs[bad[:5]], ys[bad[:5]], got[bad[:5]], want[bad[:5]])


@pytest.mark.parametrize("op", ["max", "min"])
def test_minmax_matches_fmax_fmin(lib, op):
    """fmax/fmin on the integer pipes: random pairs, pairs that are equal or
    adjacent, and every pair of the special values; the fast path must take
    every pair except NaNs and +0/-0 pairs."""
    rng = np.random.default_rng(31)
    n = 300_000
    x = random_doubles(rng, n, -1022, 1023)
    y = random_doubles(rng, n, -1022, 1023)
    y[:50_000] = x[:50_000]
    y[50_000:100_000] = np.nextafter(x[50_000:100_000], np.where(rng.random(50_000) < 0.5, np.inf, -np.inf))
    y[100_000:150_000] = -x[100_000:150_000]
    xs = np.concatenate([x, np.repeat(SPECIALS, SPECIALS.size)])
    ys = np.concatenate([y, np.tile(SPECIALS, SPECIALS.size)])
    want = np.fmax(xs, ys) if op == "max" else np.fmin(xs, ys)
    got = np.empty_like(xs)
    getattr(lib, "softfp_" + op)(_p(xs), _p(ys), xs.size, _p(got))
    special = np.isnan(xs) | np.isnan(ys) | ((xs == 0) & (ys == 0) & (np.signbit(xs) != np.signbit(ys)))
    g64, w64 = got.view(np.uint64), want.view(np.uint64)
    fast_ok = (g64 == w64) | (np.isnan(got) & np.isnan(want) & (g64 != SENTINEL))
    assert np.all(fast_ok[~special])
    assert np.all(fast_ok[special] | (g64[special] == SENTINEL))


def test_le_zero_matches_ieee(lib):
    rng = np.random.default_rng(37)
    x = np.concatenate([random_doubles(rng, 100_000, -1022, 1023), SPECIALS, -SPECIALS])
    got = np.empty(x.size, dtype=np.uint8)
    lib.softfp_le_zero(_p(x), x.size, got.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)))
    with np.errstate(invalid="ignore"):
        assert np.array_equal(got.astype(bool), x <= 0)


def test_comparisons_match_ieee(lib):
    rng = np.random.default_rng(41)
    n = 200_000
    x = random_doubles(rng, n, -1022, 1023)
    y = random_doubles(rng, n, -1022, 1023)
    y[:40_000] = x[:40_000]
    y[40_000:80_000] = np.nextafter(x[40_000:80_000], np.inf)
    y[80_000:120_000] = -x[80_000:120_000]
    xs = np.concatenate([x, np.repeat(SPECIALS, SPECIALS.size), np.repeat(-SPECIALS, SPECIALS.size)])
    ys = np.concatenate([y, np.tile(SPECIALS, SPECIALS.size), np.tile(SPECIALS, SPECIALS.size)])
    got = np.empty(xs.size, dtype=np.uint8)
    lib.softfp_cmp(_p(xs), _p(ys), xs.size, got.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)))
    with np.errstate(invalid="ignore"):
        assert np.array_equal((got & 1) != 0, xs < ys)
        assert np.array_equal((got & 2) != 0, xs <= ys)
        assert np.array_equal((got & 4) != 0, xs == ys)


def test_float_double_conversions_match_ieee(lib):
    """f2d_s (exact widening) and d2f_s (round to nearest even) against the
    host's conversions: every float exponent, random significands, doubles
    at and around binary32 rounding midpoints (ties to even both ways), the
    largest binade rounding to infinity, the subnormal boundary and specials.
    With the slow path replaced by the sentinel, every binary32-normal input
    must still convert on the fast path."""
    rng = np.random.default_rng(5)
    fp = ctypes.POINTER(ctypes.c_float)
    # widening
    bits = (rng.integers(0, 2 ** 32, 400000, dtype=np.uint64)).astype(np.uint32)
    special = np.array([0.0, -0.0, 1.0, -1.0, np.inf, -np.inf, np.nan, 1e-45, -1e-45,
                        1.17549435e-38, 3.4028235e38, -3.4028235e38], dtype=np.float32)
    xf = np.concatenate([bits.view(np.float32), special])
    out = np.empty(xf.size, dtype=np.float64)
    lib.softfp_f2d(xf.ctypes.data_as(fp), xf.size, _p(out))
    want = xf.astype(np.float64)
    e = (xf.view(np.uint32) >> 23) & 0xFF
    normal = ((e >= 1) & (e <= 254)) | (xf == 0)
    got_bits, want_bits = out.view(np.uint64), want.view(np.uint64)
    slow = got_bits == SENTINEL
    assert not slow[normal].any()
    ok = (got_bits == want_bits) | slow | (np.isnan(out) & np.isnan(want))
    assert ok.all(), xf[~ok][:5]
    # narrowing: random doubles over the binary32 range and beyond, and exact midpoints
    m = rng.integers(0, 2 ** 52, 300000, dtype=np.uint64)
    ex = rng.integers(1023 - 160, 1023 + 140, 300000, dtype=np.uint64)
    sg = rng.integers(0, 2, 300000, dtype=np.uint64) << np.uint64(63)
    xd = (sg | (ex << np.uint64(52)) | m).view(np.float64)
    f = rng.integers(1, 2 ** 31, 100000, dtype=np.uint64).astype(np.uint32).view(np.float32)
    f = f[np.isfinite(f)].astype(np.float64)
    mid = f.view(np.uint64) | np.uint64(1 << 28)  # exactly half a binary32 ulp above
    near = [mid, mid + np.uint64(1), mid - np.uint64(1)]
    edges = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 3.4028235677973366e38,
                      3.4028235677973362e38, 3.402823669209385e38, 1.1754943508222875e-38,
                      1.1754942106924411e-38, 1e-300, -1e300], dtype=np.float64)
    xd = np.concatenate([xd] + [a.view(np.float64) for a in near] + [edges])
    out = np.empty(xd.size, dtype=np.float32)
    lib.softfp_d2f(_p(xd), xd.size, out.ctypes.data_as(fp))
    with np.errstate(over="ignore"):
        want = xd.astype(np.float32)
    got_bits, want_bits = out.view(np.uint32), want.view(np.uint32)
    slow = np.isnan(out) & ~np.isnan(want)  # the sentinel narrows to a NaN
    wn = np.abs(want.astype(np.float64))
    in_range = (wn >= 1.1754943508222875e-38) & np.isfinite(want) | (xd == 0)
    assert not slow[in_range & (np.abs(xd) < 3.4028235677973366e38)].any()
    ok = (got_bits == want_bits) | slow | (np.isnan(out) & np.isnan(want))
    assert ok.all(), xd[~ok][:5]
