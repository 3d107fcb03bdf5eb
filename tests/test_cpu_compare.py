"""The integer forms of FP64 comparisons the kernels use (ge0, lt0, le0, gt0,
eq0, lt_pos, ge_pos, gt_pos, okey/bound_key/gt_key in cmcg_internal.cuh), restated here on the
uint64 bit patterns and checked against IEEE comparisons over signed zeros,
subnormals, infinities, NaNs of both signs and random values."""
import numpy as np

SIGN, INF = np.uint64(0x8000000000000000), np.uint64(0x7FF0000000000000)


def bits(x):
    return np.asarray(x, dtype=np.float64).view(np.uint64)


def ge0(x):
    b = bits(x)
    return (b <= INF) | (b == SIGN)


def lt0(x):
    b = bits(x)
    return (b > SIGN) & (b <= (SIGN | INF))


def le0(x):
    b = bits(x)
    return (b == 0) | ((b >= SIGN) & (b <= (SIGN | INF)))


def gt0(x):
    b = bits(x)
    return (b != 0) & (b <= INF)


def eq0(x):
    return (bits(x) & ~SIGN) == 0


def lt_pos(x, c):
    b = bits(x)
    return np.where(b < SIGN, b < bits(c), b <= (SIGN | INF))


def ge_pos(x, c):
    b = bits(x)
    return (b >= bits(c)) & (b <= INF)


def gt_pos(x, c):
    b = bits(x)
    return (b > bits(c)) & (b <= INF)


def okey(x):
    b = np.atleast_1d(bits(x)).astype(object)
    m = [int(v) & ~int(SIGN) for v in b]
    return [-mm if (int(v) & int(SIGN)) else mm for v, mm in zip(b, m)]


def bound_key(c):
    return (1 << 63) - 1 if (int(bits(c)) & ~int(SIGN)) > int(INF) else okey(c)[0]


def gt_key(x, kc):
    m = [int(v) & ~int(SIGN) for v in bits(x).astype(object)]
    return np.array([mm <= int(INF) and k > kc for mm, k in zip(m, okey(x))])


def _values():
    rng = np.random.default_rng(3)
    special = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, -np.nan, 5e-324, -5e-324, 2.2250738585072014e-308,
                        1e-20, -1e-20, 1.0, -1.0, 1e10, np.finfo(np.float64).max, -np.finfo(np.float64).max])
    neg_nan = np.array([0xFFF8000000000001], dtype=np.uint64).view(np.float64)
    rnd = rng.normal(size=4000) * 10.0 ** rng.integers(-30, 30, size=4000)
    return np.concatenate([special, neg_nan, rnd, -rnd])


def test_zero_comparisons_match_ieee():
    x = _values()
    with np.errstate(invalid="ignore"):
        assert np.array_equal(ge0(x), x >= 0.0)
        assert np.array_equal(lt0(x), x < 0.0)
        assert np.array_equal(le0(x), x <= 0.0)
        assert np.array_equal(gt0(x), x > 0.0)
        assert np.array_equal(eq0(x), x == 0.0)


def test_positive_constant_comparisons_match_ieee():
    x = _values()
    for c in (1e-20, 2.2250738585072014e-308, 0.19634954084936207, 1.5707963267948966, 1.0, 1e10,
              np.finfo(np.float64).max):
        with np.errstate(invalid="ignore"):
            assert np.array_equal(lt_pos(x, c), x < c), c
            assert np.array_equal(ge_pos(x, c), x >= c), c
            assert np.array_equal(gt_pos(x, c), x > c), c
    # the kernels' constant helpers and these restatements read the same patterns
    assert bits(0.0) == 0 and bits(-0.0) == SIGN and bits(np.inf) == INF


def test_signed_bound_comparisons_match_ieee():
    # k_tidal's criterion E > gierszalpha * phi_rtidal (a negative bound) or
    # r_apo > Rtidal, on ordered integer keys
    x = _values()
    for c in (-0.7321, -1e-20, -0.0, 0.0, 1e-20, 3.5, -np.inf, np.inf, np.nan, -np.nan, 5e-324, -5e-324):
        with np.errstate(invalid="ignore"):
            assert np.array_equal(gt_key(x, bound_key(c)), x > c), c


def f2_split(x):
    """hi = RN(x) to float and lo = RN(x - hi), as cmcg_internal.cuh forms them
    from the bits (fast path for 2^-74 <= |x| < 2^127, else conversions)."""
    x = float(x)
    b = int(np.array([x]).view(np.uint64)[0])
    ed = (b >> 52) & 0x7FF
    if ed < 949 or ed > 1149:
        hi = np.float32(x)
        return hi, np.float32(x - float(hi))
    S = (b & 0x000FFFFFFFFFFFFF) | (1 << 52)
    H = S >> 29
    rem = S & ((1 << 29) - 1)
    if rem > (1 << 28) or (rem == (1 << 28) and (H & 1)):
        H += 1
    D = S - (H << 29)
    sgn = (b >> 32) & 0x80000000
    hb = (((ed - 896) << 23) + (H - (1 << 23))) | sgn
    hi = np.array([hb], dtype=np.uint32).view(np.float32)[0]
    scale = np.array([(ed - 1075 + 127) << 23], dtype=np.uint32).view(np.float32)[0]
    lo = np.float32(np.float32(D) * scale)  # D as float rounds to nearest; the scaling is exact
    return hi, (-lo if sgn else lo)


def test_float_split_matches_conversions():
    rng = np.random.default_rng(9)
    xs = list(rng.normal(size=20000) * 10.0 ** rng.integers(-22, 30, size=20000))
    # ties of the 29 dropped bits, the float range edges and both fallbacks
    for k in (1, 3, 1 << 20, (1 << 23) - 1):
        for e in (0, -40, 60):
            t = (k + 0.5) * 2.0 ** (e - 23)  # exactly halfway between floats
            xs += [t, -t, np.nextafter(t, 0), np.nextafter(t, 1e300)]
    xs += [0.0, -0.0, 2.0 ** -74, 2.0 ** -75, 2.0 ** 126 * 1.999, 2.0 ** 127, 3.4e38, 1e-40, 5e-324]
    for x in xs:
        hi, lo = f2_split(x)
        want_hi = np.float32(x)
        assert hi == want_hi and np.signbit(hi) == np.signbit(want_hi), x
        want_lo = np.float32(x - float(want_hi))
        assert lo == want_lo, (x, lo, want_lo)
