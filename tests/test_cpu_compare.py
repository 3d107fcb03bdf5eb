"""The integer forms of FP64 comparisons the kernels use (ge0, lt0, le0, gt0,
eq0, lt_pos, ge_pos, gt_pos in cmcg_internal.cuh), restated here on the
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
