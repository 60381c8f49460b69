"""The FP32 gridder's integer update, restated in numpy (CPU).

The gridder caches every v kernel value as K = round(kv 2^31) (round half
to even, saturating at 2^31 - 1 for kv = 1), converts a lane's scaled value
once per item and plane to C = round(2 c) (saturating), and adds, per support
row, the high word of the 64-bit C K + 2^31 -- ``q31_mul_round`` in
``rascil_gb300/csrc/gb_invert.cu``.  The claim there: the result is within one
unit of round(kv c), for |c| <= 2^30 and kv in [0, 1], and closer than an FP32
product kv * c rounded to an integer at the same magnitudes."""
import numpy


def _round_sat_i32(x):
    r = numpy.rint(numpy.asarray(x, dtype=numpy.float64))  # half to even, as cvt.rni
    return numpy.clip(r, -2.0 ** 31, 2.0 ** 31 - 1).astype(numpy.int64)


def q31_update(kv, c):
    """The kernel's update for float32 kv in [0, 1] and float32 c."""
    kv = numpy.asarray(kv, dtype=numpy.float32)
    c = numpy.asarray(c, dtype=numpy.float32)
    K = _round_sat_i32(kv * numpy.float32(2.0 ** 31))
    C = _round_sat_i32(numpy.float32(2.0) * c)
    return (C * K + (1 << 31)) >> 32  # exact in int64: |C K| < 2^62


def test_q31_update_within_one_unit_of_the_exact_product():
    rng = numpy.random.default_rng(5)
    n = 1_000_000
    kv = rng.uniform(0.0, 1.0, n).astype(numpy.float32)
    kv[:4] = [0.0, 1.0, 1e-9, 0.5]
    c = (rng.uniform(-1.0, 1.0, n) * 2.0 ** rng.uniform(0, 30, n)).astype(numpy.float32)
    c[:4] = [2.0 ** 30, -(2.0 ** 30), 3.0, -7.5]
    got = q31_update(kv, c)
    exact = kv.astype(numpy.float64) * c.astype(numpy.float64)
    assert numpy.abs(got - numpy.rint(exact)).max() <= 1
    # an FP32 product rounded to an integer is further off at large magnitudes
    f32 = numpy.rint((kv * c).astype(numpy.float64))
    big = numpy.abs(exact) > 2.0 ** 26
    assert numpy.abs(f32[big] - numpy.rint(exact[big])).max() > 1
    assert numpy.abs(got[big] - numpy.rint(exact[big])).max() <= 1


def test_q31_update_sums_stay_in_int32():
    """A cell's sum over a chunk: every |c| is at most its item's share of
    2^30 (the chunk scale is 2^30 over the sum of the items' largest
    components) and every kv at most 1, so the sum of the updates stays
    within 2^30 plus one unit per update."""
    rng = numpy.random.default_rng(6)
    n = 256
    m = rng.uniform(0.0, 1.0, n)                    # items' largest components
    scale = 2.0 ** 30 / m.sum()
    c = (m * scale * rng.choice([-1.0, 1.0], n)).astype(numpy.float32)
    kv = numpy.ones(n, dtype=numpy.float32)          # the worst case: every kernel value 1
    total = int(q31_update(kv, c).astype(numpy.int64).sum())
    assert abs(total) <= 2 ** 30 + n < 2 ** 31
