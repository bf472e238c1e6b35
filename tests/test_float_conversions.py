"""The integer-pipe float <-> double conversions of csrc/cz_math.cuh (widen,
narrow), restated with numpy integer operations and checked against IEEE
conversions (numpy's astype: exact widening, round-to-nearest-even
narrowing) on random bit patterns of every magnitude, on ties and near-ties
of the rounding, and at the edges of float's range.  Values the kernels hand
to the conversion instruction (subnormal, out of range, infinite, NaN) are
only checked to be routed there.  CPU only; the GPU parity tests check the
kernels that use them bit for bit."""
import numpy as np


def widen_bits(f32):
    """(routed to the instruction, result bits) of widen() for float32 values."""
    b = f32.view(np.uint32).astype(np.uint64)
    e = (b >> 23) & 0xff
    m = b & 0x7fffff
    sign = b & 0x80000000
    normal = (e >= 1) & (e <= 254)
    hi = sign | ((e + 896) << 20) | (m >> 3)
    lo = (m << 29) & 0xffffffff
    out = np.where(normal, (hi << 32) | lo, 0)
    zero = ((b << 1) & 0xffffffff) == 0
    out = np.where(zero, sign << 32, out)
    return ~(normal | zero), out.astype(np.uint64)


def narrow_bits(f64):
    """(routed to the instruction, result bits) of narrow() for float64 values."""
    b = f64.view(np.uint64)
    hi = b >> 32
    lo = b & 0xffffffff
    e = (hi >> 20) & 0x7ff
    sign = hi & 0x80000000
    inrange = (e >= 897) & (e <= 1150)
    r = (((e - 896) & 0x7ff) << 23) | ((hi & 0xfffff) << 3) | (lo >> 29)
    rest = lo & 0x1fffffff
    up = (rest > 0x10000000) | ((rest == 0x10000000) & ((r & 1) == 1))
    r = (r + up.astype(np.uint64)) & 0xffffffff
    out = np.where(inrange, sign | r, 0)
    zero = (((hi << 1) & 0xffffffff) | lo) == 0
    out = np.where(zero, sign, out)
    return ~(inrange | zero), out.astype(np.uint32)


def test_widen_is_exact():
    rng = np.random.default_rng(1)
    bits = rng.integers(0, 2 ** 32, 2_000_000, dtype=np.uint64).astype(np.uint32)
    edges = np.array([0, 0x80000000, 1, 0x7fffff, 0x800000, 0x7f7fffff, 0x7f800000, 0xff800000, 0x7fc00000,
                      0x3f800000, 0xbf800000], dtype=np.uint32)
    f = np.concatenate([bits, edges]).view(np.float32)
    routed, got = widen_bits(f)
    want = f.astype(np.float64).view(np.uint64)
    ok = ~routed
    assert np.array_equal(got[ok], want[ok])
    e = (f.view(np.uint32) >> 23) & 0xff
    assert np.array_equal(routed, ((e == 0) & ((f.view(np.uint32) << 1) != 0)) | (e == 255))


def test_narrow_rounds_to_nearest_even():
    rng = np.random.default_rng(2)
    # every exponent of float's normal range and around it, random mantissas
    expo = rng.integers(880, 1170, 3_000_000, dtype=np.uint64)
    mant = rng.integers(0, 2 ** 52, 3_000_000, dtype=np.uint64)
    sign = rng.integers(0, 2, 3_000_000, dtype=np.uint64) << 63
    d = (sign | (expo << 52) | mant).view(np.float64)
    # exact ties and their neighbours (the low 29 bits at half, half +- 1)
    base = rng.integers(0, 2 ** 23, 200_000, dtype=np.uint64) << 29
    ties = []
    for low in (0x10000000, 0x0fffffff, 0x10000001, 0, 0x1fffffff):
        ties.append(((np.uint64(1023) << 52) | base | np.uint64(low)).view(np.float64))
    top = np.array([3.4028234663852886e38, 3.4028235677973366e38, 3.402823567797337e38, 3.4028236e38,
                    1.1754943508222875e-38, 1.1754942e-38, 0.0, -0.0, 1.0, -1.0, np.inf, -np.inf, np.nan])
    d = np.concatenate([d] + ties + [top])
    routed, got = narrow_bits(d)
    with np.errstate(over="ignore"):
        want = d.astype(np.float32).view(np.uint32)
    ok = ~routed
    assert np.array_equal(got[ok], want[ok])
    assert ok.sum() > 2_000_000
