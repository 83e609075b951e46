"""Exhaustive checks of the arithmetic identities the kernels rely on, over
every int16 sdf code, with exact rational arithmetic (CPU only)."""
from fractions import Fraction

import numpy as np

CODES = range(-32767, 32768)


def _f32(x: Fraction) -> Fraction:
    """x rounded to the nearest float32 (ties to even), as a Fraction."""
    f = np.float32(float(x))
    cand = (np.nextafter(f, np.float32(-np.inf)), f, np.nextafter(f, np.float32(np.inf)))
    best = min(cand, key=lambda c: (abs(Fraction(float(c)) - x), int(np.float32(c).view(np.uint32)) & 1))
    return Fraction(float(best))


def test_ref_unpack_by_corrected_reciprocal():
    """REF voxels unpack as code / 32767.f (voxel.h:36-39); the kernels compute it
    as q = code * RN(1/32767) and one correction q + fma(-q, 32767, code) * RN(1/32767)
    with fused multiply-adds.  Every code gives the correctly rounded quotient."""
    r = Fraction(float(np.float32(1) / np.float32(32767)))
    d = Fraction(32767)
    bad = []
    for k in CODES:
        x = Fraction(k)
        q = _f32(x * r)
        e = _f32(-q * d + x)   # fma: exact product and sum, one rounding
        q2 = _f32(e * r + q)   # fma
        if q2 != _f32(x / d):
            bad.append(k)
    assert not bad, bad[:10]


def test_snorm_unit_round_trips():
    """SNORM voxels unpack as code * kSnormUnit, the float just above 1/32767:
    code * unit * 32767 >= code for every code, so the map dump's truncating
    pack (x 32767, toward zero) and the rounding SNORM pack both return the code."""
    k = np.arange(-32767, 32768, dtype=np.int32)
    unit = np.float32(float.fromhex("0x1.000202p-15"))
    assert unit == np.nextafter(np.float32(1) / np.float32(32767), np.float32(1))
    v = k.astype(np.float32) * unit
    t = v * np.float32(32767)
    assert np.array_equal(np.trunc(t).astype(np.int32), k)
    assert np.array_equal(np.rint(t).astype(np.int32), k)
    assert np.abs(v).max() <= np.float32(1) + np.float32(2.0 ** -23)


def _div_rn_by(a: Fraction, b: Fraction) -> Fraction:
    """The integration's running-mean quotient: y = RN(1/b), q0 = RN(a y), then
    twice q = RN(RN(a - b q) y + q) (fused multiply-adds)."""
    y = _f32(1 / b)
    q = _f32(a * y)
    for _ in range(2):
        r = _f32(a - b * q)
        q = _f32(r * y + q)
    return q


def test_running_mean_division_by_shared_reciprocal():
    """The four running means of an integration update (sdf and three colour
    channels, depth_fusion.cu:405-426) share the denominator w_old + w_new; the
    kernel divides each by the shared reciprocal with two remainder corrections.
    Over the updates' ranges (weights 1e-4..255, sdf codes, colours 0..255) and
    adversarial quotients (exact, one unit in the last place off, power-of-two
    denominators) the result is the correctly rounded quotient."""
    rng = np.random.default_rng(7)
    f = np.float32
    cases = []
    for _ in range(6000):
        w0 = f(10.0 ** rng.uniform(-4, np.log10(255)))
        w1 = f(10.0 ** rng.uniform(-4, 1.7))
        b = w0 + w1
        if rng.random() < 0.5:
            c0, c1 = f(rng.integers(0, 256)), f(rng.integers(0, 256))
        else:
            c0 = f(rng.integers(-32767, 32768)) * f(float.fromhex("0x1.000202p-15"))
            c1 = f(min(1.0, rng.uniform(-1.2, 1.2)))
        a = c0 * w0 + c1 * w1
        cases.append((a, b))
    for _ in range(1500):
        b = f(10.0 ** rng.uniform(-3, np.log10(510)))
        k = f(rng.integers(0, 256))
        a = k * b
        cases += [(a, b), (np.nextafter(a, f(np.inf)), b), (np.nextafter(a, f(0)), b)]
        p2 = f(2.0 ** rng.integers(-8, 9))
        cases.append((f(rng.uniform(0, 255)) * p2, p2))
    bad = []
    for a, b in cases:
        A, B = Fraction(float(a)), Fraction(float(b))
        if _div_rn_by(A, B) != _f32(A / B):
            bad.append((float(a), float(b)))
    assert not bad, bad[:5]
