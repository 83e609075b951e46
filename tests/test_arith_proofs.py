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
