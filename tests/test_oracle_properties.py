"""Property tests of the oracle's integer helpers and summation yardstick
(hypothesis; skipped where it is not installed): computeHash with 32-bit
wraparound (map_struct.cu:143-148), the voxel -> block / local split
(map_struct.cu:626-655), ToVector3i's floor (vector_type.h:218-225) and the
Kahan-compensated float sum against an exactly rounded sum."""
import ctypes as C
import math

import numpy as np
import pytest

hyp = pytest.importorskip("hypothesis")
from hypothesis import given, settings, strategies as st  # noqa: E402

I32 = st.integers(-(2 ** 31), 2 ** 31 - 1)


def _wrap32(v: int) -> int:
    v &= 0xFFFFFFFF
    return v - (1 << 32) if v >= 1 << 31 else v


def _compute_hash(x: int, y: int, z: int, n: int) -> int:
    r = _wrap32((x * 73856093) ^ (y * 19349669) ^ (z * 83492791))
    q = abs(r) % n  # C's % truncates toward zero
    r = q if r >= 0 else -q
    return r + n if r < 0 else r


@settings(max_examples=3000, deadline=None)
@given(I32, I32, I32, st.integers(1, 2 ** 31 - 1))
def test_compute_hash_is_the_wrapped_formula(oracle_lib, x, y, z, n):
    h = oracle_lib.or_compute_hash(x, y, z, n)
    assert 0 <= h < n
    assert h == _compute_hash(x, y, z, n)


@settings(max_examples=3000, deadline=None)
@given(st.integers(-(2 ** 31) + 8, 2 ** 31 - 1), st.integers(-(2 ** 31) + 8, 2 ** 31 - 1),
       st.integers(-(2 ** 31) + 8, 2 ** 31 - 1))
def test_voxel_splits_into_block_and_local(oracle_lib, x, y, z):
    v = (C.c_int * 3)(x, y, z)
    b, l = (C.c_int * 3)(), (C.c_int * 3)()
    oracle_lib.or_voxel_to_block(v, b)
    oracle_lib.or_voxel_to_local(v, l)
    for k, c in enumerate((x, y, z)):
        assert b[k] == c // 8 and l[k] == c % 8  # floor division, non-negative remainder
        assert b[k] * 8 + l[k] == c
    assert oracle_lib.or_local_idx(l) == l[2] * 64 + l[1] * 8 + l[0]


@settings(max_examples=3000, deadline=None)
@given(st.floats(-2.0 ** 30, 2.0 ** 30, width=32, allow_nan=False))
def test_to_vector3i_is_floor(oracle_lib, v):
    assert oracle_lib.or_floor_ref(v) == math.floor(v)


@settings(max_examples=300, deadline=None)
@given(st.lists(st.floats(-1e4, 1e4, width=32, allow_nan=False), min_size=1, max_size=2000))
def test_kahan_sum_within_its_bound(oracle_lib, xs):
    """Kahan's compensated sum: |error| <= (2 eps + O(n eps^2)) sum |x_i|
    (Higham, Accuracy and Stability of Numerical Algorithms, 2nd ed., 4.3)."""
    a = np.asarray(xs, np.float32)
    out = (C.c_double * 1)()
    oracle_lib.or_sum_f32(a.ctypes.data, len(a), 1, 1, out)
    exact = math.fsum(float(x) for x in a)
    eps = 2.0 ** -24
    bound = (2 * eps + len(a) * eps * eps) * float(np.abs(a.astype(np.float64)).sum()) + 1e-30
    # plus the final rounding of the exact sum to float
    assert abs(out[0] - exact) <= bound + eps * abs(exact)
