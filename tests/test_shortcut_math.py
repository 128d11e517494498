"""The float shortcuts the CUDA kernels take in place of IEEE divisions, restated in numpy float32
and checked against the divisions they replace (the kernels' own results are checked bit for bit
against the oracle by the GPU tests; these tests check the error arguments the shortcuts rest on):

- carve_kernel's voxel_of: (int) (x / res) from x * (1 / res) away from integer quotients;
- update_kernel's far test: |p| > far / (z / |p|) decided by z against far away from the plane;
- the ICP's exact merge: a float split into a fixed-point integer part (2^-10) and fraction
  (2^-50) whose sum equals the float to 2^-50.
"""
from fractions import Fraction

import numpy as np

f32 = np.float32


def _voxel_of(x, res):
    inv = f32(1.0) / res
    q = (x * inv).astype(f32)
    f = (q - np.trunc(q)).astype(f32)
    tol = (q * f32(2.0 ** -20)).astype(f32)
    fast = (f > tol) & (f < f32(1.0) - tol)
    exact = (x / res).astype(f32).astype(np.int64)
    return np.where(fast, q.astype(np.int64), exact), exact, fast


def test_voxel_of_matches_the_division():
    rng = np.random.default_rng(11)
    for res in (0.01, 0.02, 0.4, 0.005, 0.0123):
        res = f32(res)
        dim = f32(1024) * res
        k = rng.integers(0, 1024, 100_000).astype(f32)
        on = (k * res).astype(f32)          # quotients at or next to integers
        x = np.concatenate([(rng.random(1_000_000, dtype=np.float32) * dim).astype(f32), on,
                            np.nextafter(on, f32(0)), np.nextafter(on, f32(1e9)), np.zeros(1, f32)])
        got, exact, fast = _voxel_of(x, res)
        assert np.array_equal(got, exact)
        assert fast[:1_000_000].mean() > 0.99   # the division is the exception


def _far_test(p):
    far = f32(6.0)
    x, y, z = p[:, 0], p[:, 1], p[:, 2]
    sq = ((x * x).astype(f32) + (y * y).astype(f32)).astype(f32)
    sq = (sq + (z * z).astype(f32)).astype(f32)
    pn = np.sqrt(sq).astype(f32)
    exact = pn > (far / (z / pn).astype(f32)).astype(f32)
    lo = (far * f32(1 - 2.0 ** -16)).astype(f32)
    hi = (far * f32(1 + 2.0 ** -16)).astype(f32)
    fast = np.where(z < lo, False, np.where(z > hi, True, exact))
    return fast, exact


def test_far_test_matches_the_divisions():
    rng = np.random.default_rng(12)
    n = 2_000_000
    z = np.concatenate([(f32(6.0) * (1 + rng.standard_normal(n) * 1e-4)).astype(f32),
                        (rng.random(n) * 12 + 1e-3).astype(f32)])
    p = np.stack([(rng.standard_normal(2 * n) * 3).astype(f32), (rng.standard_normal(2 * n) * 3).astype(f32), z], 1)
    fast, exact = _far_test(p)
    assert np.array_equal(fast, exact)


def _fixed_split(v):
    b = int(np.array(v, np.float32).view(np.uint32))
    e = (b >> 23) & 0xff
    m = (b & 0x7fffff) | (0x800000 if e else 0)
    ee = e if e else 1
    if e == 0xff or ee > 164:
        return None
    i, f = 0, 0
    if ee >= 140:
        i = m << (ee - 140)
    elif ee >= 100:
        x = m << (ee - 100)
        i, f = x >> 40, x & ((1 << 40) - 1)
    elif 100 - ee < 24:
        f = m >> (100 - ee)
    if b >> 31:
        i, f = (-i - 1, (1 << 40) - f) if f else (-i, 0)
    return i, f


def test_fixed_split_is_exact_to_2_pow_minus_50():
    rng = np.random.default_rng(13)
    vals = list((rng.standard_normal(20_000) * 10.0 ** rng.integers(-20, 11, 20_000)).astype(np.float32))
    vals += [f32(0.0), f32(-0.0), f32(1.0), f32(-1.0), f32(2.0 ** -50), f32(-3e-16), f32(2.7e11), f32(-2.7e11)]
    for v in vals:
        i, f = _fixed_split(v)
        assert 0 <= f < 2 ** 40
        got = Fraction(i, 2 ** 10) + Fraction(f, 2 ** 50)
        assert abs(got - Fraction(float(v))) < Fraction(1, 2 ** 50)
        assert abs(got) <= abs(Fraction(float(v)))   # truncation toward zero
    assert _fixed_split(f32(5e12)) is None           # outside the range: the overflow flag
    assert _fixed_split(f32(-2.8e11)) is None        # |v| >= 2^38: the count byte's headroom
    assert _fixed_split(f32(np.inf)) is None
