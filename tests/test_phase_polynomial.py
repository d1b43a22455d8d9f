"""The sine and cosine of the fast path's fixed-point phase (phase_sincos in
csrc/fast_path.cu), restated in float32 arithmetic with the coefficients read
from the source: within 1e-7 of the exact values over sampled phases, the
quarter-turn boundaries and the extremes, and exactly antisymmetric /
symmetric under a half turn."""
import os
import re

import numpy as np

SRC = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "spsslangevinintegration_gb300", "csrc",
                   "fast_path.cu")
f32 = np.float32


def coefficients():
    src = open(SRC).read()
    body = src[src.index("void phase_sincos(uint32_t P"):]
    body = body[:body.index("\n}\n")]
    nums = [float(x[:-1]) for x in re.findall(r"-?\d+\.\d+(?:e-?\d+)?f", body)]
    # order in the source: 2 pi / 2^32, then sine (s3, s2, s1), then cosine (c4, c3, c2, c1, 1)
    scale = nums[0]
    s3, s2, s1 = nums[1], nums[2], nums[3]
    c4, c3, c2, c1, one = nums[4], nums[5], nums[6], nums[7], nums[8]
    assert one == 1.0 and abs(scale - 2 * np.pi / 2 ** 32) < 1e-18
    return scale, (s1, s2, s3), (c1, c2, c3, c4)


def fma(a, b, c):
    # float32 fused multiply-add: the float32 product is exact in float64,
    # one rounding of the float64 sum is the fused result except in rare ties
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(f32)


def phase_sincos(P):
    scale, (s1, s2, s3), (c1, c2, c3, c4) = coefficients()
    P = P.astype(np.uint64)
    qd = ((P + 0x20000000) >> 30) & 3
    r = ((P - (((P + 0x20000000) >> 30) << 30)) & 0xFFFFFFFF).astype(np.uint32).view(np.int32)
    th = (r.astype(f32) * f32(scale)).astype(f32)
    t2 = (th * th).astype(f32)
    full = lambda v: np.full_like(t2, f32(v))  # noqa: E731
    ps = fma(th, (t2 * fma(t2, fma(t2, full(s3), full(s2)), full(s1))).astype(f32), th)
    pc = fma(t2, fma(t2, fma(t2, fma(t2, full(c4), full(c3)), full(c2)), full(c1)), full(1.0))
    odd = (qd & 1) == 1
    a = np.where(odd, pc, ps)
    b = np.where(odd, ps, pc)
    s = np.where((qd & 2) != 0, -a, a)
    c = np.where(((qd + 1) & 2) != 0, -b, b)
    return s, c


def test_accuracy_over_sampled_phases_and_boundaries():
    rng = np.random.default_rng(0)
    P = rng.integers(0, 2 ** 32, size=1_000_000, dtype=np.uint64).astype(np.uint32)
    edges = np.array([0, 1, 2 ** 29 - 1, 2 ** 29, 2 ** 29 + 1, 2 ** 30 - 1, 2 ** 30, 2 ** 31 - 1, 2 ** 31,
                      3 * 2 ** 29, 3 * 2 ** 30, 2 ** 32 - 1, 2 ** 32 - 2 ** 29], dtype=np.uint64).astype(np.uint32)
    P = np.concatenate([P, edges])
    s, c = phase_sincos(P)
    phi = P.astype(np.float64) * (2 * np.pi / 2 ** 32)
    assert np.abs(s - np.sin(phi)).max() <= 1e-7
    assert np.abs(c - np.cos(phi)).max() <= 1e-7
    assert np.all(np.abs(s) <= 1.0) and np.all(np.abs(c) <= 1.0)


def test_half_turn_symmetry_is_exact():
    rng = np.random.default_rng(1)
    P = rng.integers(0, 2 ** 32, size=100_000, dtype=np.uint64).astype(np.uint32)
    s0, c0 = phase_sincos(P)
    s1, c1 = phase_sincos((P.astype(np.uint64) + 2 ** 31).astype(np.uint32))
    np.testing.assert_array_equal(s1, -s0)
    np.testing.assert_array_equal(c1, -c0)
