"""The fast path's six normals from one 128-bit Philox block (box_muller6_f32
in csrc/spss_internal.cuh), restated in numpy on uniform random blocks:
three Box-Muller pairs with 24-bit radius uniforms (the top 24 bits of words
0-2) and 16-bit angle uniforms (the halves of word 3, and the low bytes of
words 0 and 1).  The scheme itself gives standard normals: moments, tail
mass, and no correlation between the six values or their squares."""
import numpy as np


def six_normals(words):
    w = words.astype(np.uint64)
    radius = [w[:, 0] >> 8, w[:, 1] >> 8, w[:, 2] >> 8]
    angle = [w[:, 3] & 0xFFFF, w[:, 3] >> 16, (w[:, 0] & 0xFF) | ((w[:, 1] & 0xFF) << 8)]
    z = []
    for a, b in zip(radius, angle):
        u1 = (a + 0.5) * 2.0 ** -24
        theta = ((b + 0.5) * 2.0 ** -16 - 0.5) * 2 * np.pi
        r = np.sqrt(-2.0 * np.log(u1))
        z += [r * np.cos(theta), r * np.sin(theta)]
    return np.stack(z, axis=1)


def test_six_normals_are_standard_and_independent():
    rng = np.random.default_rng(5)
    words = rng.integers(0, 2 ** 32, size=(1_000_000, 4), dtype=np.uint64)
    z = six_normals(words)
    m = z.shape[0]
    assert np.abs(z.mean(axis=0)).max() < 5 / np.sqrt(m)
    assert np.abs(z.var(axis=0) - 1.0).max() < 5 * np.sqrt(2.0 / m)
    assert np.abs((z ** 4).mean(axis=0) - 3.0).max() < 5 * np.sqrt(96.0 / m)
    tail = (np.abs(z) > 3.0).mean(axis=0)
    assert np.abs(tail - 2.6998e-3).max() < 5 * np.sqrt(2.7e-3 / m)
    off = ~np.eye(6, dtype=bool)
    assert np.abs(np.corrcoef(z.T)[off]).max() < 5 / np.sqrt(m)
    assert np.abs(np.corrcoef((z ** 2).T)[off]).max() < 5 / np.sqrt(m)

