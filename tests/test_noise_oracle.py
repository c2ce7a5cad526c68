"""The terrain noise of the oracle (CPU only).

The FBM field evaluates improved gradient noise (K. Perlin, SIGGRAPH 2002) in
line-separable form: each corner gradient is split into an x/y part s and a z
coefficient c, a z-layer's x/y interpolant is alpha + beta * zk, and the
value is l0 + w (l1 - l0).  That is the textbook value in exact arithmetic;
these tests hold the float evaluation to an independent FP64 textbook
evaluation written here in numpy, and to the oracle's textbook-order float
evaluation, on seeded points that include lattice wrap-around (cells 255 -> 0)
and negative coordinates.
"""
import numpy as np
import pytest

from oracle import cpu


def fade64(t):
    return t * t * t * (t * (t * 6.0 - 15.0) + 10.0)


def grad64(h, x, y, z):
    h = h & 15
    u = np.where(h < 8, x, y)
    v = np.where(h < 4, y, np.where((h == 12) | (h == 14), x, z))
    return np.where(h & 1, -u, u) + np.where(h & 2, -v, v)


def perlin64(perm, x, y, z):
    """Textbook improved noise in float64 (numpy, vectorised)."""
    P = lambda i: perm[np.asarray(i) & 255].astype(np.int64)  # noqa: E731
    fx, fy, fz = np.floor(x), np.floor(y), np.floor(z)
    X, Y, Z = fx.astype(np.int64) & 255, fy.astype(np.int64) & 255, fz.astype(np.int64) & 255
    x, y, z = x - fx, y - fy, z - fz
    u, v, w = fade64(x), fade64(y), fade64(z)
    A, B = P(X) + Y, P(X + 1) + Y
    AA, AB, BA, BB = P(A) + Z, P(A + 1) + Z, P(B) + Z, P(B + 1) + Z
    lerp = lambda t, a, b: a + t * (b - a)  # noqa: E731
    l0 = lerp(v, lerp(u, grad64(P(AA), x, y, z), grad64(P(BA), x - 1, y, z)),
              lerp(u, grad64(P(AB), x, y - 1, z), grad64(P(BB), x - 1, y - 1, z)))
    l1 = lerp(v, lerp(u, grad64(P(AA + 1), x, y, z - 1), grad64(P(BA + 1), x - 1, y, z - 1)),
              lerp(u, grad64(P(AB + 1), x, y - 1, z - 1), grad64(P(BB + 1), x - 1, y - 1, z - 1)))
    return lerp(w, l0, l1)


@pytest.fixture(scope="module")
def points():
    rng = np.random.default_rng(1337)
    pts = rng.uniform(-300.0, 300.0, (4000, 3)).astype(np.float32)
    # z close to the 255 -> 0 wrap of the lattice cell, and integer coordinates
    wrap = np.stack([rng.uniform(-50, 50, 500), rng.uniform(-50, 50, 500), rng.uniform(254.0, 257.0, 500)], 1)
    ints = rng.integers(-260, 260, (500, 3))
    return np.concatenate([pts, wrap.astype(np.float32), ints.astype(np.float32)])


def test_separable_noise_matches_fp64_textbook(points):
    perm = cpu.perm(1337)
    got = np.array([cpu.perlin(perm, *p) for p in points], np.float64)
    ref = perlin64(perm, *points.astype(np.float64).T)
    tb = np.array([cpu.perlin(perm, *p, textbook=True) for p in points], np.float64)
    assert np.abs(ref).max() < 1.1
    # float evaluations of a value bounded by ~1: a few ulps of 1.0 each
    assert np.abs(got - ref).max() < 1e-6, np.abs(got - ref).max()
    assert np.abs(tb - ref).max() < 1e-6, np.abs(tb - ref).max()
    # the two float orders differ by rounding only
    assert np.abs(got - tb).max() < 1e-6
    # integer lattice points: all fractions are 0, every gradient term vanishes
    n_int = 500
    assert np.all(got[-n_int:] == 0.0) and np.all(ref[-n_int:] == 0.0)


def test_terrain_field_matches_fp64_fbm():
    """The FBM terrain field (5 octaves) against an FP64 textbook FBM on a
    33^3 chunk at cell size 8 (the coarsest LOD: a new z lattice cell at most
    samples of the high octaves)."""
    params = [64.0, 40.0, 0.01, 2.0, 0.5, 5, 1337]
    dim, org, scale = 33, (1024.0, 0.0, 2048.0), 8.0
    d = cpu.fill_field(2, params, dim, org, scale).astype(np.float64)
    g = np.arange(dim, dtype=np.float32) * np.float32(scale)
    X, Y, Z = np.meshgrid(g + np.float32(org[0]), g + np.float32(org[1]), g + np.float32(org[2]), indexing="ij")
    perm = cpu.perm(1337)
    fbm = np.zeros(dim ** 3)
    amp, fr = 1.0, np.float32(0.01)
    for _ in range(5):
        # the field scales coordinates in float, as the kernel does
        xs, ys, zs = [(c.astype(np.float32) * fr).astype(np.float64).ravel() for c in (X, Y, Z)]
        fbm += amp * perlin64(perm, xs, ys, zs)
        amp *= 0.5
        fr = np.float32(fr * np.float32(2.0))
    ref = (Y.ravel().astype(np.float64) - 64.0) - 40.0 * fbm
    assert np.abs(d - ref).max() < 2e-4, np.abs(d - ref).max()
