"""The 2D perturbed-heightmap field of the oracle (BMF_FIELD_TERRAIN_2D; CPU only).

Its noises are this project's restatement of the reference's FastNoiseSIMD
sampler shape (NoiseSampler.cpp:148-194, not vendored): parity with the
reference is unpinned, so these tests hold the oracle's float evaluation to an
independent FP64 evaluation written here in numpy, check the value ranges the
field's definition implies, and check that the reference's default settings
(WorldOctree.cpp:49-55) give a surface inside the world band.
"""
import numpy as np

from binarymeshfitting_gb300 import workloads
from oracle import cpu

P2 = workloads.TERRAIN_2D_PARAMS


def fade64(t):
    return t * t * t * (t * (t * 6.0 - 15.0) + 10.0)


def grad2_64(h, x, z):
    h = h & 7
    gx = np.where(h < 4, np.where(h & 1, -1.0, 1.0), np.where(h & 2, 0.0, np.where(h & 1, -1.0, 1.0)))
    gz = np.where(h < 4, np.where(h & 2, -1.0, 1.0), np.where(h & 2, np.where(h & 1, -1.0, 1.0), 0.0))
    return gx * x + gz * z


def lattice(perm, x, z, off=0):
    P = lambda i: perm[np.asarray(i) & 255].astype(np.int64)  # noqa: E731
    fx, fz = np.floor(x), np.floor(z)
    X, Z = fx.astype(np.int64) & 255, fz.astype(np.int64) & 255
    xf, zf = x - fx, z - fz
    A, B = P(X + off) + Z, P(X + 1 + off) + Z
    return P, A, B, xf, zf, fade64(xf), fade64(zf)


def lerp(t, a, b):
    return a + t * (b - a)


def noise2_grad64(perm, c, x, z):
    P, A, B, xf, zf, u, w = lattice(perm, x, z, 73 * c)
    return lerp(w, lerp(u, grad2_64(P(A), xf, zf), grad2_64(P(B), xf - 1, zf)),
                lerp(u, grad2_64(P(A + 1), xf, zf - 1), grad2_64(P(B + 1), xf - 1, zf - 1)))


def noise2_value64(perm, x, z):
    P, A, B, xf, zf, u, w = lattice(perm, x, z)
    v = lambda h: h * (2.0 / 255.0) - 1.0  # noqa: E731
    return lerp(w, lerp(u, v(P(A)), v(P(B))), lerp(u, v(P(A + 1)), v(P(B + 1))))


def height64(perm, p, px, pz):
    xn, zn = px * p[0] * 0.01, pz * p[0] * 0.01
    a, fr = p[3], p[4]
    for _ in range(int(p[2])):
        sx, sz = xn * fr, zn * fr
        xn, zn = xn + a * noise2_grad64(perm, 0, sx, sz), zn + a * noise2_grad64(perm, 1, sx, sz)
        fr, a = fr * 2.0, a * p[5]
    s = b = 0.0
    amp, vf = 1.0, 1.0
    for _ in range(int(p[7])):
        s, b = s + amp * noise2_value64(perm, xn * vf, zn * vf), b + amp
        vf, amp = vf * 2.0, amp * 0.5
    return s / b


def test_noises_match_fp64_and_stay_in_range():
    perm = cpu.perm(1337)
    rng = np.random.default_rng(3)
    pts = np.concatenate([rng.uniform(-300.0, 300.0, (2000, 2)), rng.uniform(254.0, 258.0, (200, 2))])
    for x, z in pts.astype(np.float32):
        for c in (0, 1):
            g = cpu.noise2(perm, float(x), float(z), "grad", c)
            assert abs(g - noise2_grad64(perm, c, np.float64(x), np.float64(z))) <= 2e-6
            assert abs(g) <= 1.0 + 1e-6
        v = cpu.noise2(perm, float(x), float(z), "value")
        assert abs(v - noise2_value64(perm, np.float64(x), np.float64(z))) <= 2e-6
        assert abs(v) <= 1.0 + 1e-6


def test_height_matches_fp64_with_few_perturb_octaves():
    """The perturbation chains noise into coordinates, so float and FP64 drift
    apart with many high-frequency octaves; with 3 they agree closely."""
    perm = cpu.perm(1337)
    p = list(P2)
    p[2] = 3
    rng = np.random.default_rng(5)
    for x, z in rng.uniform(-2000.0, 6000.0, (300, 2)).astype(np.float32):
        h = cpu.terrain2d_height(p, float(x), float(z))
        assert abs(h - height64(perm, p, np.float64(x), np.float64(z))) <= 1e-4
        assert abs(h) <= 1.0 + 1e-6


def test_reference_defaults_give_a_surface_in_the_band():
    """-(y g) - height n = 0 at y = -height n / g: the surface of the default
    settings lies within |y| <= 300, and a column's density falls with y."""
    hs = np.array([cpu.terrain2d_height(P2, float(x), float(z))
                   for x, z in np.random.default_rng(7).uniform(0.0, 4096.0, (400, 2))])
    assert np.abs(hs).max() <= 1.0 and hs.std() > 0.05
    d = cpu.fill_field(7, list(P2), 17, (100.0, -40.0, 300.0), 5.0).reshape(17, 17, 17)
    assert (np.diff(d, axis=1) < 0).all()
    assert (d < 0).any() and (d > 0).any()
