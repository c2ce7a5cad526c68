"""The band fill's per-octave noise bound (kNoiseBound in csrc/bmf_sample.cu).

The band fill stops a run's octaves once kNoiseBound * (sum of the remaining
octaves' |amplitude|) cannot change any sample's sign, so the bound must hold
for every input or the occupancy words would be wrong.  At offsets (u, v, w)
in the lattice cell, improved noise is sum_c W_c (g_c . d_c) with corner
weights W_c >= 0 summing to one and gradients with two components +/-1, so
|noise| <= F(u, v, w) = sum_c W_c m_c, m_c the sum of the two largest of
|u - cx|, |v - cy|, |w - cz|.  |dF/du| <= fade' + 1 <= 1.875 + 1 (likewise in
v, w), so F <= (its maximum on a grid of spacing h) + 3 * 2.875 * h / 2.
"""
import os
import re

import numpy as np

from oracle import cpu

HERE = os.path.dirname(os.path.abspath(__file__))
SAMPLE_CU = os.path.join(HERE, "..", "binarymeshfitting_gb300", "csrc", "bmf_sample.cu")


def _kernel_bound():
    m = re.search(r"constexpr float kNoiseBound = ([0-9.]+)f;", open(SAMPLE_CU).read())
    assert m, "kNoiseBound not found"
    return float(m.group(1))


def _fade(t):
    return t * t * t * (t * (t * 6.0 - 15.0) + 10.0)


def test_noise_bound_covers_improved_noise():
    n = 201
    h = 1.0 / (n - 1)
    g = np.linspace(0.0, 1.0, n)
    u, v = np.meshgrid(g, g, indexing="ij")
    su, sv = _fade(u), _fade(v)
    fmax = 0.0
    for w in g:  # one z-slice at a time keeps memory small
        sw = _fade(w)
        f = np.zeros_like(u)
        for cx in (0, 1):
            for cy in (0, 1):
                for cz in (0, 1):
                    wc = (su if cx else 1 - su) * (sv if cy else 1 - sv) * (sw if cz else 1 - sw)
                    d = np.stack([np.abs(u - cx), np.abs(v - cy), np.full_like(u, abs(w - cz))])
                    f += wc * (d.sum(0) - d.min(0))
        fmax = max(fmax, float(f.max()))
    bound = fmax + 3 * 2.875 * h / 2
    assert 1.03 < fmax < 1.04  # the known maximum of improved noise, about 1.036
    assert bound <= _kernel_bound(), (fmax, bound, _kernel_bound())


def test_sampled_noise_within_bound():
    rng = np.random.default_rng(7)
    p = rng.uniform(-300.0, 300.0, (20_000, 3))
    perm = cpu.perm(1337)
    vals = np.array([cpu.perlin(perm, float(x), float(y), float(z)) for x, y, z in p])
    assert 0.8 < np.abs(vals).max() <= _kernel_bound()
