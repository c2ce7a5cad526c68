"""Seeded synthetic workloads of the chunk-extraction path.

* ``sphere_wave_field``: |p - (32,32,32)| - 20 + 1.5 sin(0.3x) sin(0.3y) sin(0.3z)
  on one 65^3-sample chunk at unit spacing.
* ``terrain_field``: y - 64 - 40 FBM(p), 5 octaves of improved gradient noise,
  base frequency 0.01, lacunarity 2, gain 0.5, seed 1337, on 129^3 samples.
* ``lod_update``: a WorldOctree-style update of 4096 chunks of the terrain field
  at mixed LOD inside a 4096^3 world: 50% 32^3-cell, 35% 64^3-cell and 15%
  128^3-cell chunks; cell size 1/2/4/8 world units by LOD level; chunk origins
  snapped to the chunk extent around a seeded camera near the terrain band.
"""
import numpy as np

from ._lib import ChunkDesc, Field, FIELD_SPHERE_WAVE, FIELD_TERRAIN_2D, FIELD_TERRAIN_FBM

WORLD = 4096.0
TERRAIN_PARAMS = (64.0, 40.0, 0.01, 2.0, 0.5, 5, 1337)
SPHERE_WAVE_PARAMS = (32.0, 32.0, 32.0, 20.0, 1.5, 0.3)
# the reference's default world sampler settings (WorldOctree.cpp:49-55): g_scale
# 0.25, height 75, 13 perturb octaves, amp 0.87, freq 0.585, gain 0.488; seed;
# 3 value-noise octaves (FastNoiseSIMD's default fractal)
TERRAIN_2D_PARAMS = (0.25, 75.0, 13, 0.87, 0.585, 0.488, 1337, 3)


def sphere_wave_field():
    return Field.make(FIELD_SPHERE_WAVE, SPHERE_WAVE_PARAMS)


def terrain_field():
    return Field.make(FIELD_TERRAIN_FBM, TERRAIN_PARAMS)


def terrain2d_field(params=TERRAIN_2D_PARAMS):
    """The perturbed 2D heightmap: -(y g) - height n(x, z) (bmf_fields.h)."""
    return Field.make(FIELD_TERRAIN_2D, params)


def lod_update(n=4096, seed=2024, tiers=((32, 0.50), (64, 0.35), (128, 0.15))):
    """Returns (descriptors, array) for an n-chunk mixed-LOD update.

    array rows are (origin x, y, z, scale, dim, level) as float64.  Chunk
    resolution tiers follow the requested split; the LOD level (cell size
    2**level) is drawn per chunk; horizontal origins are normally spread around
    the camera in units of the chunk's own extent (coarser chunks reach
    further out) and the vertical origin is spread around the terrain band
    y ~ 64, so chunks range from empty to surface-rich.
    """
    rng = np.random.default_rng(seed)
    counts = [int(round(n * f)) for _, f in tiers]
    counts[0] += n - sum(counts)
    res = np.concatenate([np.full(c, r) for (r, _), c in zip(tiers, counts)])
    rng.shuffle(res)
    level = rng.choice(4, size=n, p=[0.4, 0.3, 0.2, 0.1])
    cam = np.array([WORLD / 2 + rng.uniform(-64, 64), 64.0, WORLD / 2 + rng.uniform(-64, 64)])
    rows = np.zeros((n, 6))
    for i in range(n):
        cell = float(2 ** level[i])
        ext = res[i] * cell
        cx = cam[0] + rng.normal(0.0, 3.0 * ext)
        cz = cam[2] + rng.normal(0.0, 3.0 * ext)
        cy = 64.0 + rng.normal(0.0, 1.0 * ext) - ext / 2
        org = np.floor(np.array([cx, cy, cz]) / ext) * ext
        org = np.clip(org, 0.0, WORLD - ext)
        rows[i] = (org[0], org[1], org[2], cell, res[i] + 1, level[i])
    descs = [ChunkDesc.make(r[:3], r[3], int(r[4]), int(r[5])) for r in rows]
    return descs, rows


def shard(rows, rank, world_size):
    """Chunks of one rank when an update is split across ranks (contiguous
    blocks balanced by sample count; chunks are independent, no exchange)."""
    w = rows[:, 4] ** 3
    cum = np.cumsum(w)
    total = cum[-1]
    lo = np.searchsorted(cum, total * rank / world_size, side="right")
    hi = np.searchsorted(cum, total * (rank + 1) / world_size, side="right")
    if rank == world_size - 1:
        hi = len(rows)
    return np.arange(lo, hi)


def fit_batch(n, dim=65, seed=0, device="cuda"):
    """Learnable density grids and targets for batched fitting: chunk i holds the
    sphere |p - c| - 20 (c = chunk centre) plus N(0, 0.1) noise on dim^3 samples;
    its target is a union of 1-4 spheres, radii U[6, 20], centres U[4, dim - 5]
    per axis.  Returns (density (n * dim^3,) float32, spheres (n, 4, 4) float32);
    unused sphere rows sit at 1e6 with radius 0."""
    import torch

    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    g = torch.arange(dim, dtype=torch.float32, device=device)
    c = (dim - 1) / 2.0
    r = ((g[:, None, None] - c) ** 2 + (g[None, :, None] - c) ** 2 + (g[None, None, :] - c) ** 2).sqrt() - 20.0
    dens = r.reshape(1, -1).repeat(n, 1)
    dens += 0.1 * torch.randn(dens.shape, generator=gen, device=device)
    rng = np.random.default_rng(seed)
    sph = np.zeros((n, 4, 4), np.float32)
    sph[:, :, :3] = 1e6
    for i in range(n):
        k = int(rng.integers(1, 5))
        sph[i, :k, :3] = rng.uniform(4.0, dim - 5.0, (k, 3))
        sph[i, :k, 3] = rng.uniform(6.0, 20.0, k)
    return dens.reshape(-1).contiguous(), torch.from_numpy(sph).to(device)
