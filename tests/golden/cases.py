"""Seeded input cases shared by the golden-fixture generator and the tests.

Densities are rebuilt from a recipe, never stored: bit-reproducible fields of
the oracle (ids of include/bmf_fields.h) or numpy PCG64 uniform noise.
"""
import numpy as np

SPHERE_WAVE = 1
TERRAIN_FBM = 2
TORUS_Z, SPHERE, CUBOID, PLANE_Y = 3, 4, 5, 6


def _sw(dim):
    c = dim / 2.0
    return dict(field=SPHERE_WAVE, params=[c, c, c, dim * 0.31, 1.5, 0.3], origin=[0, 0, 0], scale=1.0)


def _fbm(dim):
    return dict(field=TERRAIN_FBM, params=[dim * 0.55, dim * 0.3, 0.05, 2.0, 0.5, 5, 1337], origin=[0, 0, 0],
                scale=1.0)


CASES = []
for _dim in (32, 64, 128):
    CASES += [
        dict(name="sphere_wave_%d" % _dim, dim=_dim, kind="field", **_sw(_dim)),
        dict(name="terrain_fbm_%d" % _dim, dim=_dim, kind="field", **_fbm(_dim)),
        dict(name="torus_%d" % _dim, dim=_dim, kind="field", field=TORUS_Z, params=[_dim * 1.0],
             origin=[-_dim / 2 + 0.5, -_dim / 2 + 0.25, -_dim / 2 + 0.5], scale=1.0),
        dict(name="cuboid_%d" % _dim, dim=_dim, kind="field", field=CUBOID, params=[_dim * 1.0],
             origin=[-_dim / 2 + 0.3, -_dim / 2 + 0.3, -_dim / 2 + 0.3], scale=1.0),
        # integer plane: samples exactly 0.0 (outside, since only < 0 is inside) and mu = 0 crossings
        dict(name="plane_zero_%d" % _dim, dim=_dim, kind="field", field=PLANE_Y, params=[_dim * 1.0],
             origin=[0, -_dim / 2, 0], scale=1.0),
        dict(name="uniform_%d" % _dim, dim=_dim, kind="uniform", seed=11 + _dim, lo=-1.0, hi=1.0),
        dict(name="all_inside_%d" % _dim, dim=_dim, kind="constant", value=-1.0),
        dict(name="all_outside_%d" % _dim, dim=_dim, kind="constant", value=1.0),
    ]
# a sparse random field: mostly outside with scattered inside samples (many isolated cells)
CASES.append(dict(name="sparse_64", dim=64, kind="uniform", seed=5, lo=-0.05, hi=1.0))

PROCESS_CASES = []
for _N in (3, 4):
    for _iters in (1, 4, 8):
        for _normals in (False, True):
            for _boundary in (False, True):
                PROCESS_CASES.append(dict(case="sphere_wave_32", N=_N, iters=_iters, normals=_normals,
                                          boundary=_boundary))
PROCESS_CASES.append(dict(case="terrain_fbm_64", N=3, iters=4, normals=True, boundary=False))
PROCESS_CASES.append(dict(case="terrain_fbm_64", N=4, iters=4, normals=True, boundary=False))


def make_density(case):
    """Rebuilds a case's float32 density (dim^3, z fastest)."""
    dim = case["dim"]
    if case["kind"] == "uniform":
        return np.random.default_rng(case["seed"]).uniform(case["lo"], case["hi"], dim ** 3).astype(np.float32)
    if case["kind"] == "constant":
        return np.full(dim ** 3, case["value"], np.float32)
    from oracle import cpu
    return cpu.fill_field(case["field"], case["params"], dim, case["origin"], case["scale"])
