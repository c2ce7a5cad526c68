"""Every Marching-Cubes / DMC corner case, and small grids of random signs,
through the GPU extraction against the oracle, bit for bit.

The reference has no tests (its correctness rests on runtime asserts), so the
case tables are exercised exhaustively here: a 2^3-sample grid holds one cell,
and its corner signs are set to each of the 256 masks (bit 4 dx + 2 dy + dz =
corner (dx, dy, dz) inside, DMCChunk.cpp:220-252), with a different magnitude
per corner so every crossing lands at its own place.  Grids of 3^3 and 4^3
samples with seeded random signs add the cases' neighbours: shared edges,
far-face cells and boundary flags.  Mode R (triangles, DMCChunk.cpp:514-576)
and Mode Q with each placement (Tables.hpp:76-354).
"""
import numpy as np
import pytest

from binarymeshfitting_gb300 import _lib as L
from oracle import cpu
from tests.test_gpu_parity import assert_float_exact, dev, np_u32

pytestmark = pytest.mark.gpu


def case_grid(mask):
    d = np.empty((2, 2, 2), np.float32)
    for k in range(8):
        dx, dy, dz = (k >> 2) & 1, (k >> 1) & 1, k & 1
        d[dx, dy, dz] = -(0.5 + 0.37 * k) if (mask >> k) & 1 else (0.25 + 0.19 * k)
    return d.reshape(-1)


def check_grid(ctx, dim, d):
    words_t, cm = ctx.label_grid(dim, dev(d))
    w, ocm = cpu.label_grid(dim, d)
    np.testing.assert_array_equal(np_u32(words_t), np.asarray(w).view(np.uint32))
    assert cm == bool(ocm)
    if not cm:
        return 0
    m = ctx.polygonize(dim, dev(d), words_t, mode=L.MODE_R)
    O = cpu.extract_r(dim, d, cpu.cell_masks(dim, w))
    np.testing.assert_array_equal(np_u32(m.idx), O["idx"])
    np.testing.assert_array_equal(m.boundary.cpu().numpy(), O["boundary"])
    np.testing.assert_array_equal(m.valence.cpu().numpy(), O["valence"])
    assert_float_exact(m.pos.cpu().numpy(), O["pos"], "mode R positions")
    for placement in (L.PLACE_CENTER, L.PLACE_MASSPOINT, L.PLACE_QEF):
        q = ctx.polygonize(dim, dev(d), words_t, mode=L.MODE_Q, placement=placement)
        Q = cpu.extract_q(dim, d, np.asarray(w).view(np.uint32), placement)
        np.testing.assert_array_equal(np_u32(q.idx), Q["idx"])
        np.testing.assert_array_equal(q.boundary.cpu().numpy(), Q["boundary"])
        np.testing.assert_array_equal(q.valence.cpu().numpy(), Q["valence"])
        assert_float_exact(q.pos.cpu().numpy(), Q["pos"], "mode Q positions (placement %d)" % placement)
    return len(O["idx"]) // 3


def test_all_256_cell_cases(ctx):
    tris = 0
    for mask in range(256):
        tris += check_grid(ctx, 2, case_grid(mask))
    assert tris > 400  # the table's 254 mixed cases hold several triangles each


@pytest.mark.parametrize("dim", [3, 4])
def test_random_sign_grids(ctx, dim):
    rng = np.random.default_rng(40 + dim)
    meshes = 0
    for _ in range(120):
        d = rng.uniform(0.05, 1.0, dim ** 3).astype(np.float32)
        d *= np.where(rng.random(dim ** 3) < rng.uniform(0.2, 0.8), -1.0, 1.0).astype(np.float32)
        meshes += check_grid(ctx, dim, d) > 0
    assert meshes > 100
