"""Draw layout (GLChunk::format_data, GLChunk.cpp:278-335) on the GPU against
the oracle's restatement, on the GPU's own meshes: bit-exact positions,
normals and colours, per vertex and unwound quads, flat and smooth normals,
for one chunk and for a whole batch arena (chunk-local indices resolved)."""
import numpy as np
import pytest
import torch

from binarymeshfitting_gb300 import _lib as L
from binarymeshfitting_gb300 import workloads
from binarymeshfitting_gb300.engine import Batch, Context
from oracle import cpu

pytestmark = pytest.mark.gpu


def bits(a):
    a = np.ascontiguousarray(np.asarray(a, np.float32))
    a = np.where(np.isnan(a), np.float32("nan"), a)
    return a.view(np.uint32) & np.where(np.isnan(a), np.uint32(0x7FC00000), np.uint32(0xFFFFFFFF))


@pytest.fixture(scope="module")
def ctx():
    c = Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("unwind,smooth", [(0, 0), (1, 0), (1, 1)])
def test_format_single_chunk(ctx, unwind, smooth):
    desc = L.ChunkDesc.make((0.0, 0.0, 0.0), 1.0, 65)
    m = ctx.extract_chunk(desc, workloads.sphere_wave_field(), mode=L.MODE_Q, placement=L.PLACE_MASSPOINT, iters=4,
                          smooth_normals=True)
    p, n, c = ctx.format(m, unwind=bool(unwind), smooth_normals=bool(smooth))
    op, on, oc = cpu.format_data(m.pos.cpu().numpy(), m.nrm.cpu().numpy(), m.idx.cpu().numpy().view(np.uint32),
                                 unwind, smooth)
    assert p.shape[0] == (m.n_idx if unwind else m.n_verts) > 0
    for g, o in ((p, op), (n, on), (c, oc)):
        assert np.array_equal(bits(g.cpu().numpy()), bits(o))


def test_format_rejects_unwinding_triangles(ctx):
    desc = L.ChunkDesc.make((0.0, 0.0, 0.0), 1.0, 33)
    m = ctx.extract_chunk(desc, workloads.sphere_wave_field(), mode=L.MODE_R)
    with pytest.raises(L.BmfError):
        ctx.format(m, unwind=True)
    p, n, c = ctx.format(m)  # per-vertex layout works for triangles
    assert torch.equal(p, m.pos) and bool((c == 1.0).all()) and bool((n == 0.0).all())


@pytest.mark.parametrize("smooth", [0, 1])
def test_batch_format_matches_per_chunk(ctx, smooth):
    descs, rows = workloads.lod_update(n=24, seed=5)
    for d in descs:
        d.dim = min(d.dim, 65)
    b = Batch(ctx, descs, workloads.terrain_field(), mode=L.MODE_Q, placement=L.PLACE_MASSPOINT, iters=2,
              smooth_normals=True)
    b.allocate(400000, 1600000, normals=True)
    nv, ni = b.run(use_graph=True)
    p, n, c = b.format(unwind=True, smooth_normals=bool(smooth))
    assert p.shape[0] == ni
    got = [bits(t.cpu().numpy()) for t in (p, n, c)]
    off = 0
    for i in range(len(descs)):
        ch = b.chunk_mesh(i)
        if ch["idx"].numel() == 0:
            continue
        op, on, oc = cpu.format_data(ch["pos"].cpu().numpy(), ch["nrm"].cpu().numpy(),
                                     ch["idx"].cpu().numpy().view(np.uint32), 1, smooth)
        k = len(op)
        for g, o in zip(got, (op, on, oc)):
            assert np.array_equal(g[off:off + k], bits(o)), i
        off += k
    assert off == ni
    b.close()
