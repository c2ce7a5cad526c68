"""Device-side descriptor generation (bmf_lod_generate) against the oracle's
restatement of the WorldOctree split policy: the same leaves, in the same
(depth-first stack) order, with bit-identical chunk frames; then the
generated queue drives a batched update."""
import numpy as np
import pytest

from binarymeshfitting_gb300 import _lib as L
from binarymeshfitting_gb300 import workloads
from binarymeshfitting_gb300.engine import Batch, Context
from oracle import cpu

pytestmark = pytest.mark.gpu

ROOT, SIZE = (-4096.0, -4096.0, -4096.0), 8192.0


@pytest.fixture(scope="module")
def ctx():
    c = Context(0)
    yield c
    c.close()


def as_rows(t):
    r = t.cpu().numpy()
    f = r[:, :4].copy().view(np.float32)
    return np.concatenate([f, r[:, 4:6].astype(np.float32)], axis=1)


@pytest.mark.parametrize("focus,sm,smod,lo,hi,dim,bp,iters", [
    ((10.0, 64.0, 20.0), 1.0, 0.0, 1, 7, 33, False, 0),
    ((1000.0, -300.0, 5.0), 1.5, 16.0, 2, 8, 65, True, 4),
    ((3.25, 70.5, -12.0), 2.0, 0.0, 1, 9, 129, False, 4)])
def test_lod_generate_matches_oracle(ctx, focus, sm, smod, lo, hi, dim, bp, iters):
    g = as_rows(ctx.lod_generate(ROOT, SIZE, focus, sm, smod, lo, hi, dim, boundary_processing=bp, iters=iters))
    o = cpu.lod_generate(ROOT, SIZE, focus, sm, smod, lo, hi, dim, boundary_processing=bp, iters=iters)
    assert len(g) == len(o) > 8
    assert np.array_equal(g.view(np.uint32), o.view(np.uint32))


def test_lod_generate_reports_overflow(ctx):
    with pytest.raises(L.BmfError):
        ctx.lod_generate(ROOT, SIZE, (10.0, 64.0, 20.0), 1.0, 0.0, 1, 9, 33, cap=64)


def test_generated_queue_drives_a_batch(ctx):
    rows = ctx.lod_generate((-512.0, -512.0, -512.0), 1024.0, (0.0, 64.0, 0.0), 1.0, 0.0, 1, 5, 33)
    descs = Context.descs_from_rows(rows)
    b = Batch(ctx, descs, workloads.terrain_field(), mode=L.MODE_R, iters=2, smooth_normals=True)
    b.allocate(2_000_000, 12_000_000, normals=True)
    nv, ni = b.run(use_graph=True)
    assert nv > 0 and ni > 0
    i = next(k for k in range(len(descs)) if b.chunk_mesh(k)["contains_mesh"])
    r = as_rows(rows[i:i + 1])[0]
    d = cpu.fill_field(L.FIELD_TERRAIN_FBM, list(workloads.TERRAIN_PARAMS), 33, r[:3], r[3])
    w, cm = cpu.label_grid(33, d)
    O = cpu.extract_r(33, d, cpu.cell_masks(33, w))
    assert np.array_equal(b.chunk_mesh(i)["idx"].cpu().numpy().view(np.uint32), O["idx"])
    b.close()
