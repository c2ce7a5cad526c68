"""Parity on the benchmarked configuration: a batched update of 2048+ chunks
(the size at which the batch runs its sweeps chunk by chunk) that contains
full-size 129^3 chunks at LOD cell sizes 4 and 8, compared chunk by chunk with
the oracle; the 129^3 terrain chunk with hermite-QEF placement, 4 sweeps and
smoothed normals; and overlapping chunks from the LOD generator with
boundary processing on.

Chunk-by-chunk comparison uses digests: the oracle runs the whole CPU path per
chunk (ChunkGenerator::extract_chunk order, ChunkGenerator.cpp:80-147) and
reports a digest of each chunk's indices, positions, boundary flags and
normals; the same digest is taken of each chunk's slice of the GPU arena.  A
mismatching chunk is re-run through the oracle for a readable diff.
"""
import numpy as np
import pytest

from binarymeshfitting_gb300 import _lib as L
from binarymeshfitting_gb300 import workloads
from binarymeshfitting_gb300.engine import Batch
from oracle import cpu
from tests.test_gpu_parity import assert_float_exact, np_u32

pytestmark = pytest.mark.gpu

TERRAIN = list(workloads.TERRAIN_PARAMS)


def run_sized(b, normals, vcap=2_000_000, icap=12_000_000):
    """Allocates the arena, growing it once from the reported needed counts."""
    for _ in range(3):
        b.allocate(vcap, icap, normals=normals)
        try:
            return b.run(use_graph=False, sync=True)
        except L.BmfError as e:
            if e.status != L.ERR_CAPACITY:
                raise
            vcap, icap = int(b.out.n_verts) + 1024, int(b.out.n_idx) + 1024
    raise AssertionError("arena sizing did not converge")


def arena_digests(b, normals):
    """Per chunk: (contains_mesh, status, vertices, indices) and the oracle's
    digests of the chunk's arena slice."""
    info = b.bufs["info"].cpu().numpy()
    pos = b.bufs["pos"].cpu().numpy()
    idx = b.bufs["idx"].cpu().numpy().view(np.uint32)
    bnd = b.bufs["boundary"].cpu().numpy()
    nrm = b.bufs["nrm"].cpu().numpy() if normals else None
    dig = np.zeros((len(info), 4), np.uint64)
    for i, (vo, vc, io, ic, _, _) in enumerate(info):
        dig[i] = cpu.chunk_digests(pos[vo:vo + vc], idx[io:io + ic], bnd[vo:vo + vc],
                                   nrm[vo:vo + vc] if nrm is not None else None)
    return info, dig


def oracle_chunk(r, mode, placement, iters, process_boundary, normals):
    dim = int(r[4])
    d = cpu.fill_field(L.FIELD_TERRAIN_FBM, TERRAIN, dim, r[:3], r[3])
    w, cm = cpu.label_grid(dim, d)
    if mode == L.MODE_R:
        O, N = cpu.extract_r(dim, d, cpu.cell_masks(dim, w)), 3
    else:
        O, N = cpu.extract_q(dim, d, w, placement), 4
    p, n = O["pos"], np.zeros_like(O["pos"])
    if iters:
        p, n = cpu.process(N, O["pos"], O["boundary"], O["valence"], O["idx"], iters, process_boundary, normals)
    return O, p, n


def compare_update(b, rows, mode, placement, iters, process_boundary, normals, field=L.FIELD_TERRAIN_FBM,
                   params=TERRAIN):
    """Every chunk of the update against the oracle; returns the number of
    chunks with a mesh."""
    info, got = arena_digests(b, normals)
    counts, want = cpu.extract_batch_digest(rows[:, :5].astype(np.float32), field, list(params), mode,
                                            placement, iters, process_boundary, normals)
    assert (info[:, 5] == 0).all(), "a chunk reported a capacity overflow"
    np.testing.assert_array_equal(info[:, 4], counts[:, 0], "contains_mesh")
    np.testing.assert_array_equal(info[:, 1], counts[:, 1], "vertex counts")
    np.testing.assert_array_equal(info[:, 3], counts[:, 2], "index counts")
    bad = np.flatnonzero((got != want).any(axis=1))
    for i in (bad[:3] if field == L.FIELD_TERRAIN_FBM else []):  # readable diff of the first mismatching chunks
        O, p, n = oracle_chunk(rows[i], mode, placement, iters, process_boundary, normals)
        m = b.chunk_mesh(int(i))
        np.testing.assert_array_equal(np_u32(m["idx"]), O["idx"], "chunk %d indices" % i)
        np.testing.assert_array_equal(m["boundary"].cpu().numpy(), O["boundary"], "chunk %d boundary" % i)
        assert_float_exact(m["pos"].cpu().numpy(), p, "chunk %d positions" % i)
        if normals:
            assert_float_exact(m["nrm"].cpu().numpy(), n, "chunk %d normals" % i)
    assert len(bad) == 0, "%d chunks differ from the oracle: %s" % (len(bad), bad[:16].tolist())
    return int((counts[:, 1] > 0).sum())


def mixed_update(n=2100, seed=11):
    """n chunks of the update's layout, most shrunk to 17^3 samples so the
    oracle stays quick, plus full-size chunks: 129^3 at cell sizes 4 and 8 on
    the terrain band (where the persistent fill's line items, the busy-word
    emit and the 1024-thread chunk sweeps see 128^3-cell chunks), and 65^3 /
    33^3 chunks at cell sizes 1 and 2."""
    descs, rows = workloads.lod_update(n=n, seed=seed)
    full = [((1024.0, -64.0, 2048.0), 4.0, 129, 2), ((2560.0, 0.0, 512.0), 8.0, 129, 3),
            ((1536.0, -256.0, 1536.0), 8.0, 129, 3), ((3000.0, 32.0, 100.0), 4.0, 129, 2),
            ((2048.0, -96.0, 2048.0), 4.0, 129, 2), ((700.0, 0.0, 3300.0), 8.0, 129, 3),
            ((2048.0, 0.0, 2112.0), 2.0, 65, 1), ((1900.0, 32.0, 2000.0), 1.0, 65, 0),
            ((2050.0, 40.0, 2050.0), 1.0, 33, 0), ((2100.0, 0.0, 1990.0), 2.0, 33, 1)]
    stride = n // len(full)
    slots = set(range(0, n, stride)[:len(full)])
    k = 0
    for i in range(n):
        if i in slots:
            org, scale, dim, level = full[k]
            k += 1
            rows[i] = (*org, scale, dim, level)
        else:
            rows[i, 4] = 17
        descs[i] = L.ChunkDesc.make(rows[i, :3], rows[i, 3], int(rows[i, 4]), int(rows[i, 5]))
    return descs, rows


@pytest.mark.parametrize("mode,placement", [(L.MODE_R, L.PLACE_CENTER), (L.MODE_Q, L.PLACE_MASSPOINT)])
def test_update_with_full_size_chunks_matches_oracle(ctx, mode, placement):
    descs, rows = mixed_update()
    assert len(descs) >= 2048 and (rows[:, 4] == 129).sum() == 6
    b = Batch(ctx, descs, workloads.terrain_field(), mode=mode, placement=placement, iters=4, smooth_normals=True)
    assert b.tuning()["fill_mode"] == 2  # the persistent line-item queue
    nv, ni = run_sized(b, True)
    for _ in range(2):  # graph replays give the same arena
        assert b.run(use_graph=True) == (nv, ni)
    with_mesh = compare_update(b, rows, mode, placement, 4, False, True)
    big = [i for i in range(len(rows)) if rows[i, 4] == 129]
    assert all(b.chunk_mesh(i)["pos"].shape[0] > 1000 for i in big), "the 129^3 chunks must hold surface"
    assert with_mesh >= 10
    b.close()


def test_update_arena_equals_per_chunk_extraction(ctx):
    """The batched update and the plain per-chunk drop-in give the same bytes
    for the full-size chunks of the update."""
    descs, rows = mixed_update()
    b = Batch(ctx, descs, workloads.terrain_field(), mode=L.MODE_R, iters=4, smooth_normals=True)
    run_sized(b, True)
    b.run(use_graph=True)
    for i in [i for i in range(len(rows)) if rows[i, 4] >= 65]:
        m = ctx.extract_chunk(descs[i], workloads.terrain_field(), mode=L.MODE_R, iters=4, smooth_normals=True)
        g = b.chunk_mesh(i)
        assert np.array_equal(np_u32(m.idx), np_u32(g["idx"]))
        assert np.array_equal(m.pos.cpu().numpy().view(np.uint32), g["pos"].cpu().numpy().view(np.uint32))
        assert np.array_equal(m.nrm.cpu().numpy().view(np.uint32), g["nrm"].cpu().numpy().view(np.uint32))
    b.close()


def test_terrain_129_qef_smoothing_normals(ctx):
    """The 128^3-cell terrain chunk with the hermite-QEF placement variant
    (central-difference grid gradients), 4 dual/primal sweeps and smoothed
    normals, through bmf_extract_chunk."""
    desc = L.ChunkDesc.make((0, 0, 0), 1.0, 129)
    m = ctx.extract_chunk(desc, workloads.terrain_field(), mode=L.MODE_Q, placement=L.PLACE_QEF, iters=4,
                          smooth_normals=True)
    d = cpu.fill_field(L.FIELD_TERRAIN_FBM, TERRAIN, 129)
    w, _ = cpu.label_grid(129, d)
    O = cpu.extract_q(129, d, w, L.PLACE_QEF)
    op, on = cpu.process(4, O["pos"], O["boundary"], O["valence"], O["idx"], 4, False, True)
    assert m.n_verts == len(op) > 10000
    np.testing.assert_array_equal(np_u32(m.idx), O["idx"])
    np.testing.assert_array_equal(m.boundary.cpu().numpy(), O["boundary"])
    assert_float_exact(m.pos.cpu().numpy(), op, "positions")
    assert_float_exact(m.nrm.cpu().numpy(), on, "normals")


@pytest.mark.parametrize("mode,placement", [(L.MODE_R, L.PLACE_CENTER), (L.MODE_Q, L.PLACE_QEF)])
def test_overlapping_chunks_with_boundary_processing(ctx, mode, placement):
    """WorldOctree leaves framed with ChunkGenerator.cpp:98's overlap
    (boundary_processing on, 4 iterations: every chunk overlaps its
    neighbours by 0.035 + 0.005 * 4 of its size), extracted in one batch with
    MeshProcessor's process_boundary (MeshProcessor.cpp:247) so boundary
    vertices move too; every chunk matches the oracle."""
    rows_t = ctx.lod_generate((-512.0, -512.0, -512.0), 1024.0, (0.0, 64.0, 0.0), 1.0, 0.0, 2, 5, 33,
                              boundary_processing=True, iters=4)
    descs = ctx.descs_from_rows(rows_t)
    r = rows_t.cpu().numpy()
    rows = np.concatenate([r[:, :4].copy().view(np.float32), r[:, 4:6].astype(np.float32)], axis=1)
    o = cpu.lod_generate((-512.0, -512.0, -512.0), 1024.0, (0.0, 64.0, 0.0), 1.0, 0.0, 2, 5, 33,
                         boundary_processing=True, iters=4)
    assert np.array_equal(rows.view(np.uint32), o.view(np.uint32))
    # frames overlap: a chunk's sample extent is (1 + 2 * 0.055) times its node
    node = rows[:, 3] * 32 / (1 + 2 * 0.055)
    assert np.allclose(node, 2.0 ** np.round(np.log2(node)), rtol=1e-5)
    b = Batch(ctx, descs, workloads.terrain_field(), mode=mode, placement=placement, iters=4,
              process_boundary=True, smooth_normals=True)
    run_sized(b, True)
    b.run(use_graph=True)
    assert compare_update(b, rows, mode, placement, 4, True, True) >= 4
    # boundary vertices moved: process_boundary on differs from off
    nb = Batch(ctx, descs, workloads.terrain_field(), mode=mode, placement=placement, iters=4,
               process_boundary=False, smooth_normals=True)
    run_sized(nb, True)
    i = next(k for k in range(len(descs)) if b.chunk_mesh(k)["boundary"].sum().item() > 0)
    on, off = b.chunk_mesh(i), nb.chunk_mesh(i)
    moved = (on["pos"] != off["pos"]).any(dim=1)
    assert moved[on["boundary"].bool()].any()
    b.close()
    nb.close()


@pytest.mark.parametrize("mode,placement", [(L.MODE_R, L.PLACE_CENTER), (L.MODE_Q, L.PLACE_MASSPOINT)])
def test_terrain2d_update_matches_oracle(ctx, mode, placement):
    """The reference's default world sampler shape (BMF_FIELD_TERRAIN_2D, the
    perturbed heightmap of NoiseSampler.cpp:148-194 with WorldOctree.cpp:49-55's
    settings) through a batched update: the x-plane fill evaluates each (x, z)
    column's height once; every chunk matches the oracle."""
    descs, rows = workloads.lod_update(n=96, seed=21)
    for dsc, r in zip(descs, rows):
        dsc.dim = min(dsc.dim, 65)
        r[4] = dsc.dim
        dsc.origin[1] = float(r[1]) - 128.0  # the band of this field: |y| <= 300
        r[1] = dsc.origin[1]
    field = workloads.terrain2d_field()
    b = Batch(ctx, descs, field, mode=mode, placement=placement, iters=4, smooth_normals=True)
    run_sized(b, True)
    b.run(use_graph=True)
    assert compare_update(b, rows, mode, placement, 4, False, True, L.FIELD_TERRAIN_2D,
                          workloads.TERRAIN_2D_PARAMS) >= 20
    b.close()


def test_terrain2d_column_fill_matches_full_fill(ctx):
    """The 2D heightmap's band form -- the column fill: occupancy words and
    (x, z) column heights only, densities at the ends of crossings computed
    from the stored heights by the fix-up -- gives an arena bit-identical to
    the full fill's, with and without graph replay."""
    import torch
    descs, rows = workloads.lod_update(n=160, seed=23)
    for dsc, r in zip(descs, rows):
        dsc.dim = min(dsc.dim, 65)
        dsc.origin[1] = float(r[1]) - 128.0
    b = Batch(ctx, descs, workloads.terrain2d_field(), mode=L.MODE_R, iters=4, smooth_normals=True)
    assert b.tuning()["fill_band"] == 1
    run_sized(b, True)
    bufs = b.bufs
    b.set_tuning(fill_band=0)
    nv, ni = b.run(use_graph=False)
    assert nv > 0
    ref = {k: bufs[k][:n].clone() for k, n in (("pos", nv), ("nrm", nv), ("idx", ni), ("boundary", nv))}
    ref["info"] = bufs["info"].clone()
    b.set_tuning(fill_band=1)
    for use_graph in (False, True):
        assert b.run(use_graph=use_graph) == (nv, ni)
        for k, r in ref.items():
            g = bufs[k][:r.shape[0]]
            if r.is_floating_point():
                r, g = r.view(torch.int32), g.view(torch.int32)
            assert torch.equal(r, g), (k, use_graph)
    b.close()
