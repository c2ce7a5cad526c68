"""The reference's call surface (Sampler / DMCChunk / MeshProcessor /
ChunkGenerator) driven exactly as ChunkGenerator::extract_chunk drives it
(BinaryMeshFitting/ChunkGenerator.cpp:98-124), checked against the oracle."""
import numpy as np
import pytest

from binarymeshfitting_gb300 import _lib as L
from binarymeshfitting_gb300 import reference_api as R
from binarymeshfitting_gb300 import workloads
from oracle import cpu

pytestmark = pytest.mark.gpu


def _oracle_chunk(origin, scale, dim, iters=0, normals=False):
    d = cpu.fill_field(L.FIELD_TERRAIN_FBM, list(workloads.TERRAIN_PARAMS), dim, origin, scale)
    w, cm = cpu.label_grid(dim, d)
    if not cm:
        return None
    O = cpu.extract_r(dim, d, cpu.cell_masks(dim, w))
    if iters:
        O["pos"], O["nrm"] = cpu.process(3, O["pos"], O["boundary"], O["valence"], O["idx"], iters, False, normals)
    return O


def test_dmcchunk_pipeline_and_mesh_processor(ctx):
    sampler = R.Sampler(workloads.terrain_field(), world_size=4096.0)
    chunk = R.DMCChunk(pos=(2000.0, 40.0, 1990.0), size=62.0, level=2, sampler=sampler, dim=32)
    chunk.label_grid(overlap=0.035 + 0.005 * 4)
    chunk.label_edges()
    chunk.polygonize()
    assert chunk.contains_mesh
    O = _oracle_chunk(chunk.overlap_pos, chunk.scale, 32)
    np.testing.assert_array_equal(chunk.vi.mesh_indexes.cpu().numpy().view(np.uint32), O["idx"])
    np.testing.assert_array_equal(chunk.vi.vertices.pos.cpu().numpy().view(np.uint32), O["pos"].view(np.uint32))
    mp = R.MeshProcessor(3, True, True)
    assert mp.init(chunk.vi.vertices, chunk.vi.mesh_indexes, sampler)
    mp.optimize_dual_grid(4, False)
    mp.optimize_primal_grid(False, False, False)
    mesh = mp.flush()
    O = _oracle_chunk(chunk.overlap_pos, chunk.scale, 32, iters=4, normals=True)
    np.testing.assert_array_equal(mesh.pos.cpu().numpy().view(np.uint32), O["pos"].view(np.uint32))
    v_out, i_out = [], []
    chunk.copy_verts_and_inds(v_out, i_out)
    chunk.copy_verts_and_inds(v_out, i_out)
    assert int(i_out[1].min()) == mesh.n_verts


def test_chunk_generator_process_queue_matches_per_chunk(ctx):
    props = R.WorldProperties(max_level=3, process_iters=2, boundary_processing=False, smooth_normals=True)
    gen = R.ChunkGenerator(props, R.Sampler(workloads.terrain_field()), dim=33)
    nodes = [R.WorldOctreeNode(pos=(2048.0 + 32 * i, 32.0, 2048.0), size=32.0, level=3) for i in range(3)]
    nodes += [R.WorldOctreeNode(pos=(1024.0, 0.0, 1024.0 + 64 * i), size=64.0, level=2) for i in range(3)]
    gen.process_queue(nodes)
    for n in nodes:
        delta, org = R.chunk_frame(n.pos, n.size, gen.overlap_for(n), 33)
        O = _oracle_chunk(org, delta, 33, iters=2, normals=True)
        if O is None:
            assert len(n.vi["pos"]) == 0
            continue
        assert n.vi["contains_mesh"]
        np.testing.assert_array_equal(n.vi["idx"].cpu().numpy().view(np.uint32), O["idx"])
        np.testing.assert_array_equal(n.vi["pos"].cpu().numpy().view(np.uint32), O["pos"].view(np.uint32))
    assert gen.overlap_for(nodes[0]) == 0.0  # max level, no boundary processing
    assert gen.overlap_for(nodes[3]) == pytest.approx(0.045)


def test_process_queue_reuses_its_plan(ctx):
    """A second queue of the same shape swaps its descriptors into the kept
    plan and replays the graph; its meshes match the oracle, and the first
    queue's meshes (copied out of the arena) are unchanged."""
    props = R.WorldProperties(max_level=3, process_iters=2, boundary_processing=False, smooth_normals=True)
    gen = R.ChunkGenerator(props, R.Sampler(workloads.terrain_field()), dim=33)
    q1 = [R.WorldOctreeNode(pos=(1000.0 + 64 * i, 16.0, 2000.0), size=64.0, level=2) for i in range(4)]
    q2 = [R.WorldOctreeNode(pos=(3000.0, 40.0 - 32 * i, 100.0 + 32 * i), size=32.0, level=3) for i in range(4)]
    gen.process_queue(q1)
    first = [n.vi["pos"].clone() for n in q1]
    gen.process_queue(q2)
    assert gen.plans_reused == 1
    for n, p in zip(q1, first):
        assert n.vi["pos"].equal(p)
    checked = 0
    for n in q2:
        delta, org = R.chunk_frame(n.pos, n.size, gen.overlap_for(n), 33)
        O = _oracle_chunk(org, delta, 33, iters=2, normals=True)
        if O is None:
            assert len(n.vi["pos"]) == 0
            continue
        np.testing.assert_array_equal(n.vi["idx"].cpu().numpy().view(np.uint32), O["idx"])
        np.testing.assert_array_equal(n.vi["pos"].cpu().numpy().view(np.uint32), O["pos"].view(np.uint32))
        checked += 1
    assert checked >= 2
    gen.close()
