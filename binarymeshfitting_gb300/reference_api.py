"""The reference's chunk-extraction call surface, backed by libbmf_gb300.so.

Same class and method names and the same argument meaning as the reference's
Sampler (BinaryMeshFitting/Sampler.hpp:24-34), DMCChunk (DMCChunk.hpp:21-85),
MeshProcessor<N> (MeshProcessor.hpp:55-84) and ChunkGenerator
(ChunkGenerator.hpp:15-57), so a caller of the reference's per-chunk path can
switch by changing imports.  Every stage runs on the GPU through the C ABI;
buffers are device tensors (VerticesIndicesBlock's SmartContainers become
tensors).  Errors surface as BmfError (status codes) where the reference
asserted or silently ignored a failed allocation.
"""
from dataclasses import dataclass, field as dc_field
from typing import List, Optional

import numpy as np
import torch

from . import _lib as L
from .engine import Batch, ChunkMesh, Context

RESOLUTION = 32  # DMCChunk.cpp:34 (samples per axis of a world chunk)

_ctx: Optional[Context] = None


def context() -> Context:
    """The process-wide context (one per host thread in the C ABI's terms)."""
    global _ctx
    if _ctx is None:
        _ctx = Context(torch.cuda.current_device() if torch.cuda.is_available() else 0)
    return _ctx


def chunk_frame(pos, size, overlap, dim):
    """Sample spacing and world origin of a chunk, in single precision and in
    the reference's operation order (DMCChunk.cpp:94-97):
    delta = size * (1 + overlap * 2) / (dim - 1);  overlap_pos = pos - size * overlap."""
    f = np.float32
    s, o = f(size), f(overlap)
    delta = f(f(s * f(f(1.0) + f(o * f(2.0)))) / f(dim - 1))
    shift = f(s * o)
    return float(delta), tuple(float(f(f(p) - shift)) for p in pos)


class Sampler:
    """Density source (Sampler.hpp:24-34): world_size plus the field that the
    reference's block function would fill."""

    def __init__(self, field: L.Field, world_size: float = 256.0):
        self.field = field
        self.world_size = world_size

    def block(self, world_size, p, size, scale, out=None):
        """Sampler::block: fills size^3 samples at p + (x,y,z)*scale (ImplicitSampler.hpp:14-36)."""
        assert size[0] == size[1] == size[2], "chunks are cubic"
        desc = L.ChunkDesc.make(p, scale, size[0])
        return context().sample_block(desc, self.field, out)


@dataclass
class VerticesIndicesBlock:
    """ChunkBlocks.hpp:161-179 as device tensors."""
    vertices: Optional[ChunkMesh] = None
    mesh_indexes: Optional[torch.Tensor] = None


class DMCChunk:
    """DMCChunk's main pipeline (DMCChunk.hpp:66-73) for one chunk."""

    def __init__(self, pos=(0.0, 0.0, 0.0), size=1.0, level=0, sampler: Sampler = None, parent_code=0,
                 dim=RESOLUTION):
        self.init(pos, size, level, sampler, parent_code, dim)

    def init(self, pos, size, level, sampler, parent_code=0, dim=RESOLUTION):
        self.pos = tuple(float(v) for v in pos)
        self.size = float(size)
        self.level = level
        self.sampler = sampler
        self.parent_code = parent_code
        self.dim = dim
        self.contains_mesh = False
        self.vi: Optional[VerticesIndicesBlock] = None
        self.density = None
        self.words = None

    def label_grid(self, overlap=0.0, properties=None):
        """DMCChunk.cpp:79-166: samples the chunk and builds its binary grid."""
        d = self.dim
        self.delta, self.overlap_pos = chunk_frame(self.pos, self.size, overlap, d)
        self.scale = self.delta
        desc = L.ChunkDesc.make(self.overlap_pos, self.delta, d, self.level)
        self.density, self.words, self.contains_mesh = context().sample_label(desc, self.sampler.field)

    def label_edges(self):
        """DMCChunk.cpp:168-508.  The masks, the surface-cell enumeration and the
        iso-vertices are computed inside polygonize's kernels straight from the
        occupancy words, so this stage has nothing left to store."""
        return None

    def polygonize(self, mode=L.MODE_R, placement=L.PLACE_CENTER):
        """DMCChunk.cpp:514-576 (Mode R); Mode Q gives the DMC quads instead."""
        if not self.contains_mesh:
            return
        m = context().polygonize(self.dim, self.density, self.words, mode=mode, placement=placement, normals=True)
        self.vi = VerticesIndicesBlock(vertices=m, mesh_indexes=m.idx)

    def copy_verts_and_inds(self, v_out: list, i_out: list):
        """DMCChunk.cpp:578-591: appends this chunk's vertices and its indices
        offset by the vertex count already in v_out (lists of tensors)."""
        if not self.contains_mesh or self.vi is None:
            return
        offset = sum(v.shape[0] for v in v_out)
        self.mesh_offset = offset
        v_out.append(self.vi.vertices.pos)
        i_out.append(self.vi.mesh_indexes + offset)


class MeshProcessor:
    """MeshProcessor<N> (MeshProcessor.hpp:55-84).  The GPU runs the dual and
    primal sweeps as one sequence, so the calls are recorded and executed at
    flush(); the supported sequence is the one ChunkGenerator::extract_chunk
    makes (ChunkGenerator.cpp:114-121): init, optimize_dual_grid(iters,
    boundary), optimize_primal_grid(False, False, boundary), flush."""

    def __init__(self, N=3, simple_quality=True, smooth_normals=False):
        assert N in (3, 4)
        self.N = N
        self.simple_quality = simple_quality
        self.smooth_normals = smooth_normals
        self.mesh = None
        self.iters = None
        self.boundary = False

    def init(self, vertices: ChunkMesh, inds=None, sampler=None):
        """MeshProcessor.cpp:26-55: returns True, or False when the mesh has no
        adjacency (zero valence everywhere)."""
        if vertices is None or vertices.n_verts == 0 or vertices.n_idx < self.N:
            return True
        if vertices.prim_size != self.N:
            raise ValueError("mesh has %d-gons, processor expects %d" % (vertices.prim_size, self.N))
        self.mesh = vertices
        if vertices.nrm is None:
            vertices.nrm = torch.zeros_like(vertices.pos)
        return int(vertices.valence.sum().item()) > 0

    def optimize_dual_grid(self, iterations, process_boundary=True):
        self.iters = iterations
        self.boundary = process_boundary

    def optimize_primal_grid(self, qef=False, set_colors=False, process_boundary=True):
        if self.iters is None or qef or set_colors or process_boundary != self.boundary:
            raise NotImplementedError("only the ChunkGenerator::extract_chunk call sequence is supported")

    def flush(self):
        if self.mesh is not None and self.iters:
            context().process(self.mesh, self.iters, self.boundary, self.smooth_normals)
        return self.mesh


@dataclass
class WorldProperties:
    """The extraction knobs of WorldProperties (WorldOctree.cpp:20-33)."""
    max_level: int = 7
    process_iters: int = 0
    overlap: float = 0.035
    boundary_processing: bool = False
    smooth_normals: bool = False


@dataclass
class WorldOctreeNode:
    """The fields of a queued node that extraction reads."""
    pos: tuple
    size: float
    level: int
    chunk: Optional[DMCChunk] = None
    vi: Optional[dict] = None


class ChunkGenerator:
    """ChunkGenerator::process_queue (ChunkGenerator.cpp:27-147): the whole
    queue goes through one batched, graph-captured update.  The plan and its
    output arena are kept while queues keep their shape (same chunk count and
    resolution): the next queue's descriptors are swapped in with
    bmf_batch_set_descs and the captured graph replays."""

    def __init__(self, properties: WorldProperties, sampler: Sampler, dim=RESOLUTION, mode=L.MODE_R,
                 placement=L.PLACE_CENTER):
        self.properties = properties
        self.sampler = sampler
        self.dim = dim
        self.mode = mode
        self.placement = placement
        self._plan: Optional[Batch] = None
        self.plans_reused = 0

    def overlap_for(self, node: WorldOctreeNode):
        """ChunkGenerator.cpp:98."""
        p = self.properties
        if node.level == p.max_level and (not p.boundary_processing or p.process_iters == 0):
            return 0.0
        return p.overlap + 0.005 * float(p.process_iters)

    def _descs(self, batch):
        out = []
        for n in batch:
            delta, org = chunk_frame(n.pos, n.size, self.overlap_for(n), self.dim)
            out.append(L.ChunkDesc.make(org, delta, self.dim, n.level))
        return out

    def process_queue(self, batch: List[WorldOctreeNode]):
        p = self.properties
        if not batch:
            return batch
        descs = self._descs(batch)
        ctx = context()
        b = self._plan
        if b is not None and b.n == len(batch):
            b.set_descs(descs)
            self.plans_reused += 1
        else:
            self.close()
            b = Batch(ctx, descs, self.sampler.field, mode=self.mode, placement=self.placement,
                      iters=p.process_iters, process_boundary=p.boundary_processing, smooth_normals=p.smooth_normals)
            self._plan = b
            vcap, icap = max(4096, len(batch) * self.dim ** 2 * 4), max(16384, len(batch) * self.dim ** 2 * 24)
            b.allocate(vcap, icap, normals=p.smooth_normals)
        for _ in range(3):
            try:
                b.run(use_graph=True, sync=True)
                break
            except L.BmfError as e:
                if e.status != L.ERR_CAPACITY:
                    raise
                b.allocate(int(b.out.n_verts) + 1024, int(b.out.n_idx) + 1024, normals=p.smooth_normals)
        for i, n in enumerate(batch):
            # copies: the arena is overwritten by the next queue
            n.vi = {k: (v.clone() if isinstance(v, torch.Tensor) else v) for k, v in b.chunk_mesh(i).items()}
        return batch

    def close(self):
        if self._plan is not None:
            self._plan.close()
            self._plan = None
