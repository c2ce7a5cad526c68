// Pinning harness around the reference's OWN chunk-extraction code.
//
// Test infrastructure only.  This file is compiled together with the
// reference's unmodified BinaryMeshFitting/DMCChunk.cpp, MeshProcessor.cpp and
// ImplicitSampler.cpp (plus qef_simd.h through PCH.h) against the compat shim
// in oracle/shim/, by oracle/Makefile, into oracle/_ref/libbmf_ref.so.  It is
// only buildable where the reference sources are present, and it is used to
// (1) prove the C restatement in oracle/bmf_oracle.c bit-identical to the
// reference at dim = 32/64/128 and (2) generate the golden fixtures under
// tests/golden/.  The product never links or calls it.
//
// The sequence mirrors ChunkGenerator::extract_chunk
// (BinaryMeshFitting/ChunkGenerator.cpp:80-147):
//   label_grid -> label_edges -> polygonize -> [MeshProcessor<3> init ->
//   optimize_dual_grid(iters, boundary) -> optimize_primal_grid(false, false,
//   boundary) -> flush].
#include "PCH.h"
#include "DMCChunk.hpp"
#include "MeshProcessor.hpp"
#include "ImplicitSampler.hpp"
#include "NoiseSampler.hpp"

#include <vector>

// DMCNode is defined in WorldOctreeNode.cpp, which drags in the GL upload path;
// these two constructors follow WorldOctreeNode.cpp:165-181 field by field.
DMCNode::DMCNode() : OctreeNode() {
  world_node_flag = false;
  leaf_flag = true;
  sample = 0.0f;
}
DMCNode::DMCNode(DMCChunk* _chunk, float _size, glm::vec3 _pos, glm::ivec3 _xyz, uint8_t _level,
                 uint32_t _int_size, float _sample)
    : OctreeNode(0, 0, _size, _pos, _level) {
  world_node_flag = false;
  leaf_flag = true;
  root = _chunk;
  xyz = _xyz;
  i_size = _int_size;
  sample = _sample;
}

namespace {

const float dummy_value(const float, const glm::vec3&) { return 0.0f; }

struct RefRun {
  int dim = 0;
  int contains_mesh = 0;
  std::vector<uint32_t> words;
  std::vector<uint64_t> masks;
  std::vector<uint16_t> cell_mask;
  std::vector<uint32_t> cell_lin;
  std::vector<uint32_t> cell_vidx;  // per cell: vertex id of edges x,y,z or 0xFFFFFFFF
  std::vector<uint32_t> inds;
  std::vector<float> vpos, vnorm, vcolor;
  std::vector<uint8_t> vboundary, vvalence;
  std::vector<uint32_t> idx;
};

template <int N>
void run_processor(SmartContainer<DualVertex>& verts, SmartContainer<uint32_t>& inds, int iters,
                   bool boundary, bool smooth_normals) {
  Sampler sampler;
  Processing::MeshProcessor<N> mp(true, smooth_normals);
  mp.init(verts, inds, sampler);
  mp.optimize_dual_grid(iters, boundary);
  mp.optimize_primal_grid(false, false, boundary);
  verts.count = 0;
  inds.count = 0;
  mp.flush(verts, inds);
}

void export_vertices(RefRun* r, SmartContainer<DualVertex>& v, SmartContainer<uint32_t>& i) {
  r->vpos.resize(v.count * 3);
  r->vnorm.resize(v.count * 3);
  r->vcolor.resize(v.count * 3);
  r->vboundary.resize(v.count);
  r->vvalence.resize(v.count);
  for (size_t k = 0; k < v.count; ++k) {
    const DualVertex& d = v.elements[k];
    r->vpos[3 * k + 0] = d.p.x; r->vpos[3 * k + 1] = d.p.y; r->vpos[3 * k + 2] = d.p.z;
    r->vnorm[3 * k + 0] = d.n.x; r->vnorm[3 * k + 1] = d.n.y; r->vnorm[3 * k + 2] = d.n.z;
    r->vcolor[3 * k + 0] = d.color.x; r->vcolor[3 * k + 1] = d.color.y; r->vcolor[3 * k + 2] = d.color.z;
    r->vboundary[k] = d.boundary ? 1 : 0;
    r->vvalence[k] = d.init_valence;
  }
  r->idx.assign(i.elements, i.elements + i.count);
}

}  // namespace

extern "C" {

// Runs the reference extraction on a caller-provided density block
// (dim^3 floats, z fastest; dim must be a multiple of 32 for the reference's
// mask layout).  iters > 0 adds the MeshProcessor<3> pass exactly as
// ChunkGenerator::extract_chunk does.  Returns an opaque handle.
void* bmfref_run(int dim, const float* density, int iters, int boundary_processing, int smooth_normals) {
  RefRun* r = new RefRun();
  r->dim = dim;

  ResourceAllocator<BinaryBlock> binary_allocator;
  ResourceAllocator<DensityBlock> density_allocator;
  ResourceAllocator<NoiseBlock> noise_allocator;
  ResourceAllocator<VerticesIndicesBlock> vi_allocator;
  ResourceAllocator<DMC_CellsBlock> cell_allocator;
  ResourceAllocator<IndexesBlock> inds_allocator;
  ResourceAllocator<MasksBlock> masks_allocator;

  Sampler sampler;
  sampler.world_size = (float)dim;
  sampler.value = dummy_value;
  const size_t n = (size_t)dim * dim * dim;
  sampler.block = [density, n](const float, const glm::vec3&, const glm::ivec3&, const float, void** out,
                               FastNoiseVectorSet*, float*, int, int, SamplerProperties*) {
    std::memcpy(*out, density, n * sizeof(float));
  };

  DMCChunk* chunk = new DMCChunk();
  chunk->init(glm::vec3(0, 0, 0), (float)(dim - 1), 0, sampler, 0);
  chunk->dim = (uint32_t)dim;
  NoiseSamplers::NoiseSamplerProperties props;
  chunk->label_grid(&binary_allocator, &density_allocator, &noise_allocator, 0.0f, props);
  r->contains_mesh = chunk->contains_mesh ? 1 : 0;
  const uint32_t zc = (dim + 31) / 32;
  r->words.assign(chunk->binary_block->data, chunk->binary_block->data + (size_t)dim * dim * zc);

  chunk->label_edges(&vi_allocator, &cell_allocator, &inds_allocator, &density_allocator, &masks_allocator);
  if (chunk->contains_mesh) {
    // label_edges returns its MasksBlock to the allocator's free list; asking
    // for a block again hands back the same, still-filled buffer.
    MasksBlock* mb = masks_allocator.new_element();
    const size_t count8 = (size_t)((dim + 7) / 8) * dim * dim;
    r->masks.assign(mb->data, mb->data + count8);
    masks_allocator.free_element(mb);

    auto& cells = chunk->cell_block->cells;
    for (size_t c = 0; c < cells.count; ++c) {
      r->cell_mask.push_back(cells.elements[c].mask);
      r->cell_lin.push_back(cells.elements[c].edges[0].grid_v0);
      for (int e = 0; e < 3; ++e) {
        const DMC_Edge& ed = cells.elements[c].edges[e];
        r->cell_vidx.push_back(ed.grid_v1 != (uint32_t)-1 ? ed.iso_vertex.index : 0xFFFFFFFFu);
      }
    }
    r->inds.assign(chunk->indexes_block->inds, chunk->indexes_block->inds + n);
  }

  chunk->polygonize();
  if (chunk->contains_mesh) {
    auto& v = chunk->vi->vertices;
    auto& i = chunk->vi->mesh_indexes;
    if (iters > 0 && v.count && i.count) run_processor<3>(v, i, iters, boundary_processing != 0, smooth_normals != 0);
    export_vertices(r, v, i);
  }
  delete chunk;
  return r;
}

// what: 0 words(u32) 1 masks(u64) 2 cells 3 vertices 4 indices 5 contains_mesh 6 inds(u32, dim^3)
long long bmfref_count(void* h, int what) {
  RefRun* r = (RefRun*)h;
  switch (what) {
    case 0: return (long long)r->words.size();
    case 1: return (long long)r->masks.size();
    case 2: return (long long)r->cell_mask.size();
    case 3: return (long long)r->vboundary.size();
    case 4: return (long long)r->idx.size();
    case 5: return r->contains_mesh;
    case 6: return (long long)r->inds.size();
  }
  return -1;
}

// Copies one result array.  what: 0 words, 1 masks, 2 cell masks (u16),
// 3 cell linear index (u32), 4 cell edge vertex ids (3 x u32 per cell),
// 5 vertex positions (3 x f32), 6 vertex normals, 7 vertex colours,
// 8 vertex boundary flags (u8), 9 vertex valence (u8), 10 indices (u32),
// 11 cell index per sample (u32, dim^3).
void bmfref_copy(void* h, int what, void* dst) {
  RefRun* r = (RefRun*)h;
  auto cp = [dst](const auto& v) { if (!v.empty()) std::memcpy(dst, v.data(), v.size() * sizeof(v[0])); };
  switch (what) {
    case 0: cp(r->words); break;
    case 1: cp(r->masks); break;
    case 2: cp(r->cell_mask); break;
    case 3: cp(r->cell_lin); break;
    case 4: cp(r->cell_vidx); break;
    case 5: cp(r->vpos); break;
    case 6: cp(r->vnorm); break;
    case 7: cp(r->vcolor); break;
    case 8: cp(r->vboundary); break;
    case 9: cp(r->vvalence); break;
    case 10: cp(r->idx); break;
    case 11: cp(r->inds); break;
  }
}

void bmfref_free(void* h) { delete (RefRun*)h; }

// Runs MeshProcessor<N> (N = 3 or 4) on a caller-provided mesh, in the order
// ChunkGenerator::extract_chunk uses.  pos/norm are updated in place; colours
// start at (1,1,1) as DMCChunk::calculate_dual_vertex sets them, normals at the
// caller's values.
void bmfref_process(int N, long long nverts, float* pos, float* norm, float* color, const uint8_t* boundary,
                    const uint8_t* valence, long long nidx, uint32_t* idx, int iters, int boundary_processing,
                    int smooth_normals) {
  SmartContainer<DualVertex> v;
  SmartContainer<uint32_t> i;
  for (long long k = 0; k < nverts; ++k) {
    DualVertex d;
    d.p = glm::vec3(pos[3 * k], pos[3 * k + 1], pos[3 * k + 2]);
    d.n = glm::vec3(norm[3 * k], norm[3 * k + 1], norm[3 * k + 2]);
    d.color = glm::vec3(1, 1, 1);
    d.boundary = boundary[k] != 0;
    d.init_valence = valence[k];
    d.valence = 0;
    d.adj_next = 0;
    d.adj_offset = 0;
    d.index = (uint32_t)k;
    v.push_back(d);
  }
  i.push_back(idx, (size_t)nidx);
  if (N == 3) run_processor<3>(v, i, iters, boundary_processing != 0, smooth_normals != 0);
  else run_processor<4>(v, i, iters, boundary_processing != 0, smooth_normals != 0);
  for (size_t k = 0; k < v.count; ++k) {
    pos[3 * k] = v.elements[k].p.x; pos[3 * k + 1] = v.elements[k].p.y; pos[3 * k + 2] = v.elements[k].p.z;
    norm[3 * k] = v.elements[k].n.x; norm[3 * k + 1] = v.elements[k].n.y; norm[3 * k + 2] = v.elements[k].n.z;
    color[3 * k] = v.elements[k].color.x; color[3 * k + 1] = v.elements[k].color.y; color[3 * k + 2] = v.elements[k].color.z;
  }
  for (size_t k = 0; k < i.count && (long long)k < nidx; ++k) idx[k] = i.elements[k];
}

// The reference's analytic fields through its own block filler
// (ImplicitSampler.cpp:4-65).  kind: 0 torus_z, 1 sphere, 2 cuboid, 3 plane_y.
void bmfref_implicit(int kind, float resolution, float px, float py, float pz, int sx, int sy, int sz, float scale,
                     float* out) {
  glm::vec3 p(px, py, pz);
  glm::ivec3 size(sx, sy, sz);
  void* o = out;
  switch (kind) {
    case 0: ImplicitFunctions::torus_z_block(resolution, p, size, scale, &o, nullptr, nullptr, 0, 4, nullptr); break;
    case 1: ImplicitFunctions::implicit_block(ImplicitFunctions::sphere, resolution, p, size, scale, &o, nullptr, nullptr, 0, 4); break;
    case 2: ImplicitFunctions::cuboid_block(resolution, p, size, scale, &o, nullptr, nullptr, 0, 4, nullptr); break;
    case 3: ImplicitFunctions::implicit_block(ImplicitFunctions::plane_y, resolution, p, size, scale, &o, nullptr, nullptr, 0, 4); break;
  }
}

// The reference QEF (qef_simd.h:550-579), with its SSE rsqrt approximation.
float bmfref_qef_3d(const float* positions, const float* normals, int count, float* solved) {
  float out[4] = {0, 0, 0, 0};
  float e = qef_solve_from_points_3d(positions, normals, count, out);
  solved[0] = out[0]; solved[1] = out[1]; solved[2] = out[2];
  return e;
}

}  // extern "C"
