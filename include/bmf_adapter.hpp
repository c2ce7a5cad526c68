/* bmf_adapter.hpp -- the reference's per-chunk C++ call surface over the C ABI.
 *
 * Header-only C++17 for hosts written against BinaryMeshFitting's own classes:
 * the names, argument meaning and call order of
 *   DMCChunk        (DMCChunk.hpp:61-73: init, label_grid, label_edges, polygonize),
 *   MeshProcessor<N> (MeshProcessor.hpp:66-74: init, optimize_dual_grid,
 *                     optimize_primal_grid, flush),
 *   ChunkGenerator  (ChunkGenerator.hpp:23: process_queue; overlap rule of
 *                     ChunkGenerator.cpp:98)
 * with every stage running in libbmf_gb300.so.  Buffers are device memory
 * (VerticesIndicesBlock's SmartContainers become DeviceArray); errors are
 * thrown as bmf::Error carrying the bmf_status where the reference asserted or
 * ignored a failed allocation.  One Context per host thread, as the C ABI.
 */
#ifndef BMF_ADAPTER_HPP
#define BMF_ADAPTER_HPP

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "bmf.h"

namespace bmf {

struct vec3 {
  float x, y, z;
};

class Error : public std::runtime_error {
 public:
  Error(bmf_status s, const std::string& what) : std::runtime_error(what), status(s) {}
  bmf_status status;
};

inline void check(bmf_status s, const bmf_ctx* ctx = nullptr) {
  if (s != BMF_OK) {
    std::string msg = bmf_status_string(s);
    if (ctx) msg += std::string(": ") + bmf_last_error(ctx);
    throw Error(s, msg);
  }
}

inline void check_cuda(cudaError_t e) {
  if (e != cudaSuccess) throw Error(BMF_ERR_CUDA, cudaGetErrorString(e));
}

/* A grow-only device array (the role of a ResourceAllocator block). */
template <class T>
class DeviceArray {
 public:
  DeviceArray() = default;
  DeviceArray(const DeviceArray&) = delete;
  DeviceArray& operator=(const DeviceArray&) = delete;
  DeviceArray(DeviceArray&& o) noexcept : p_(o.p_), n_(o.n_) { o.p_ = nullptr, o.n_ = 0; }
  ~DeviceArray() {
    if (p_) cudaFree(p_);
  }
  /* Makes room for n elements; the contents are not kept. */
  void reserve(size_t n) {
    if (n <= n_) return;
    if (p_) check_cuda(cudaFree(p_));
    p_ = nullptr;
    n_ = 0;
    check_cuda(cudaMalloc((void**)&p_, (n ? n : 1) * sizeof(T)));
    n_ = n;
  }
  void zero(cudaStream_t s) {
    if (n_) check_cuda(cudaMemsetAsync(p_, 0, n_ * sizeof(T), s));
  }
  /* The first n elements, copied on `s` after the work already queued there. */
  std::vector<T> to_host(size_t n, cudaStream_t s) const {
    std::vector<T> h(n);
    if (n) {
      check_cuda(cudaMemcpyAsync(h.data(), p_, n * sizeof(T), cudaMemcpyDeviceToHost, s));
      check_cuda(cudaStreamSynchronize(s));
    }
    return h;
  }
  T* get() const { return p_; }
  size_t capacity() const { return n_; }

 private:
  T* p_ = nullptr;
  size_t n_ = 0;
};

/* One bmf_ctx on one device, with its stream (not thread-safe). */
class Context {
 public:
  explicit Context(int device = 0) {
    check_cuda(cudaSetDevice(device));
    bmf_config cfg = {device, 0, 0};
    check(bmf_create(&cfg, &h_));
    check_cuda(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
  }
  Context(const Context&) = delete;
  Context& operator=(const Context&) = delete;
  ~Context() {
    if (stream_) cudaStreamDestroy(stream_);
    if (h_) bmf_destroy(h_);
  }
  bmf_ctx* get() const { return h_; }
  cudaStream_t stream() const { return stream_; }

 private:
  bmf_ctx* h_ = nullptr;
  cudaStream_t stream_ = nullptr;
};

/* Sampler (Sampler.hpp:24-34): the density source a chunk samples. */
struct Sampler {
  bmf_field field;
  float world_size;
};

/* A chunk mesh in device memory (VerticesIndicesBlock, ChunkBlocks.hpp:161-179,
 * as structure-of-arrays): positions in sample-index units, normals, the
 * reference's DualVertex::boundary and init_valence, chunk-local indices. */
struct VerticesIndicesBlock {
  DeviceArray<float> pos, nrm;
  DeviceArray<uint8_t> boundary, valence;
  DeviceArray<uint32_t> idx;
  int64_t n_verts = 0, n_idx = 0;
  int32_t prim_size = 3;

  bmf_mesh view() {
    bmf_mesh m = {};
    m.d_pos = pos.get();
    m.d_nrm = nrm.get();
    m.d_boundary = boundary.get();
    m.d_valence = valence.get();
    m.d_idx = idx.get();
    m.vcap = (int64_t)(pos.capacity() / 3);
    m.icap = (int64_t)idx.capacity();
    m.n_verts = n_verts;
    m.n_idx = n_idx;
    m.contains_mesh = n_verts > 0;
    m.prim_size = prim_size;
    return m;
  }
  void reserve(int64_t vcap, int64_t icap) {
    pos.reserve((size_t)vcap * 3);
    nrm.reserve((size_t)vcap * 3);
    boundary.reserve((size_t)vcap);
    valence.reserve((size_t)vcap);
    idx.reserve((size_t)icap);
  }
};

/* The chunk frame of DMCChunk::label_grid (DMCChunk.cpp:94-97), in single
 * precision and in the reference's operation order:
 * delta = size * (1 + overlap * 2) / (dim - 1); overlap_pos = pos - size * overlap. */
inline void chunk_frame(vec3 pos, float size, float overlap, int dim, float* delta, vec3* overlap_pos) {
  volatile float two_o = overlap * 2.0f;  // separately rounded, whatever the host compiler contracts
  volatile float grow = 1.0f + two_o;
  volatile float ext = size * grow;
  *delta = ext / (float)(dim - 1);
  volatile float shift = size * overlap;
  *overlap_pos = {pos.x - shift, pos.y - shift, pos.z - shift};
}

/* DMCChunk's main pipeline (DMCChunk.hpp:66-73) for one chunk. */
class DMCChunk {
 public:
  DMCChunk(Context& ctx, vec3 pos, float size, int level, const Sampler& sampler, int dim = 33)
      : ctx_(&ctx), sampler_(sampler) {
    init(pos, size, level, dim);
  }
  /* DMCChunk::init (DMCChunk.cpp:46-77). */
  void init(vec3 pos, float size, int level, int dim) {
    this->pos = pos;
    this->size = size;
    this->level = level;
    this->dim = dim;
    contains_mesh = false;
    vi.n_verts = vi.n_idx = 0;
  }
  /* DMCChunk::label_grid (DMCChunk.cpp:79-166): the chunk frame, the density
   * block and the binary grid (occupancy words), and contains_mesh. */
  void label_grid(float overlap) {
    chunk_frame(pos, size, overlap, dim, &scale, &overlap_pos);
    bmf_chunk_desc d = {{overlap_pos.x, overlap_pos.y, overlap_pos.z}, scale, dim, level};
    size_t s = (size_t)dim * dim * dim;
    density_.reserve(s);
    words_.reserve((size_t)dim * dim * ((dim + 31) / 32));
    int32_t cm = 0;
    check(bmf_sample_label(ctx_->get(), &d, &sampler_.field, density_.get(), words_.get(), &cm, ctx_->stream()),
          ctx_->get());
    contains_mesh = cm != 0;
  }
  /* DMCChunk::label_edges (DMCChunk.cpp:168-508): the cell masks, the surface
   * cell enumeration and the iso-vertices are computed inside polygonize's
   * kernels from the occupancy words, so nothing is stored at this stage. */
  void label_edges() {}
  /* DMCChunk::polygonize (DMCChunk.cpp:514-576): Mode R (the reference's
   * triangles) by default; Mode Q gives the DMC quads.  Grows the output
   * block when the first capacity guess is too small. */
  void polygonize(int mode = BMF_MODE_R, int placement = BMF_PLACE_CENTER) {
    vi.n_verts = vi.n_idx = 0;
    vi.prim_size = mode == BMF_MODE_R ? 3 : 4;
    if (!contains_mesh) return;
    int64_t vcap = (int64_t)dim * dim * dim / 16 + 1024, icap = (int64_t)dim * dim * dim / 3 + 4096;
    for (int attempt = 0; attempt < 2; ++attempt) {
      vi.reserve(vcap, icap);
      bmf_mesh m = vi.view();
      m.d_nrm = nullptr;  // normals come from MeshProcessor
      bmf_status s = bmf_polygonize(ctx_->get(), dim, density_.get(), words_.get(), mode, placement, &m,
                                    ctx_->stream());
      if (s == BMF_ERR_CAPACITY) {
        vcap = m.n_verts, icap = m.n_idx;
        continue;
      }
      check(s, ctx_->get());
      vi.n_verts = m.n_verts;
      vi.n_idx = m.n_idx;
      return;
    }
    throw Error(BMF_ERR_CAPACITY, "polygonize: capacity did not converge");
  }

  vec3 pos{0, 0, 0}, overlap_pos{0, 0, 0};
  float size = 1.0f, scale = 1.0f;
  int level = 0, dim = 33;
  bool contains_mesh = false;
  VerticesIndicesBlock vi;

 private:
  Context* ctx_;
  Sampler sampler_;
  DeviceArray<float> density_;
  DeviceArray<uint32_t> words_;
};

/* MeshProcessor<N> (MeshProcessor.hpp:66-74).  The dual and primal sweeps run
 * as one device sequence, so the calls are recorded and executed by flush();
 * the supported sequence is ChunkGenerator::extract_chunk's
 * (ChunkGenerator.cpp:114-121): init, optimize_dual_grid(iters, boundary),
 * optimize_primal_grid(false, false, boundary), flush. */
template <int N>
class MeshProcessor {
  static_assert(N == 3 || N == 4, "triangles or quads");

 public:
  MeshProcessor(Context& ctx, bool simple_quality, bool smooth_normals)
      : ctx_(&ctx), simple_quality(simple_quality), smooth_normals_(smooth_normals) {}
  /* MeshProcessor::init (MeshProcessor.cpp:26-55): false when the mesh has
   * no primitives to process. */
  bool init(VerticesIndicesBlock& vertices) {
    if (vertices.prim_size != N) throw Error(BMF_ERR_INVALID_ARGUMENT, "mesh primitive size differs from N");
    mesh_ = &vertices;
    if (vertices.n_verts > 0) check_cuda(cudaMemsetAsync(vertices.nrm.get(), 0, vertices.n_verts * 12, ctx_->stream()));
    return vertices.n_verts > 0 && vertices.n_idx >= N;
  }
  void optimize_dual_grid(int iterations, bool process_boundary = true) {
    iters_ = iterations;
    boundary_ = process_boundary;
  }
  void optimize_primal_grid(bool qef, bool set_colors, bool process_boundary = true) {
    if (iters_ < 0 || qef || set_colors || process_boundary != boundary_)
      throw Error(BMF_ERR_NOT_SUPPORTED, "only the ChunkGenerator::extract_chunk call sequence is supported");
  }
  /* MeshProcessor::flush (MeshProcessor.cpp:57-71): positions and normals
   * are updated in place; no primitive is destroyed on this path, so the
   * index list is unchanged.  Returns with the mesh final, as the
   * reference's flush does (the context's stream is synchronised). */
  void flush() {
    if (!mesh_ || mesh_->n_verts == 0 || iters_ <= 0) return;
    bmf_mesh m = mesh_->view();
    check(bmf_process(ctx_->get(), &m, iters_, boundary_ ? 1 : 0, smooth_normals_ ? 1 : 0, ctx_->stream()),
          ctx_->get());
    check_cuda(cudaStreamSynchronize(ctx_->stream()));
  }

  bool simple_quality;

 private:
  Context* ctx_;
  bool smooth_normals_;
  VerticesIndicesBlock* mesh_ = nullptr;
  int iters_ = -1;
  bool boundary_ = true;
};

/* The extraction knobs of WorldProperties (WorldOctree.cpp:20-33). */
struct WorldProperties {
  int max_level = 7;
  int process_iters = 0;
  float overlap = 0.035f;
  bool boundary_processing = false;
  bool smooth_normals = false;
};

/* The fields of a queued WorldOctreeNode that extraction reads and writes:
 * its chunk's slice of the generator's output arena. */
struct WorldOctreeNode {
  vec3 pos;
  float size;
  int level;
  bool contains_mesh = false;
  int64_t vertex_offset = 0, vertex_count = 0, index_offset = 0, index_count = 0;
};

/* ChunkGenerator::process_queue (ChunkGenerator.hpp:23) as one batched,
 * graph-replayed update.  The plan is kept while the queue keeps its shape
 * (same chunk count and resolution): the next queue's descriptors are swapped
 * in with bmf_batch_set_descs and the captured graph replays. */
class ChunkGenerator {
 public:
  ChunkGenerator(Context& ctx, const WorldProperties& props, const Sampler& sampler, int dim = 33,
                 int mode = BMF_MODE_R, int placement = BMF_PLACE_CENTER)
      : ctx_(&ctx), props(props), sampler_(sampler), dim_(dim), mode_(mode), placement_(placement) {}
  ChunkGenerator(const ChunkGenerator&) = delete;
  ChunkGenerator& operator=(const ChunkGenerator&) = delete;
  ~ChunkGenerator() {
    if (plan_) bmf_batch_destroy(plan_);
  }

  /* ChunkGenerator.cpp:98. */
  float overlap_for(const WorldOctreeNode& n) const {
    if (n.level == props.max_level && (!props.boundary_processing || props.process_iters == 0)) return 0.0f;
    return props.overlap + 0.005f * (float)props.process_iters;
  }

  void process_queue(std::vector<WorldOctreeNode*>& batch) {
    const int n = (int)batch.size();
    if (n == 0) return;
    std::vector<bmf_chunk_desc> descs(n);
    for (int i = 0; i < n; ++i) {
      float delta;
      vec3 op;
      chunk_frame(batch[i]->pos, batch[i]->size, overlap_for(*batch[i]), dim_, &delta, &op);
      descs[i] = {{op.x, op.y, op.z}, delta, dim_, batch[i]->level};
    }
    bool fresh = false;
    if (plan_ && plan_chunks_ == n) {
      check(bmf_batch_set_descs(plan_, descs.data(), n, ctx_->stream()), ctx_->get());
      ++plans_reused;
    } else {
      if (plan_) bmf_batch_destroy(plan_);
      plan_ = nullptr;
      bmf_extract_opts o = {mode_, placement_, props.process_iters, props.boundary_processing ? 1 : 0,
                            props.smooth_normals ? 1 : 0, 0};
      check(bmf_batch_create(ctx_->get(), descs.data(), n, &sampler_.field, &o, &plan_), ctx_->get());
      plan_chunks_ = n;
      info.reserve((size_t)n * 6);
      fresh = true;
    }
    if (fresh && vcap_ == 0) {
      vcap_ = std::max<int64_t>(4096, (int64_t)n * dim_ * dim_ * 4);
      icap_ = std::max<int64_t>(16384, (int64_t)n * dim_ * dim_ * 24);
    }
    for (int attempt = 0; attempt < 3; ++attempt) {
      pos.reserve((size_t)vcap_ * 3);
      if (props.smooth_normals) nrm.reserve((size_t)vcap_ * 3);
      boundary.reserve((size_t)vcap_);
      idx.reserve((size_t)icap_);
      bmf_batch_out out = {pos.get(), props.smooth_normals ? nrm.get() : nullptr, boundary.get(), idx.get(),
                           vcap_, icap_, info.get(), 0, 0};
      bmf_status s = bmf_batch_run(plan_, &out, /*use_graph=*/1, /*sync=*/1, ctx_->stream());
      if (s == BMF_ERR_CAPACITY) {
        vcap_ = out.n_verts + 1024;
        icap_ = out.n_idx + 1024;
        continue;
      }
      check(s, ctx_->get());
      n_verts = out.n_verts;
      n_idx = out.n_idx;
      std::vector<int64_t> h = info.to_host((size_t)n * 6, ctx_->stream());
      for (int i = 0; i < n; ++i) {
        WorldOctreeNode* nd = batch[i];
        nd->vertex_offset = h[6 * i + 0];
        nd->vertex_count = h[6 * i + 1];
        nd->index_offset = h[6 * i + 2];
        nd->index_count = h[6 * i + 3];
        nd->contains_mesh = h[6 * i + 4] != 0;
      }
      return;
    }
    throw Error(BMF_ERR_CAPACITY, "process_queue: arena sizing did not converge");
  }

  WorldProperties props;
  /* The output arena of the last queue (chunk-local indices). */
  DeviceArray<float> pos, nrm;
  DeviceArray<uint8_t> boundary;
  DeviceArray<uint32_t> idx;
  DeviceArray<int64_t> info;
  int64_t n_verts = 0, n_idx = 0;
  int plans_reused = 0;

 private:
  Context* ctx_;
  Sampler sampler_;
  int dim_, mode_, placement_;
  bmf_batch* plan_ = nullptr;
  int plan_chunks_ = 0;
  int64_t vcap_ = 0, icap_ = 0;
};

}  // namespace bmf

#endif
