// C ABI (include/bmf.h): context, scratch arena, per-chunk entry points and
// the batched, CUDA-graph-captured update.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/bmf.h"
#include "bmf_device.cuh"
#include "bmf_trace.h"
#include "bmf_internal.h"

using namespace bmf;

namespace {

enum Slot {
  S_CHUNKS, S_UNITS, S_FLAGS, S_TOT, S_INFO, S_TOTALS, S_WORDS, S_DENS, S_VCNT, S_ICNT, S_GPL,
  S_OFF, S_CURSOR, S_ADJ, S_DUALP, S_DUALN, S_SCANTMP, S_VKEY, S_CLIST, S_LOD, S_NUM
};

constexpr int kMaxDim = 512;
// below this many chunks the sweeps run as whole-mesh kernels: one CTA per
// chunk needs several chunks per resident CTA to balance.  Mode R batches of
// the mixed-LOD update run chunk by chunk from 512 chunks (processing stage,
// whole-mesh -> chunk by chunk: 512 chunks 1.79 -> 1.68 ms, 1024 chunks 2.48
// -> 1.73, 1536 chunks 3.21 -> 2.03); Mode Q batches and fit plans from 2048
// (Mode Q chunk by chunk: mixed 512 / 1024 chunks 1.59 -> 2.21 / 2.24 -> 2.75
// ms, 512 equal chunks lose 3 %)
constexpr int kChunkSweepMinChunks = 2048;
constexpr int kChunkSweepMinChunksR = 512;
// fit plans: the adjoint sweeps run chunk by chunk from this many chunks (one
// 512-thread CTA per chunk, four per SM)
constexpr int kChunkSweepBwdMinChunks = 256;

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

}  // namespace

struct bmf_ctx {
  int device = 0;
  std::string err;
  int64_t launches = 0;
  DevBuf bufs[S_NUM];
  int64_t* h_pinned = nullptr;  // readback staging
};

struct bmf_batch {
  bmf_ctx* ctx = nullptr;
  int n = 0, n_units = 0, max_dim = 0;
  bmf_extract_opts opts{};
  FieldDev field{};
  std::vector<ChunkDev> h_chunks;
  ChunkDev* d_chunks = nullptr;
  int* d_units = nullptr;
  uint32_t* d_flags = nullptr;
  uint32_t* d_tot = nullptr;
  int64_t* d_totals = nullptr;
  float* d_dens = nullptr;
  uint32_t* d_words = nullptr;
  WordScratch ws{};
  // processing scratch (grown with the output capacity)
  int64_t proc_vcap = 0, proc_icap = 0;
  ProcessScratch ps{};
  uint32_t* d_idxg = nullptr;
  uint8_t* d_valence = nullptr;
  uint8_t* d_boundary = nullptr;
  uint32_t* d_vkey = nullptr;
  // captured graph and the output it was captured for
  cudaGraphExec_t exec = nullptr;
  bmf_batch_out graph_out{};
  int64_t graph_kernels = 0;
  int64_t* h_pinned = nullptr;
  ChunkDev* h_stage = nullptr;       // pinned staging for bmf_batch_set_descs
  cudaEvent_t stage_done = nullptr;  // the last staging copy has been consumed
  cudaEvent_t run_done = nullptr;    // recorded after every bmf_batch_run (bmf_batch_wait polls it)
  cudaEvent_t extract_done = nullptr;  // recorded inside every run after the emit (bmf_batch_wait_extraction)
  cudaStream_t aux = nullptr;        // private stream for bmf_batch_wait's read of the totals
  bool ran = false;
  // terrain fill: line items {chunk, first line}, largest chunks first, and
  // the work queue of the persistent form; fill_mode 0 = x-plane kernel,
  // 1 = one CTA per item, 2 = persistent CTAs on the queue
  int2* d_fill_items = nullptr;
  int n_fill_items = 0;
  int* d_queue = nullptr;
  // the chunk-by-chunk sweeps: chunk indices by size, largest first, and their queue
  int* d_order = nullptr;
  int* d_pqueue = nullptr;
  int fill_grid = 0;
  int fill_mode = 0;
  int fill_run = 16;  // the tile height the autotuner picks on the mixed-LOD update
  // band fill (Mode R, terrain): exact densities only where the mesh reads
  // them; d_exact is its per-sample exactness mask (words layout)
  int fill_band = 0;
  uint32_t* d_exact = nullptr;
  // the 2D heightmap's band form (the column fill): the fill stores each
  // (x, z) column height (words layout: chunk.words + x * dim + z) and the
  // occupancy words, no densities; the emit computes a crossing end's
  // density from its column height.  With the band off, the fill still
  // evaluates the heights here once and writes every density from them.
  float* d_cols = nullptr;
  uint2* d_fix = nullptr;  // samples to make exact (+ counter), sized 2 vcap + 1
  int64_t fix_cap = 0;
  // Mode R work list, sized by the output capacity (vcap + icap / 3 + 1)
  uint2* d_clist = nullptr;
  int64_t clist_cap = 0;
};

namespace {

bmf_status fail(bmf_ctx* ctx, bmf_status s, const std::string& msg) {
  if (ctx) ctx->err = msg;
  return s;
}

bmf_status cuda_check(bmf_ctx* ctx, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return BMF_OK;
  return fail(ctx, e == cudaErrorMemoryAllocation ? BMF_ERR_OUT_OF_MEMORY : BMF_ERR_CUDA,
              std::string(what) + ": " + cudaGetErrorString(e));
}

#define BMF_CUDA(ctx, call)                                      \
  do {                                                           \
    bmf_status _s = cuda_check((ctx), (call), #call);            \
    if (_s != BMF_OK) return _s;                                 \
  } while (0)

#define BMF_LAUNCHED(ctx, k)                                                   \
  do {                                                                         \
    (ctx)->launches += (k);                                                    \
    bmf_status _s = cuda_check((ctx), cudaPeekAtLastError(), "kernel launch"); \
    if (_s != BMF_OK) return _s;                                               \
  } while (0)

template <class T>
bmf_status scratch(bmf_ctx* ctx, Slot s, size_t count, T** out) {
  const size_t bytes = count * sizeof(T) + 256;
  DevBuf& b = ctx->bufs[s];
  if (b.bytes < bytes) {
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
    const size_t want = bytes + bytes / 4;
    BMF_CUDA(ctx, cudaMalloc(&b.p, want));
    b.bytes = want;
  }
  *out = (T*)b.p;
  return BMF_OK;
}

uint64_t splitmix64(uint64_t* st) {
  uint64_t z = (*st += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// Noise permutation: Fisher-Yates over 0..255 driven by splitmix64(seed).
FieldDev make_field(const bmf_field* f) {
  FieldDev d{};
  d.kind = f->kind;
  for (int i = 0; i < BMF_FIELD_MAX_PARAMS; ++i) d.p[i] = f->params[i];
  for (int i = 0; i < 256; ++i) d.perm[i] = (uint8_t)i;
  if (f->kind == BMF_FIELD_TERRAIN_FBM || f->kind == BMF_FIELD_TERRAIN_2D) {
    uint64_t st = (uint64_t)(int64_t)f->params[6];
    for (int i = 255; i > 0; --i) {
      const int j = (int)(splitmix64(&st) % (uint64_t)(i + 1));
      const uint8_t t = d.perm[i];
      d.perm[i] = d.perm[j];
      d.perm[j] = t;
    }
  }
  return d;
}

bool field_ok(const bmf_field* f) {
  if (!f || f->kind < BMF_FIELD_GRID || f->kind > BMF_FIELD_TERRAIN_2D) return false;
  for (int i = 0; i < BMF_FIELD_MAX_PARAMS; ++i)
    if (!std::isfinite(f->params[i])) return false;
  if (f->kind == BMF_FIELD_TERRAIN_2D)
    return f->params[2] >= 0 && f->params[2] <= 32 && f->params[7] >= 0 && f->params[7] <= 32;
  return f->kind != BMF_FIELD_TERRAIN_FBM || (f->params[5] >= 0 && f->params[5] <= 32);
}

bool dim_ok(int dim) { return dim >= 2 && dim <= kMaxDim; }

// A chunk descriptor the kernels can sample: dim in range, a finite origin
// and a finite positive sample spacing (a NaN or infinite frame would give
// NaN densities whose signs mean nothing).
bool desc_ok(const bmf_chunk_desc* d) {
  return d && dim_ok(d->dim) && std::isfinite(d->origin[0]) && std::isfinite(d->origin[1]) &&
         std::isfinite(d->origin[2]) && std::isfinite(d->scale) && d->scale > 0.0f;
}

ChunkDev chunk_of(const bmf_chunk_desc* d) {
  ChunkDev c{};
  c.ox = d->origin[0];
  c.oy = d->origin[1];
  c.oz = d->origin[2];
  c.scale = d->scale;
  c.dim = d->dim;
  c.zc = (d->dim + 31) / 32;
  return c;
}

// Uploads a single chunk record and its unit range [0, dim).
bmf_status upload_single(bmf_ctx* ctx, const ChunkDev& c, cudaStream_t st, ChunkDev** d_c, int** d_u) {
  bmf_status s;
  if ((s = scratch(ctx, S_CHUNKS, 1, d_c)) != BMF_OK) return s;
  if ((s = scratch(ctx, S_UNITS, 2, d_u)) != BMF_OK) return s;
  const int units[2] = {0, c.dim};
  BMF_CUDA(ctx, cudaMemcpyAsync(*d_c, &c, sizeof(ChunkDev), cudaMemcpyHostToDevice, st));
  BMF_CUDA(ctx, cudaMemcpyAsync(*d_u, units, sizeof(units), cudaMemcpyHostToDevice, st));
  return BMF_OK;
}

// Count -> scan -> offsets -> emit for chunks already labelled.  Totals land
// in d_totals[0..1] (vertices, indices); flags must be set.
bmf_status extract_core(bmf_ctx* ctx, int mode, int placement, ChunkDev* d_chunks, int n_chunks, const int* d_units,
                        int n_units, const uint32_t* d_words, const float* d_dens, const uint32_t* d_flags,
                        int64_t words_total, const MeshOut& mo, int64_t* d_info, int64_t* d_totals,
                        cudaStream_t st, WordScratch* ws_out = nullptr) {
  WordScratch ws{};
  uint32_t* tot = nullptr;
  bmf_status s;
  if ((s = scratch(ctx, S_VCNT, (size_t)words_total, &ws.vcnt)) != BMF_OK) return s;
  if ((s = scratch(ctx, S_ICNT, (size_t)words_total, &ws.icnt)) != BMF_OK) return s;
  if ((s = scratch(ctx, S_GPL, (size_t)words_total * 3, &ws.gpl)) != BMF_OK) return s;
  if ((s = scratch(ctx, S_TOT, (size_t)n_chunks * 2, &tot)) != BMF_OK) return s;
  {
    // work list of active cells: each one owns a vertex or emits a primitive
    ws.clist_cap = mo.vcap + mo.icap / (mode == BMF_MODE_R ? 3 : 4) + 1;
    uint2* list;
    if ((s = scratch(ctx, S_CLIST, (size_t)ws.clist_cap + 1, &list)) != BMF_OK) return s;
    ws.clist = list;
    ws.ccount = (uint32_t*)(list + ws.clist_cap);
  }
  if (ws_out) *ws_out = ws;
  launch_count(mode, d_chunks, n_chunks, d_units, n_units, d_words, d_flags, ws, st);
  BMF_LAUNCHED(ctx, 1);
  launch_scan_chunks(d_chunks, n_chunks, ws, tot, st);
  BMF_LAUNCHED(ctx, 1);
  launch_chunk_offsets(d_chunks, n_chunks, tot, d_flags, mo.vcap, mo.icap, d_info, d_totals, st);
  BMF_LAUNCHED(ctx, 1);
  BMF_LAUNCHED(ctx, launch_emit(mode, placement, d_chunks, n_chunks, d_units, n_units, d_words, d_dens, d_flags, ws,
                                mo, d_totals, st));
  return BMF_OK;
}

bmf_status mesh_valid(bmf_ctx* ctx, const bmf_mesh* m) {
  if (!m || !m->d_pos || !m->d_idx || m->vcap < 0 || m->icap < 0)
    return fail(ctx, BMF_ERR_INVALID_ARGUMENT, "mesh output: d_pos and d_idx are required");
  return BMF_OK;
}

bmf_status process_mesh(bmf_ctx* ctx, bmf_mesh* mesh, int iters, int pb, int sn, cudaStream_t st,
                        const StructuredAdj* sa = nullptr) {
  const int N = mesh->prim_size;
  if (N != 3 && N != 4) return fail(ctx, BMF_ERR_INVALID_ARGUMENT, "prim_size must be 3 or 4");
  if (!mesh->d_valence || !mesh->d_boundary)
    return fail(ctx, BMF_ERR_INVALID_ARGUMENT, "bmf_process needs d_valence and d_boundary");
  const int64_t nv = mesh->n_verts, n_prims = mesh->n_idx / N;
  // MeshProcessor::init returns early without work on an empty mesh (MeshProcessor.cpp:28-29)
  if (iters <= 0 || nv == 0 || mesh->n_idx < N) return BMF_OK;
  ProcessScratch ps{};
  bmf_status s;
  if ((s = scratch(ctx, S_OFF, (size_t)nv + 1, &ps.off)) != BMF_OK) return s;
  if ((s = scratch(ctx, S_CURSOR, (size_t)nv, &ps.cursor)) != BMF_OK) return s;
  if ((s = scratch(ctx, S_ADJ, (size_t)n_prims * N, &ps.adj)) != BMF_OK) return s;
  if ((s = scratch(ctx, S_DUALP, (size_t)n_prims * 3, &ps.dual_p)) != BMF_OK) return s;
  if ((s = scratch(ctx, S_DUALN, (size_t)n_prims * 3, &ps.dual_n)) != BMF_OK) return s;
  if ((s = scratch(ctx, S_SCANTMP, (size_t)(nv / 4096 + 2), &ps.tmp)) != BMF_OK) return s;
  const int k = launch_process(N, nv, n_prims, nullptr, mesh->d_pos, mesh->d_nrm, mesh->d_boundary,
                               mesh->d_valence, mesh->d_idx, iters, pb, sn, ps, sa, st);
  BMF_LAUNCHED(ctx, k);
  return BMF_OK;
}

}  // namespace

extern "C" {

const char* bmf_status_string(bmf_status s) {
  switch (s) {
    case BMF_OK: return "ok";
    case BMF_ERR_INVALID_ARGUMENT: return "invalid argument";
    case BMF_ERR_CUDA: return "CUDA error";
    case BMF_ERR_CAPACITY: return "output capacity exceeded";
    case BMF_ERR_TIMEOUT: return "device wait timed out";
    case BMF_ERR_OUT_OF_MEMORY: return "out of device memory";
    case BMF_ERR_NOT_SUPPORTED: return "not supported";
  }
  return "unknown status";
}

bmf_status bmf_create(const bmf_config* cfg, bmf_ctx** out) {
  if (!out) return BMF_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) return BMF_ERR_CUDA;
  const int dev = cfg ? cfg->device : 0;
  if (dev < 0 || dev >= n) return BMF_ERR_INVALID_ARGUMENT;
  if (cudaSetDevice(dev) != cudaSuccess) return BMF_ERR_CUDA;
  bmf_ctx* ctx = new bmf_ctx();
  ctx->device = dev;
  if (cudaMallocHost(&ctx->h_pinned, 64 * sizeof(int64_t)) != cudaSuccess) {
    delete ctx;
    return BMF_ERR_OUT_OF_MEMORY;
  }
  *out = ctx;
  return BMF_OK;
}

bmf_status bmf_destroy(bmf_ctx* ctx) {
  if (!ctx) return BMF_ERR_INVALID_ARGUMENT;
  cudaSetDevice(ctx->device);
  for (auto& b : ctx->bufs)
    if (b.p) cudaFree(b.p);
  if (ctx->h_pinned) cudaFreeHost(ctx->h_pinned);
  delete ctx;
  return BMF_OK;
}

const char* bmf_last_error(const bmf_ctx* ctx) { return ctx ? ctx->err.c_str() : "no context"; }
int64_t bmf_launch_count(const bmf_ctx* ctx) { return ctx ? ctx->launches : 0; }

bmf_status bmf_sample_label(bmf_ctx* ctx, const bmf_chunk_desc* desc, const bmf_field* field, float* d_density,
                            uint32_t* d_words, int32_t* h_contains_mesh, void* stream) {
  BMF_TRACE("bmf_sample_label");
  if (!ctx) return BMF_ERR_INVALID_ARGUMENT;
  if (!desc_ok(desc) || !field_ok(field) || !d_words)
    return fail(ctx, BMF_ERR_INVALID_ARGUMENT, "bmf_sample_label: bad descriptor, field or words pointer");
  if (field->kind == BMF_FIELD_GRID && !d_density)
    return fail(ctx, BMF_ERR_INVALID_ARGUMENT, "BMF_FIELD_GRID reads d_density, which must be given");
  cudaStream_t st = (cudaStream_t)stream;
  ChunkDev c = chunk_of(desc);
  ChunkDev* d_c;
  int* d_u;
  uint32_t* d_flags;
  bmf_status s;
  if ((s = upload_single(ctx, c, st, &d_c, &d_u)) != BMF_OK) return s;
  if ((s = scratch(ctx, S_FLAGS, 1, &d_flags)) != BMF_OK) return s;
  BMF_CUDA(ctx, cudaMemsetAsync(d_flags, 0, sizeof(uint32_t), st));
  const FieldDev fd = make_field(field);
  launch_sample_label(d_c, 1, d_u, c.dim, c.dim, fd, d_density, field->kind == BMF_FIELD_GRID ? nullptr : d_density,
                      d_words, d_flags, st);
  BMF_LAUNCHED(ctx, 1);
  if (h_contains_mesh) {
    uint32_t f = 0;
    BMF_CUDA(ctx, cudaMemcpyAsync(&f, d_flags, sizeof(f), cudaMemcpyDeviceToHost, st));
    BMF_CUDA(ctx, cudaStreamSynchronize(st));
    *h_contains_mesh = ((f & 1u) || ((f & 6u) == 6u)) ? 1 : 0;
  }
  return BMF_OK;
}

bmf_status bmf_sample_block(bmf_ctx* ctx, const bmf_chunk_desc* desc, const bmf_field* field, float* d_density,
                            void* stream) {
  BMF_TRACE("bmf_sample_block");
  if (!ctx) return BMF_ERR_INVALID_ARGUMENT;
  if (!desc_ok(desc) || !field_ok(field) || field->kind == BMF_FIELD_GRID || !d_density)
    return fail(ctx, BMF_ERR_INVALID_ARGUMENT, "bmf_sample_block: bad descriptor, field or density pointer");
  const int dim = desc->dim, zc = (dim + 31) / 32;
  uint32_t* words;
  bmf_status s;
  if ((s = scratch(ctx, S_WORDS, (size_t)dim * dim * zc, &words)) != BMF_OK) return s;
  return bmf_sample_label(ctx, desc, field, d_density, words, nullptr, stream);
}

bmf_status bmf_label_grid(bmf_ctx* ctx, int32_t dim, const float* d_density, uint32_t* d_words,
                          int32_t* h_contains_mesh, void* stream) {
  BMF_TRACE("bmf_label_grid");
  if (!ctx) return BMF_ERR_INVALID_ARGUMENT;
  bmf_chunk_desc d{};
  d.scale = 1.0f;
  d.dim = dim;
  bmf_field f{};
  f.kind = BMF_FIELD_GRID;
  return bmf_sample_label(ctx, &d, &f, const_cast<float*>(d_density), d_words, h_contains_mesh, stream);
}

bmf_status bmf_cell_masks(bmf_ctx* ctx, int32_t dim, const uint32_t* d_words, uint8_t* d_masks, void* stream) {
  BMF_TRACE("bmf_cell_masks");
  if (!ctx) return BMF_ERR_INVALID_ARGUMENT;
  if (!dim_ok(dim) || !d_words || !d_masks) return fail(ctx, BMF_ERR_INVALID_ARGUMENT, "bmf_cell_masks: bad args");
  launch_cell_masks(dim, d_words, d_masks, (cudaStream_t)stream);
  BMF_LAUNCHED(ctx, 1);
  return BMF_OK;
}

bmf_status bmf_polygonize(bmf_ctx* ctx, int32_t dim, const float* d_density, const uint32_t* d_words, int32_t mode,
                          int32_t placement, bmf_mesh* out, void* stream) {
  BMF_TRACE("bmf_polygonize");
  if (!ctx) return BMF_ERR_INVALID_ARGUMENT;
  bmf_status s;
  if ((s = mesh_valid(ctx, out)) != BMF_OK) return s;
  if (!dim_ok(dim) || !d_words || (mode != BMF_MODE_R && mode != BMF_MODE_Q) || placement < 0 || placement > 2)
    return fail(ctx, BMF_ERR_INVALID_ARGUMENT, "bmf_polygonize: bad dim, words, mode or placement");
  if (!d_density && (mode == BMF_MODE_R || placement != BMF_PLACE_CENTER))
    return fail(ctx, BMF_ERR_INVALID_ARGUMENT, "bmf_polygonize: this mode needs d_density");
  cudaStream_t st = (cudaStream_t)stream;
  ChunkDev c{};
  c.scale = 1.0f;
  c.dim = dim;
  c.zc = (dim + 31) / 32;
  ChunkDev* d_c;
  int* d_u;
  uint32_t* d_flags;
  int64_t* d_totals;
  if ((s = upload_single(ctx, c, st, &d_c, &d_u)) != BMF_OK) return s;
  if ((s = scratch(ctx, S_FLAGS, 1, &d_flags)) != BMF_OK) return s;
  if ((s = scratch(ctx, S_TOTALS, 2, &d_totals)) != BMF_OK) return s;
  launch_word_flags(d_c, 1, d_words, d_flags, st);
  BMF_LAUNCHED(ctx, 1);
  MeshOut mo{out->d_pos, out->d_nrm, out->d_boundary, out->d_valence, out->d_idx, nullptr, out->vcap, out->icap};
  if (mode == BMF_MODE_Q && placement == BMF_PLACE_QEF &&
      (s = scratch(ctx, S_VKEY, (size_t)out->vcap + 1, &mo.vkey)) != BMF_OK)
    return s;
  if ((s = extract_core(ctx, mode, placement, d_c, 1, d_u, dim, d_words, d_density, d_flags,
                        (int64_t)dim * dim * c.zc, mo, nullptr, d_totals, st)) != BMF_OK)
    return s;
  BMF_CUDA(ctx, cudaMemcpyAsync(ctx->h_pinned, d_totals, 2 * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  BMF_CUDA(ctx, cudaMemcpyAsync(ctx->h_pinned + 2, d_flags, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  BMF_CUDA(ctx, cudaStreamSynchronize(st));
  out->n_verts = ctx->h_pinned[0];
  out->n_idx = ctx->h_pinned[1];
  const uint32_t f = (uint32_t)ctx->h_pinned[2];
  out->contains_mesh = ((f & 1u) || ((f & 6u) == 6u)) ? 1 : 0;
  out->prim_size = mode == BMF_MODE_R ? 3 : 4;
  if (out->n_verts > out->vcap || out->n_idx > out->icap)
    return fail(ctx, BMF_ERR_CAPACITY, "bmf_polygonize: output capacity exceeded (needed counts reported)");
  return BMF_OK;
}

bmf_status bmf_process(bmf_ctx* ctx, bmf_mesh* mesh, int32_t iters, int32_t process_boundary,
                       int32_t smooth_normals, void* stream) {
  BMF_TRACE("bmf_process");
  if (!ctx) return BMF_ERR_INVALID_ARGUMENT;
  bmf_status s;
  if ((s = mesh_valid(ctx, mesh)) != BMF_OK) return s;
  if (mesh->n_verts > mesh->vcap || mesh->n_idx > mesh->icap || iters < 0)
    return fail(ctx, BMF_ERR_INVALID_ARGUMENT, "bmf_process: counts exceed capacities or negative iters");
  return process_mesh(ctx, mesh, iters, process_boundary, smooth_normals, (cudaStream_t)stream);
}

bmf_status bmf_lod_generate(bmf_ctx* ctx, const bmf_lod_params* p, bmf_chunk_desc* d_descs, int32_t cap,
                            int32_t* d_count, void* stream) {
  BMF_TRACE("bmf_lod_generate");
  if (!ctx) return BMF_ERR_INVALID_ARGUMENT;
  if (!p || !d_descs || !d_count || cap <= 0 || cap > kLodMaxLeaves || p->max_level < 0 || p->max_level > 20 ||
      p->min_level < 0 || !dim_ok(p->dim) || !(p->root_size > 0.0f))
    return fail(ctx, BMF_ERR_INVALID_ARGUMENT,
                "bmf_lod_generate: params, device outputs, 0 < cap <= 16384, max_level <= 20 and a valid dim needed");
  char* scr;
  bmf_status s;
  if ((s = scratch(ctx, S_LOD, lod_scratch_bytes(cap), &scr)) != BMF_OK) return s;
  BMF_LAUNCHED(ctx, lod_generate(*p, d_descs, cap, d_count, scr, (cudaStream_t)stream));
  return BMF_OK;
}

bmf_status bmf_format(bmf_ctx* ctx, const bmf_mesh* mesh, int32_t unwind, int32_t smooth_normals, float* d_p,
                      float* d_n, float* d_c, int64_t cap, int64_t* h_count, void* stream) {
  BMF_TRACE("bmf_format");
  if (!ctx) return BMF_ERR_INVALID_ARGUMENT;
  if (!mesh || !mesh->d_pos || !d_p || !d_n || !d_c || cap < 0 || mesh->n_verts < 0 || mesh->n_idx < 0 ||
      (unwind && (mesh->prim_size != 4 || !mesh->d_idx)) || (unwind && smooth_normals && !mesh->d_nrm))
    return fail(ctx, BMF_ERR_INVALID_ARGUMENT,
                "bmf_format: mesh and output buffers required; unwinding needs quads (prim_size 4) and, with "
                "smooth_normals, vertex normals");
  const int64_t count = unwind ? mesh->n_idx / 4 * 4 : mesh->n_verts;
  if (count > cap) {
    if (h_count) *h_count = count;
    return fail(ctx, BMF_ERR_CAPACITY, "bmf_format: output capacity exceeded (needed count reported)");
  }
  cudaStream_t st = (cudaStream_t)stream;
  BMF_LAUNCHED(ctx, launch_format(nullptr, 1, mesh->n_verts, mesh->n_idx, nullptr, mesh->d_pos, mesh->d_nrm,
                                  mesh->d_idx, unwind, smooth_normals, d_p, d_n, d_c, cap, st));
  BMF_CUDA(ctx, cudaPeekAtLastError());
  if (h_count) {
    BMF_CUDA(ctx, cudaStreamSynchronize(st));
    *h_count = count;
  }
  return BMF_OK;
}

bmf_status bmf_extract_chunk(bmf_ctx* ctx, const bmf_chunk_desc* desc, const bmf_field* field,
                             const bmf_extract_opts* opts, bmf_mesh* out, void* stream) {
  BMF_TRACE("bmf_extract_chunk");
  if (!ctx) return BMF_ERR_INVALID_ARGUMENT;
  bmf_status s;
  if ((s = mesh_valid(ctx, out)) != BMF_OK) return s;
  if (!desc_ok(desc) || !field_ok(field) || field->kind == BMF_FIELD_GRID || !opts ||
      (opts->mode != BMF_MODE_R && opts->mode != BMF_MODE_Q) || opts->placement < 0 || opts->placement > 2 ||
      opts->iters < 0)
    return fail(ctx, BMF_ERR_INVALID_ARGUMENT, "bmf_extract_chunk: bad descriptor, field or options");
  if (opts->iters > 0 && (!out->d_valence || !out->d_boundary))
    return fail(ctx, BMF_ERR_INVALID_ARGUMENT, "bmf_extract_chunk: smoothing needs d_valence and d_boundary");
  cudaStream_t st = (cudaStream_t)stream;
  const ChunkDev c = chunk_of(desc);
  const int dim = c.dim;
  ChunkDev* d_c;
  int* d_u;
  uint32_t* d_flags;
  int64_t* d_totals;
  float* d_dens;
  uint32_t* d_words;
  if ((s = upload_single(ctx, c, st, &d_c, &d_u)) != BMF_OK) return s;
  if ((s = scratch(ctx, S_FLAGS, 1, &d_flags)) != BMF_OK) return s;
  if ((s = scratch(ctx, S_TOTALS, 2, &d_totals)) != BMF_OK) return s;
  if ((s = scratch(ctx, S_DENS, (size_t)dim * dim * dim, &d_dens)) != BMF_OK) return s;
  if ((s = scratch(ctx, S_WORDS, (size_t)dim * dim * c.zc, &d_words)) != BMF_OK) return s;
  BMF_CUDA(ctx, cudaMemsetAsync(d_flags, 0, sizeof(uint32_t), st));
  const FieldDev fd = make_field(field);
  launch_sample_label(d_c, 1, d_u, dim, dim, fd, nullptr, d_dens, d_words, d_flags, st);
  BMF_LAUNCHED(ctx, 1);
  MeshOut mo{out->d_pos, out->d_nrm, out->d_boundary, out->d_valence, out->d_idx, nullptr, out->vcap, out->icap};
  if ((opts->iters > 0 || (opts->mode == BMF_MODE_Q && opts->placement == BMF_PLACE_QEF)) &&
      (s = scratch(ctx, S_VKEY, (size_t)out->vcap + 1, &mo.vkey)) != BMF_OK)
    return s;
  WordScratch ws{};
  if ((s = extract_core(ctx, opts->mode, opts->placement, d_c, 1, d_u, dim, d_words, d_dens, d_flags,
                        (int64_t)dim * dim * c.zc, mo, nullptr, d_totals, st, &ws)) != BMF_OK)
    return s;
  BMF_CUDA(ctx, cudaMemcpyAsync(ctx->h_pinned, d_totals, 2 * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  BMF_CUDA(ctx, cudaMemcpyAsync(ctx->h_pinned + 2, d_flags, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  BMF_CUDA(ctx, cudaStreamSynchronize(st));
  out->n_verts = ctx->h_pinned[0];
  out->n_idx = ctx->h_pinned[1];
  const uint32_t f = (uint32_t)ctx->h_pinned[2];
  out->contains_mesh = ((f & 1u) || ((f & 6u) == 6u)) ? 1 : 0;
  out->prim_size = opts->mode == BMF_MODE_R ? 3 : 4;
  if (out->n_verts > out->vcap || out->n_idx > out->icap)
    return fail(ctx, BMF_ERR_CAPACITY, "bmf_extract_chunk: output capacity exceeded (needed counts reported)");
  // ChunkGenerator.cpp:112: processing only when the chunk has a mesh
  if (opts->iters > 0 && out->contains_mesh && out->n_verts && out->n_idx) {
    const StructuredAdj sa{opts->mode, d_c, 1, d_words, ws, mo.vkey};
    if ((s = process_mesh(ctx, out, opts->iters, opts->process_boundary, opts->smooth_normals, st, &sa)) != BMF_OK)
      return s;
    BMF_CUDA(ctx, cudaStreamSynchronize(st));
  }
  return BMF_OK;
}

// ---------------------------------------------------------------------------
// batched update
// ---------------------------------------------------------------------------

bmf_status bmf_batch_create(bmf_ctx* ctx, const bmf_chunk_desc* h_descs, int32_t n_chunks, const bmf_field* field,
                            const bmf_extract_opts* opts, bmf_batch** out) {
  BMF_TRACE("bmf_batch_create");
  if (!ctx || !out) return BMF_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  if (!h_descs || n_chunks <= 0 || !field_ok(field) || field->kind == BMF_FIELD_GRID || !opts ||
      (opts->mode != BMF_MODE_R && opts->mode != BMF_MODE_Q) || opts->placement < 0 || opts->placement > 2 ||
      opts->iters < 0)
    return fail(ctx, BMF_ERR_INVALID_ARGUMENT, "bmf_batch_create: bad descriptors, field or options");
  bmf_batch* b = new bmf_batch();
  b->ctx = ctx;
  b->n = n_chunks;
  b->opts = *opts;
  b->field = make_field(field);
  b->h_chunks.resize(n_chunks);
  std::vector<int> units(n_chunks + 1);
  int64_t dens = 0, words = 0;
  int n_units = 0;
  for (int i = 0; i < n_chunks; ++i) {
    if (!desc_ok(h_descs + i)) {
      delete b;
      return fail(ctx, BMF_ERR_INVALID_ARGUMENT,
                  "bmf_batch_create: chunk " + std::to_string(i) +
                      ": dim out of range, or a non-finite origin or a non-positive / non-finite scale");
    }
    ChunkDev c = chunk_of(h_descs + i);
    c.dens = dens;
    c.words = words;
    dens += (int64_t)c.dim * c.dim * c.dim;
    words += (int64_t)c.dim * c.dim * c.zc;
    units[i] = n_units;
    n_units += c.dim;
    b->max_dim = c.dim > b->max_dim ? c.dim : b->max_dim;
    b->h_chunks[i] = c;
  }
  units[n_chunks] = n_units;
  b->n_units = n_units;
  auto bail = [&](cudaError_t e, const char* what) {
    bmf_status s = cuda_check(ctx, e, what);
    if (s != BMF_OK) bmf_batch_destroy(b);
    return s;
  };
  bmf_status s;
  if ((s = bail(cudaMalloc(&b->d_chunks, sizeof(ChunkDev) * n_chunks), "chunks")) != BMF_OK) return s;
  if ((s = bail(cudaMalloc(&b->d_units, sizeof(int) * (n_chunks + 1)), "units")) != BMF_OK) return s;
  if ((s = bail(cudaMalloc(&b->d_flags, sizeof(uint32_t) * n_chunks), "flags")) != BMF_OK) return s;
  if ((s = bail(cudaMalloc(&b->d_tot, sizeof(uint32_t) * 2 * n_chunks), "tot")) != BMF_OK) return s;
  if ((s = bail(cudaMalloc(&b->d_totals, sizeof(int64_t) * 2), "totals")) != BMF_OK) return s;
  if ((s = bail(cudaMalloc(&b->d_dens, sizeof(float) * dens), "density")) != BMF_OK) return s;
  if ((s = bail(cudaMalloc(&b->d_words, sizeof(uint32_t) * words), "words")) != BMF_OK) return s;
  if ((s = bail(cudaMalloc(&b->ws.vcnt, sizeof(uint32_t) * words), "vcnt")) != BMF_OK) return s;
  if ((s = bail(cudaMalloc(&b->ws.icnt, sizeof(uint32_t) * words), "icnt")) != BMF_OK) return s;
  if ((s = bail(cudaMalloc(&b->ws.gpl, sizeof(uint32_t) * 3 * words), "gpl")) != BMF_OK) return s;
  if ((s = bail(cudaMallocHost(&b->h_pinned, sizeof(int64_t) * 4), "pinned")) != BMF_OK) return s;
  if ((s = bail(cudaMemcpy(b->d_chunks, b->h_chunks.data(), sizeof(ChunkDev) * n_chunks, cudaMemcpyHostToDevice),
                "upload chunks")) != BMF_OK)
    return s;
  if ((s = bail(cudaMemcpy(b->d_units, units.data(), sizeof(int) * (n_chunks + 1), cudaMemcpyHostToDevice),
                "upload units")) != BMF_OK)
    return s;
  // chunks by size, largest first (longest-processing-time order for the
  // work queues of the fill and of the chunk-by-chunk sweeps)
  std::vector<int> order(n_chunks);
  for (int i = 0; i < n_chunks; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int c) { return b->h_chunks[a].dim > b->h_chunks[c].dim; });
  if ((s = bail(cudaMalloc(&b->d_order, sizeof(int) * n_chunks), "chunk order")) != BMF_OK) return s;
  if ((s = bail(cudaMalloc(&b->d_pqueue, sizeof(int)), "sweep queue")) != BMF_OK) return s;
  if ((s = bail(cudaMemcpy(b->d_order, order.data(), sizeof(int) * n_chunks, cudaMemcpyHostToDevice),
                "upload chunk order")) != BMF_OK)
    return s;
  if (b->field.kind == BMF_FIELD_TERRAIN_FBM) {
    // line items in that order
    std::vector<int2> items;
    for (int i : order) {
      const int n_it = fill_terrain_items(b->h_chunks[i].dim);
      for (int k = 0; k < n_it; ++k) items.push_back(make_int2(i, k * fill_terrain_lines()));
    }
    b->n_fill_items = (int)items.size();
    if ((s = bail(cudaMalloc(&b->d_fill_items, sizeof(int2) * items.size()), "fill items")) != BMF_OK) return s;
    if ((s = bail(cudaMalloc(&b->d_queue, sizeof(int)), "fill queue")) != BMF_OK) return s;
    if ((s = bail(cudaMemcpy(b->d_fill_items, items.data(), sizeof(int2) * items.size(), cudaMemcpyHostToDevice),
                  "upload fill items")) != BMF_OK)
      return s;
    b->fill_mode = 2;
    if (b->opts.mode == BMF_MODE_R && fill_band_supported(b->field)) {
      if ((s = bail(cudaMalloc(&b->d_exact, sizeof(uint32_t) * words), "exactness mask")) != BMF_OK) return s;
      b->fill_band = 1;
    }
    b->fill_grid = fill_terrain_resident_ctas(b->fill_run, (int)b->field.p[5], b->fill_band != 0);
  }
  if (b->field.kind == BMF_FIELD_TERRAIN_2D && b->opts.mode == BMF_MODE_R && fill_band_supported(b->field)) {
    // column items {chunk, first column}, largest chunks first
    std::vector<int2> items;
    const int per = columns2d_item();
    for (int i : order) {
      const int nc = b->h_chunks[i].dim * b->h_chunks[i].dim;
      for (int k = 0; k < nc; k += per) items.push_back(make_int2(i, k));
    }
    b->n_fill_items = (int)items.size();
    if ((s = bail(cudaMalloc(&b->d_fill_items, sizeof(int2) * items.size()), "column items")) != BMF_OK) return s;
    if ((s = bail(cudaMemcpy(b->d_fill_items, items.data(), sizeof(int2) * items.size(), cudaMemcpyHostToDevice),
                  "upload column items")) != BMF_OK)
      return s;
    if ((s = bail(cudaMalloc(&b->d_cols, sizeof(float) * words), "column heights")) != BMF_OK) return s;
    b->fill_band = 1;
  }
  if ((s = bail(cudaEventCreateWithFlags(&b->extract_done, cudaEventDisableTiming), "extraction event")) != BMF_OK)
    return s;
  *out = b;
  return BMF_OK;
}

namespace {

// The band form of the fill is on: the terrain FBM's band fill, or the 2D
// heightmap's column fill.
bool batch_band(const bmf_batch* b) {
  if (!b->fill_band) return false;
  if (b->field.kind == BMF_FIELD_TERRAIN_FBM) return b->d_exact && b->fill_mode != 0;
  return b->field.kind == BMF_FIELD_TERRAIN_2D && b->d_cols;
}

// The work list of active cells for an output arena of (vcap, icap) (+ its counter).
bmf_status batch_list_scratch(bmf_batch* b, int64_t vcap, int64_t icap) {
  const int64_t cap = vcap + icap / (b->opts.mode == BMF_MODE_R ? 3 : 4) + 1;
  if (cap > b->clist_cap) {
    if (b->d_clist) cudaFree(b->d_clist);
    b->d_clist = nullptr;
    b->clist_cap = 0;
    BMF_CUDA(b->ctx, cudaMalloc(&b->d_clist, sizeof(uint2) * (cap + 1)));
    b->clist_cap = cap;
  }
  b->ws.clist = b->d_clist;
  b->ws.ccount = (uint32_t*)(b->d_clist + b->clist_cap);
  b->ws.clist_cap = b->clist_cap;
  if (b->d_exact) {
    // band fill: every crossing (one vertex each in Mode R) lists at most its two ends
    const int64_t fcap = 2 * vcap + 1;
    if (fcap > b->fix_cap) {
      if (b->d_fix) cudaFree(b->d_fix);
      b->d_fix = nullptr;
      b->fix_cap = 0;
      BMF_CUDA(b->ctx, cudaMalloc(&b->d_fix, sizeof(uint2) * (fcap + 1)));
      b->fix_cap = fcap;
    }
    b->ws.fix = b->d_fix;
    b->ws.fcount = (uint32_t*)(b->d_fix + b->fix_cap);
    b->ws.fix_cap = b->fix_cap;
  }
  const bool band = batch_band(b);
  b->ws.exact = band && b->field.kind == BMF_FIELD_TERRAIN_FBM ? b->d_exact : nullptr;
  const bool col2d = band && b->field.kind == BMF_FIELD_TERRAIN_2D;
  b->ws.cols2d = col2d ? b->d_cols : nullptr;
  b->ws.c2d_g = b->field.p[0];
  b->ws.c2d_height = b->field.p[1];
  return BMF_OK;
}

// Vertex keys are kept for the sweeps' adjacency and for per-vertex QEF placement.
bool batch_keys(const bmf_batch* b) {
  return b->opts.iters > 0 || (b->opts.mode == BMF_MODE_Q && b->opts.placement == BMF_PLACE_QEF);
}

// Density fill + occupancy words of a whole update.

void batch_fill(bmf_batch* b, cudaStream_t st) {
  if (b->field.kind == BMF_FIELD_TERRAIN_FBM && b->fill_mode != 0)
    launch_fill_terrain(b->fill_run, b->d_chunks, b->d_fill_items, b->n_fill_items,
                        b->fill_mode == 2 ? b->d_queue : nullptr, b->fill_grid, b->field, b->d_dens, b->d_words,
                        b->d_flags, batch_band(b) ? b->d_exact : nullptr, st);
  else if (b->d_cols) {
    // the 2D heightmap: every column height once, then the words (and, with
    // the column fill off, every density) from them
    launch_columns2d(b->d_chunks, b->d_fill_items, b->n_fill_items, b->field, b->d_cols, st);
    if (batch_band(b))
      launch_words2d(b->d_chunks, b->n, b->d_units, b->n_units, b->field, b->d_cols, b->d_words, b->d_flags, st);
    else
      launch_sample_label(b->d_chunks, b->n, b->d_units, b->n_units, b->max_dim, b->field, nullptr, b->d_dens,
                          b->d_words, b->d_flags, st, b->d_cols);
  } else
    launch_sample_label(b->d_chunks, b->n, b->d_units, b->n_units, b->max_dim, b->field, nullptr, b->d_dens,
                        b->d_words, b->d_flags, st);
}

bmf_status batch_proc_scratch(bmf_batch* b, int64_t vcap, int64_t icap) {
  if (vcap <= b->proc_vcap && icap <= b->proc_icap) return BMF_OK;
  bmf_ctx* ctx = b->ctx;
  const int N = b->opts.mode == BMF_MODE_R ? 3 : 4;
  const int64_t np = icap / N;
  void* ptrs[] = {b->ps.off, b->ps.cursor, b->ps.adj, b->ps.dual_p, b->ps.dual_n, b->ps.tmp,
                  b->d_idxg, b->d_valence, b->d_boundary, b->d_vkey};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  b->proc_vcap = b->proc_icap = 0;
  BMF_CUDA(ctx, cudaMalloc(&b->ps.off, sizeof(uint32_t) * (vcap + 1)));
  BMF_CUDA(ctx, cudaMalloc(&b->ps.cursor, sizeof(uint32_t) * (vcap + 1)));
  BMF_CUDA(ctx, cudaMalloc(&b->ps.adj, sizeof(uint32_t) * (np * N + 1)));
  // 4 floats per primitive: the chunk-by-chunk sweeps keep (p, n.x) as one float4
  BMF_CUDA(ctx, cudaMalloc(&b->ps.dual_p, sizeof(float) * (4 * np + 4)));
  BMF_CUDA(ctx, cudaMalloc(&b->ps.dual_n, sizeof(float) * (3 * np + 3)));
  BMF_CUDA(ctx, cudaMalloc(&b->ps.tmp, sizeof(uint32_t) * (vcap / 4096 + 2)));
  BMF_CUDA(ctx, cudaMalloc(&b->d_idxg, sizeof(uint32_t) * (icap + 1)));
  BMF_CUDA(ctx, cudaMalloc(&b->d_valence, vcap + 1));
  BMF_CUDA(ctx, cudaMalloc(&b->d_boundary, vcap + 1));
  BMF_CUDA(ctx, cudaMalloc(&b->d_vkey, sizeof(uint32_t) * (vcap + 1)));
  b->proc_vcap = vcap;
  b->proc_icap = icap;
  return BMF_OK;
}

// The structured adjacency of a batch; with enough chunks to fill the GPU
// the sweeps run chunk by chunk (one CTA per chunk, largest chunks first).
StructuredAdj batch_adj(const bmf_batch* b) {
  StructuredAdj sa{b->opts.mode, b->d_chunks, b->n, b->d_words, b->ws, b->d_vkey};
  if (b->n >= (b->opts.mode == BMF_MODE_R ? kChunkSweepMinChunksR : kChunkSweepMinChunks)) {
    sa.tot = b->d_tot;
    sa.order = b->d_order;
    sa.queue = b->d_pqueue;
  }
  return sa;
}

// Enqueues one whole update on st (captured into the graph, or run directly).
bmf_status batch_record(bmf_batch* b, const bmf_batch_out* out, cudaStream_t st, int64_t* kernels) {
  bmf_ctx* ctx = b->ctx;
  const bool proc = b->opts.iters > 0;
  BMF_CUDA(ctx, cudaMemsetAsync(b->d_flags, 0, sizeof(uint32_t) * b->n, st));
  batch_fill(b, st);
  launch_count(b->opts.mode, b->d_chunks, b->n, b->d_units, b->n_units, b->d_words, b->d_flags, b->ws, st);
  const bool band = batch_band(b) && b->field.kind == BMF_FIELD_TERRAIN_FBM;  // the 2D column fill needs no fix-up
  if (band) launch_fill_fixup(b->d_chunks, b->ws, b->field, b->d_dens, st);
  launch_scan_chunks(b->d_chunks, b->n, b->ws, b->d_tot, st, b->d_order);
  launch_chunk_offsets(b->d_chunks, b->n, b->d_tot, b->d_flags, out->vcap, out->icap, out->d_chunk_info,
                       b->d_totals, st);
  MeshOut mo{out->d_pos, out->d_nrm, proc ? b->d_boundary : out->d_boundary, proc ? b->d_valence : nullptr,
             out->d_idx, proc ? b->d_idxg : nullptr, out->vcap, out->icap, batch_keys(b) ? b->d_vkey : nullptr};
  int64_t k = (band ? 5 : 4) + (b->d_cols ? 1 : 0);
  k += launch_emit(b->opts.mode, b->opts.placement, b->d_chunks, b->n, b->d_units, b->n_units, b->d_words, b->d_dens,
                   b->d_flags, b->ws, mo, b->d_totals, st);
  // indices and chunk table are final here (bmf_batch_wait_extraction); an
  // external record, so that under capture the graph records the event itself
  // and streams outside the graph can wait on it
  if (b->extract_done) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    BMF_CUDA(ctx, cudaStreamIsCapturing(st, &cs));
    if (cs == cudaStreamCaptureStatusActive)
      BMF_CUDA(ctx, cudaEventRecordWithFlags(b->extract_done, st, cudaEventRecordExternal));
    else
      BMF_CUDA(ctx, cudaEventRecord(b->extract_done, st));
  }
  if (proc) {
    const int N = b->opts.mode == BMF_MODE_R ? 3 : 4;
    const StructuredAdj sa = batch_adj(b);
    k += launch_process(N, out->vcap, out->icap / N, b->d_totals, out->d_pos, out->d_nrm, b->d_boundary,
                        b->d_valence, b->d_idxg, b->opts.iters, b->opts.process_boundary, b->opts.smooth_normals,
                        b->ps, &sa, st);
    if (out->d_boundary)
      BMF_CUDA(ctx, cudaMemcpyAsync(out->d_boundary, b->d_boundary, (size_t)out->vcap, cudaMemcpyDeviceToDevice, st));
  }
  BMF_CUDA(ctx, cudaPeekAtLastError());
  *kernels = k;
  return BMF_OK;
}

bool same_out(const bmf_batch_out& a, const bmf_batch_out& b) {
  return a.d_pos == b.d_pos && a.d_nrm == b.d_nrm && a.d_boundary == b.d_boundary && a.d_idx == b.d_idx &&
         a.vcap == b.vcap && a.icap == b.icap && a.d_chunk_info == b.d_chunk_info;
}

}  // namespace

bmf_status bmf_batch_run(bmf_batch* b, bmf_batch_out* out, int32_t use_graph, int32_t sync, void* stream) {
  BMF_TRACE("bmf_batch_run");
  if (!b) return BMF_ERR_INVALID_ARGUMENT;
  bmf_ctx* ctx = b->ctx;
  if (!out || !out->d_pos || !out->d_idx || out->vcap < 0 || out->icap < 0)
    return fail(ctx, BMF_ERR_INVALID_ARGUMENT, "bmf_batch_run: output arena needs d_pos and d_idx");
  cudaStream_t st = (cudaStream_t)stream;
  bmf_status s;
  if (batch_keys(b) && (s = batch_proc_scratch(b, out->vcap, out->icap)) != BMF_OK) return s;
  if ((s = batch_list_scratch(b, out->vcap, out->icap)) != BMF_OK) return s;
  if (use_graph) {
    if (!b->exec || !same_out(b->graph_out, *out)) {
      if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
      }
      cudaStream_t cap;
      BMF_CUDA(ctx, cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
      cudaGraph_t g;
      BMF_CUDA(ctx, cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
      int64_t k = 0;
      s = batch_record(b, out, cap, &k);
      cudaError_t e = cudaStreamEndCapture(cap, &g);
      cudaStreamDestroy(cap);
      if (s != BMF_OK) return s;
      BMF_CUDA(ctx, e);
      e = cudaGraphInstantiate(&b->exec, g, 0);
      cudaGraphDestroy(g);
      BMF_CUDA(ctx, e);
      b->graph_out = *out;
      b->graph_kernels = k;
    }
    BMF_CUDA(ctx, cudaGraphLaunch(b->exec, st));
    ctx->launches += b->graph_kernels;
  } else {
    int64_t k = 0;
    if ((s = batch_record(b, out, st, &k)) != BMF_OK) return s;
    ctx->launches += k;
  }
  if (!b->run_done) BMF_CUDA(ctx, cudaEventCreateWithFlags(&b->run_done, cudaEventDisableTiming));
  BMF_CUDA(ctx, cudaEventRecord(b->run_done, st));
  b->ran = true;
  if (sync) {
    BMF_CUDA(ctx, cudaMemcpyAsync(b->h_pinned, b->d_totals, 2 * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    BMF_CUDA(ctx, cudaStreamSynchronize(st));
    out->n_verts = b->h_pinned[0];
    out->n_idx = b->h_pinned[1];
    if (out->n_verts > out->vcap || out->n_idx > out->icap)
      return fail(ctx, BMF_ERR_CAPACITY, "bmf_batch_run: output capacity exceeded (needed totals reported)");
  }
  return BMF_OK;
}

bmf_status bmf_batch_wait(bmf_batch* b, bmf_batch_out* out, int32_t timeout_ms) {
  BMF_TRACE("bmf_batch_wait");
  if (!b) return BMF_ERR_INVALID_ARGUMENT;
  bmf_ctx* ctx = b->ctx;
  if (!out || timeout_ms < 0) return fail(ctx, BMF_ERR_INVALID_ARGUMENT, "bmf_batch_wait: no output or timeout < 0");
  if (!b->ran) return fail(ctx, BMF_ERR_INVALID_ARGUMENT, "bmf_batch_wait: the plan has not run");
  const auto deadline = std::chrono::steady_clock::now() + std::chrono::milliseconds(timeout_ms);
  for (;;) {
    const cudaError_t e = cudaEventQuery(b->run_done);
    if (e == cudaSuccess) break;
    if (e != cudaErrorNotReady) return cuda_check(ctx, e, "bmf_batch_wait");
    if (std::chrono::steady_clock::now() >= deadline)
      return fail(ctx, BMF_ERR_TIMEOUT,
                  "bmf_batch_wait: the update is still running after " + std::to_string(timeout_ms) +
                      " ms (nothing was cancelled; wait again)");
    std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
  if (!b->aux) BMF_CUDA(ctx, cudaStreamCreateWithFlags(&b->aux, cudaStreamNonBlocking));
  BMF_CUDA(ctx, cudaMemcpyAsync(b->h_pinned, b->d_totals, 2 * sizeof(int64_t), cudaMemcpyDeviceToHost, b->aux));
  BMF_CUDA(ctx, cudaStreamSynchronize(b->aux));
  out->n_verts = b->h_pinned[0];
  out->n_idx = b->h_pinned[1];
  if (out->n_verts > out->vcap || out->n_idx > out->icap)
    return fail(ctx, BMF_ERR_CAPACITY, "bmf_batch_wait: output capacity exceeded (needed totals reported)");
  return BMF_OK;
}

bmf_status bmf_batch_wait_extraction(bmf_batch* b, void* stream) {
  BMF_TRACE("bmf_batch_wait_extraction");
  if (!b) return BMF_ERR_INVALID_ARGUMENT;
  bmf_ctx* ctx = b->ctx;
  if (b->extract_done) BMF_CUDA(ctx, cudaStreamWaitEvent((cudaStream_t)stream, b->extract_done, 0));
  return BMF_OK;
}

bmf_status bmf_batch_set_descs(bmf_batch* b, const bmf_chunk_desc* h_descs, int32_t n_chunks, void* stream) {
  BMF_TRACE("bmf_batch_set_descs");
  if (!b) return BMF_ERR_INVALID_ARGUMENT;
  bmf_ctx* ctx = b->ctx;
  if (!h_descs || n_chunks != b->n) return fail(ctx, BMF_ERR_INVALID_ARGUMENT, "bmf_batch_set_descs: count differs");
  for (int i = 0; i < n_chunks; ++i) {
    if (h_descs[i].dim != b->h_chunks[i].dim)
      return fail(ctx, BMF_ERR_INVALID_ARGUMENT, "bmf_batch_set_descs: a chunk's dim differs from the plan");
    if (!desc_ok(h_descs + i))
      return fail(ctx, BMF_ERR_INVALID_ARGUMENT,
                  "bmf_batch_set_descs: chunk " + std::to_string(i) + ": non-finite origin or bad scale");
  }
  cudaStream_t st = (cudaStream_t)stream;
  if (!b->h_stage) {
    BMF_CUDA(ctx, cudaMallocHost(&b->h_stage, sizeof(ChunkDev) * b->n));
    BMF_CUDA(ctx, cudaEventCreateWithFlags(&b->stage_done, cudaEventDisableTiming));
  } else {
    BMF_CUDA(ctx, cudaEventSynchronize(b->stage_done));
  }
  for (int i = 0; i < n_chunks; ++i) {
    ChunkDev c = b->h_chunks[i];
    c.ox = h_descs[i].origin[0];
    c.oy = h_descs[i].origin[1];
    c.oz = h_descs[i].origin[2];
    c.scale = h_descs[i].scale;
    b->h_chunks[i] = c;
    b->h_stage[i] = c;
  }
  BMF_CUDA(ctx, cudaMemcpyAsync(b->d_chunks, b->h_stage, sizeof(ChunkDev) * b->n, cudaMemcpyHostToDevice, st));
  BMF_CUDA(ctx, cudaEventRecord(b->stage_done, st));
  return BMF_OK;
}

bmf_status bmf_batch_profile(bmf_batch* b, bmf_batch_out* out, float* h_stage_ms, void* stream) {
  BMF_TRACE("bmf_batch_profile");
  if (!b || !h_stage_ms) return BMF_ERR_INVALID_ARGUMENT;
  bmf_ctx* ctx = b->ctx;
  if (!out || !out->d_pos || !out->d_idx) return fail(ctx, BMF_ERR_INVALID_ARGUMENT, "bmf_batch_profile: no output");
  cudaStream_t st = (cudaStream_t)stream;
  bmf_status s;
  const bool proc = b->opts.iters > 0;
  if (batch_keys(b) && (s = batch_proc_scratch(b, out->vcap, out->icap)) != BMF_OK) return s;
  if ((s = batch_list_scratch(b, out->vcap, out->icap)) != BMF_OK) return s;
  cudaEvent_t ev[8];
  for (auto& e : ev) BMF_CUDA(ctx, cudaEventCreate(&e));
  BMF_CUDA(ctx, cudaEventRecord(ev[0], st));
  BMF_CUDA(ctx, cudaMemsetAsync(b->d_flags, 0, sizeof(uint32_t) * b->n, st));
  batch_fill(b, st);
  BMF_CUDA(ctx, cudaEventRecord(ev[1], st));
  launch_count(b->opts.mode, b->d_chunks, b->n, b->d_units, b->n_units, b->d_words, b->d_flags, b->ws, st);
  BMF_CUDA(ctx, cudaEventRecord(ev[2], st));
  // the band fill's exact-density fix-up belongs to the fill stage
  const bool fixup = batch_band(b) && b->field.kind == BMF_FIELD_TERRAIN_FBM;
  if (fixup) launch_fill_fixup(b->d_chunks, b->ws, b->field, b->d_dens, st);
  BMF_CUDA(ctx, cudaEventRecord(ev[7], st));
  launch_scan_chunks(b->d_chunks, b->n, b->ws, b->d_tot, st, b->d_order);
  BMF_CUDA(ctx, cudaEventRecord(ev[3], st));
  launch_chunk_offsets(b->d_chunks, b->n, b->d_tot, b->d_flags, out->vcap, out->icap, out->d_chunk_info,
                       b->d_totals, st);
  BMF_CUDA(ctx, cudaEventRecord(ev[4], st));
  MeshOut mo{out->d_pos, out->d_nrm, proc ? b->d_boundary : out->d_boundary, proc ? b->d_valence : nullptr,
             out->d_idx, proc ? b->d_idxg : nullptr, out->vcap, out->icap, batch_keys(b) ? b->d_vkey : nullptr};
  const int ek = launch_emit(b->opts.mode, b->opts.placement, b->d_chunks, b->n, b->d_units, b->n_units, b->d_words,
                             b->d_dens, b->d_flags, b->ws, mo, b->d_totals, st);
  BMF_CUDA(ctx, cudaEventRecord(ev[5], st));
  int pk = 0;
  if (proc) {
    const int N = b->opts.mode == BMF_MODE_R ? 3 : 4;
    const StructuredAdj sa = batch_adj(b);
    pk = launch_process(N, out->vcap, out->icap / N, b->d_totals, out->d_pos, out->d_nrm, b->d_boundary,
                        b->d_valence, b->d_idxg, b->opts.iters, b->opts.process_boundary, b->opts.smooth_normals,
                        b->ps, &sa, st);
  }
  BMF_CUDA(ctx, cudaEventRecord(ev[6], st));
  BMF_CUDA(ctx, cudaEventSynchronize(ev[6]));
  BMF_CUDA(ctx, cudaPeekAtLastError());
  float fix = 0.0f;
  BMF_CUDA(ctx, cudaEventElapsedTime(&h_stage_ms[0], ev[0], ev[1]));
  BMF_CUDA(ctx, cudaEventElapsedTime(&fix, ev[2], ev[7]));
  h_stage_ms[0] += fix;
  BMF_CUDA(ctx, cudaEventElapsedTime(&h_stage_ms[1], ev[1], ev[2]));
  BMF_CUDA(ctx, cudaEventElapsedTime(&h_stage_ms[2], ev[7], ev[3]));
  for (int k = 3; k < 6; ++k) BMF_CUDA(ctx, cudaEventElapsedTime(&h_stage_ms[k], ev[k], ev[k + 1]));
  for (auto& e : ev) cudaEventDestroy(e);
  ctx->launches += (fixup ? 5 : 4) + (b->d_cols ? 1 : 0) + ek + pk;
  return BMF_OK;
}

bmf_status bmf_batch_format(bmf_batch* b, const bmf_batch_out* out, int32_t unwind, int32_t smooth_normals,
                            float* d_p, float* d_n, float* d_c, int64_t cap, void* stream) {
  BMF_TRACE("bmf_batch_format");
  if (!b) return BMF_ERR_INVALID_ARGUMENT;
  bmf_ctx* ctx = b->ctx;
  const int N = b->opts.mode == BMF_MODE_R ? 3 : 4;
  if (!out || !out->d_pos || !out->d_idx || !d_p || !d_n || !d_c || cap < 0 || (unwind && N != 4) ||
      (unwind && smooth_normals && !out->d_nrm))
    return fail(ctx, BMF_ERR_INVALID_ARGUMENT,
                "bmf_batch_format: output buffers required; unwinding needs quads (Mode Q) and, with "
                "smooth_normals, vertex normals");
  BMF_LAUNCHED(ctx, launch_format(b->d_chunks, b->n, out->vcap, out->icap, b->d_totals, out->d_pos, out->d_nrm,
                                  out->d_idx, unwind, smooth_normals, d_p, d_n, d_c, cap, (cudaStream_t)stream));
  BMF_CUDA(ctx, cudaPeekAtLastError());
  return BMF_OK;
}

bmf_status bmf_batch_get_tuning(const bmf_batch* b, bmf_batch_tuning* t) {
  if (!b || !t) return BMF_ERR_INVALID_ARGUMENT;
  std::memset(t, 0, sizeof(*t));
  t->fill_mode = b->fill_mode;
  t->fill_run = b->fill_run;
  t->sweep_block = b->ps.block > 0 ? b->ps.block : 256;
  t->fill_band = b->fill_band;
  return BMF_OK;
}

bmf_status bmf_batch_set_tuning(bmf_batch* b, const bmf_batch_tuning* t) {
  if (!b || !t) return BMF_ERR_INVALID_ARGUMENT;
  bmf_ctx* ctx = b->ctx;
  const bool terrain = b->field.kind == BMF_FIELD_TERRAIN_FBM;
  if (t->fill_mode < 0 || t->fill_mode > 2 || (!terrain && t->fill_mode != 0) ||
      (t->fill_run != 4 && t->fill_run != 8 && t->fill_run != 16) ||
      (t->sweep_block != 128 && t->sweep_block != 256 && t->sweep_block != 512) ||
      (t->fill_band != 0 && t->fill_band != 1) || (t->fill_band && !b->d_exact && !b->d_cols))
    return fail(ctx, BMF_ERR_INVALID_ARGUMENT,
                "bmf_batch_set_tuning: fill_mode 0..2 (1, 2 for terrain fields only), fill_run 4/8/16, "
                "sweep_block 128/256/512, fill_band 0/1 (1 for Mode R terrain and 2D heightmap plans only)");
  b->fill_mode = t->fill_mode;
  if (t->fill_run != b->fill_run || t->fill_band != b->fill_band) {
    b->fill_run = t->fill_run;
    b->fill_band = t->fill_band;
    if (terrain) b->fill_grid = fill_terrain_resident_ctas(b->fill_run, (int)b->field.p[5], b->fill_band != 0);
  }
  b->ps.block = t->sweep_block;
  if (b->exec) {
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
  return BMF_OK;
}

namespace {
float median_of(std::vector<float> v) {
  std::sort(v.begin(), v.end());
  return v.empty() ? 0.0f : v[v.size() / 2];
}
}  // namespace

bmf_status bmf_batch_autotune(bmf_batch* b, bmf_batch_out* out, int32_t reps, void* stream, bmf_batch_tuning* chosen,
                              float* h_ms, int32_t max_report, int32_t* n_report) {
  BMF_TRACE("bmf_batch_autotune");
  if (!b) return BMF_ERR_INVALID_ARGUMENT;
  bmf_ctx* ctx = b->ctx;
  if (!out || !out->d_pos || !out->d_idx || reps <= 0)
    return fail(ctx, BMF_ERR_INVALID_ARGUMENT, "bmf_batch_autotune: output arena and reps > 0 required");
  cudaStream_t st = (cudaStream_t)stream;
  bmf_status s;
  bmf_batch_tuning best;
  if ((s = bmf_batch_get_tuning(b, &best)) != BMF_OK) return s;
  std::vector<float> report;
  cudaEvent_t e0, e1;
  BMF_CUDA(ctx, cudaEventCreate(&e0));
  BMF_CUDA(ctx, cudaEventCreate(&e1));
  auto time_it = [&](auto&& enqueue, float* ms) -> bmf_status {
    std::vector<float> t;
    enqueue();  // warm-up
    for (int r = 0; r < reps; ++r) {
      BMF_CUDA(ctx, cudaEventRecord(e0, st));
      enqueue();
      BMF_CUDA(ctx, cudaEventRecord(e1, st));
      BMF_CUDA(ctx, cudaEventSynchronize(e1));
      BMF_CUDA(ctx, cudaPeekAtLastError());
      float v = 0.0f;
      BMF_CUDA(ctx, cudaEventElapsedTime(&v, e0, e1));
      t.push_back(v);
    }
    *ms = median_of(t);
    return BMF_OK;
  };
  // stage 1: density fill + labels
  if (b->field.kind == BMF_FIELD_TERRAIN_FBM) {
    const int cand[7][2] = {{0, 8}, {1, 4}, {1, 8}, {1, 16}, {2, 4}, {2, 8}, {2, 16}};
    float best_ms = 1e30f;
    for (const auto& c : cand) {
      bmf_batch_tuning t = best;
      t.fill_mode = c[0];
      t.fill_run = c[1];
      if ((s = bmf_batch_set_tuning(b, &t)) != BMF_OK) return s;
      float ms = 0.0f;
      s = time_it([&] {
        cudaMemsetAsync(b->d_flags, 0, sizeof(uint32_t) * b->n, st);
        batch_fill(b, st);
      }, &ms);
      if (s != BMF_OK) return s;
      report.push_back(ms);
      if (ms < best_ms) {
        best_ms = ms;
        best.fill_mode = c[0];
        best.fill_run = c[1];
      }
    }
    if ((s = bmf_batch_set_tuning(b, &best)) != BMF_OK) return s;
  }
  // stage 2: the sweeps, on the mesh of one real update
  if (b->opts.iters > 0) {
    if ((s = bmf_batch_run(b, out, 0, 1, stream)) != BMF_OK) return s;
    const int N = b->opts.mode == BMF_MODE_R ? 3 : 4;
    const StructuredAdj sa = batch_adj(b);
    const int blocks[3] = {128, 256, 512};
    float best_ms = 1e30f;
    for (int bs : blocks) {
      b->ps.block = bs;
      float ms = 0.0f;
      s = time_it([&] {
        launch_process(N, out->vcap, out->icap / N, b->d_totals, out->d_pos, out->d_nrm, b->d_boundary,
                       b->d_valence, b->d_idxg, b->opts.iters, b->opts.process_boundary, b->opts.smooth_normals,
                       b->ps, &sa, st);
      }, &ms);
      if (s != BMF_OK) return s;
      report.push_back(ms);
      if (ms < best_ms) {
        best_ms = ms;
        best.sweep_block = bs;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if ((s = bmf_batch_set_tuning(b, &best)) != BMF_OK) return s;
  // leave a correct update in `out`
  if ((s = bmf_batch_run(b, out, 0, 1, stream)) != BMF_OK) return s;
  if (chosen) *chosen = best;
  if (n_report) *n_report = (int32_t)report.size();
  if (h_ms)
    for (int i = 0; i < (int)report.size() && i < max_report; ++i) h_ms[i] = report[i];
  return BMF_OK;
}

// ---------------------------------------------------------------------------
// differentiable extraction (fitting)
// ---------------------------------------------------------------------------
}  // extern "C"

struct bmf_fit {
  bmf_ctx* ctx = nullptr;
  int n = 0, dim = 0, placement = 0, iters = 0, flags = 0;
  int64_t vcap = 0, icap = 0;
  ChunkDev* d_chunks = nullptr;
  int* d_units = nullptr;
  uint32_t *d_flags = nullptr, *d_tot = nullptr, *d_words = nullptr;
  int64_t* d_totals = nullptr;
  WordScratch ws{};
  ProcessScratch ps{};
  uint32_t *d_idxg = nullptr, *d_vkey = nullptr;
  uint8_t *d_valence = nullptr, *d_boundary = nullptr;
  float* d_g = nullptr;           // position-gradient work buffer
  int* d_order = nullptr;         // chunk order of the chunk-by-chunk sweeps (identity) and its queue
  int* d_pqueue = nullptr;
  uint32_t* d_qlist = nullptr;    // QEF-placed vertices of the forward, for the wide backward (+ counter at [vcap])
  float* d_qseed = nullptr;       // their FP32 eigenvectors (9 per entry), recorded by the forward
  uint8_t* d_qflag = nullptr;     // per vertex: took the QEF branch in the forward
  uint2* d_clist = nullptr;       // work list of active cells (+ counter after it)
  const float* last_density = nullptr;
  int64_t* h_pinned = nullptr;
  float* d_lpart = nullptr;       // per-block partial sums of bmf_fit_loss_spheres
};
constexpr int kFitLossPartials = 1024;

extern "C" {

bmf_status bmf_fit_destroy(bmf_fit* f) {
  if (!f) return BMF_ERR_INVALID_ARGUMENT;
  void* ptrs[] = {f->d_chunks, f->d_units, f->d_flags, f->d_tot, f->d_words, f->d_totals, f->ws.vcnt, f->ws.icnt,
                  f->ws.gpl, f->ps.off, f->ps.cursor, f->ps.adj, f->ps.dual_p, f->ps.dual_n, f->ps.tmp, f->d_idxg,
                  f->d_vkey, f->d_valence, f->d_boundary, f->d_g, f->d_qlist, f->d_qseed, f->d_clist, f->d_order,
                  f->d_pqueue, f->d_qflag, f->d_lpart};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (f->h_pinned) cudaFreeHost(f->h_pinned);
  delete f;
  return BMF_OK;
}

bmf_status bmf_fit_create(bmf_ctx* ctx, int32_t n_chunks, int32_t dim, int32_t placement, int32_t iters,
                          int64_t vcap, int64_t icap, int32_t flags, bmf_fit** out) {
  BMF_TRACE("bmf_fit_create");
  if (!ctx || !out) return BMF_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  if (n_chunks <= 0 || !dim_ok(dim) || (placement != BMF_PLACE_MASSPOINT && placement != BMF_PLACE_QEF) ||
      iters < 0 || vcap <= 0 || icap <= 0 || (flags & ~(BMF_FIT_ADJOINT_F64 | BMF_FIT_ADJOINT_DF)) ||
      (flags & BMF_FIT_ADJOINT_F64 && flags & BMF_FIT_ADJOINT_DF))
    return fail(ctx, BMF_ERR_INVALID_ARGUMENT,
                "bmf_fit_create: bad count, dim, placement, iters, capacity or flags");
  bmf_fit* f = new bmf_fit();
  f->ctx = ctx;
  f->n = n_chunks;
  f->dim = dim;
  f->placement = placement;
  f->iters = iters;
  f->flags = flags;
  f->vcap = vcap;
  f->icap = icap;
  const int zc = (dim + 31) / 32;
  const int64_t words = (int64_t)n_chunks * dim * dim * zc;
  std::vector<ChunkDev> hc(n_chunks);
  std::vector<int> units(n_chunks + 1);
  for (int i = 0; i < n_chunks; ++i) {
    ChunkDev c{};
    c.scale = 1.0f;
    c.dim = dim;
    c.zc = zc;
    c.dens = (int64_t)i * dim * dim * dim;
    c.words = (int64_t)i * dim * dim * zc;
    hc[i] = c;
    units[i] = i * dim;
  }
  units[n_chunks] = n_chunks * dim;
  const int64_t np = icap / 4;
  bool ok = cudaMalloc(&f->d_chunks, sizeof(ChunkDev) * n_chunks) == cudaSuccess &&
            cudaMalloc(&f->d_units, sizeof(int) * (n_chunks + 1)) == cudaSuccess &&
            cudaMalloc(&f->d_flags, sizeof(uint32_t) * n_chunks) == cudaSuccess &&
            cudaMalloc(&f->d_tot, sizeof(uint32_t) * 2 * n_chunks) == cudaSuccess &&
            cudaMalloc(&f->d_words, sizeof(uint32_t) * words) == cudaSuccess &&
            cudaMalloc(&f->d_totals, sizeof(int64_t) * 2) == cudaSuccess &&
            cudaMalloc(&f->ws.vcnt, sizeof(uint32_t) * words) == cudaSuccess &&
            cudaMalloc(&f->ws.icnt, sizeof(uint32_t) * words) == cudaSuccess &&
            cudaMalloc(&f->ws.gpl, sizeof(uint32_t) * 3 * words) == cudaSuccess &&
            cudaMalloc(&f->ps.off, sizeof(uint32_t) * (vcap + 1)) == cudaSuccess &&
            cudaMalloc(&f->ps.adj, sizeof(uint32_t) * (np * 4 + 1)) == cudaSuccess &&
            cudaMalloc(&f->ps.dual_p, sizeof(float) * (4 * np + 4)) == cudaSuccess &&
            cudaMalloc(&f->ps.tmp, sizeof(uint32_t) * (vcap / 4096 + 2)) == cudaSuccess &&
            cudaMalloc(&f->d_idxg, sizeof(uint32_t) * (icap + 1)) == cudaSuccess &&
            cudaMalloc(&f->d_vkey, sizeof(uint32_t) * (vcap + 1)) == cudaSuccess &&
            cudaMalloc(&f->d_valence, vcap + 1) == cudaSuccess && cudaMalloc(&f->d_boundary, vcap + 1) == cudaSuccess &&
            cudaMalloc(&f->d_g, sizeof(float) * 3 * (vcap + 1)) == cudaSuccess &&
            cudaMalloc(&f->d_qlist, sizeof(uint32_t) * (vcap + 1)) == cudaSuccess &&
            cudaMalloc(&f->d_order, sizeof(int) * n_chunks) == cudaSuccess &&
            cudaMalloc(&f->d_pqueue, sizeof(int)) == cudaSuccess &&
            (!(flags & (BMF_FIT_ADJOINT_F64 | BMF_FIT_ADJOINT_DF)) ||
             (cudaMalloc(&f->d_qseed, sizeof(float) * 9 * (vcap + 1)) == cudaSuccess &&
              cudaMalloc(&f->d_qflag, vcap + 1) == cudaSuccess)) &&
            cudaMalloc(&f->d_clist, sizeof(uint2) * (vcap + icap / 4 + 2)) == cudaSuccess &&
            cudaMalloc(&f->d_lpart, sizeof(float) * kFitLossPartials) == cudaSuccess &&
            cudaMallocHost(&f->h_pinned, sizeof(int64_t) * 4) == cudaSuccess &&
            cudaMemcpy(f->d_chunks, hc.data(), sizeof(ChunkDev) * n_chunks, cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMemcpy(f->d_units, units.data(), sizeof(int) * (n_chunks + 1), cudaMemcpyHostToDevice) == cudaSuccess;
  if (ok) {  // every chunk has the same size: the sweep queue takes them in index order
    std::vector<int> order(n_chunks);
    for (int i = 0; i < n_chunks; ++i) order[i] = i;
    ok = cudaMemcpy(f->d_order, order.data(), sizeof(int) * n_chunks, cudaMemcpyHostToDevice) == cudaSuccess;
  }
  if (!ok) {
    bmf_fit_destroy(f);
    return fail(ctx, BMF_ERR_OUT_OF_MEMORY, "bmf_fit_create: device allocation failed");
  }
  f->ws.clist = f->d_clist;
  f->ws.clist_cap = vcap + icap / 4 + 1;
  f->ws.ccount = (uint32_t*)(f->d_clist + f->ws.clist_cap);
  *out = f;
  return BMF_OK;
}

bmf_status bmf_fit_forward(bmf_fit* f, const float* d_density, float* d_pos, uint32_t* d_idx, int64_t* d_chunk_info,
                           int64_t* h_counts, void* stream) {
  BMF_TRACE("bmf_fit_forward");
  if (!f) return BMF_ERR_INVALID_ARGUMENT;
  bmf_ctx* ctx = f->ctx;
  if (!d_density || !d_pos || !d_idx) return fail(ctx, BMF_ERR_INVALID_ARGUMENT, "bmf_fit_forward: null buffer");
  cudaStream_t st = (cudaStream_t)stream;
  FieldDev fd{};
  fd.kind = BMF_FIELD_GRID;
  BMF_CUDA(ctx, cudaMemsetAsync(f->d_flags, 0, sizeof(uint32_t) * f->n, st));
  launch_sample_label(f->d_chunks, f->n, f->d_units, f->n * f->dim, f->dim, fd, d_density, nullptr, f->d_words,
                      f->d_flags, st);
  launch_count(BMF_MODE_Q, f->d_chunks, f->n, f->d_units, f->n * f->dim, f->d_words, f->d_flags, f->ws, st);
  launch_scan_chunks(f->d_chunks, f->n, f->ws, f->d_tot, st);
  launch_chunk_offsets(f->d_chunks, f->n, f->d_tot, f->d_flags, f->vcap, f->icap, d_chunk_info, f->d_totals, st);
  MeshOut mo{d_pos, nullptr, f->d_boundary, f->d_valence, d_idx, f->d_idxg, f->vcap, f->icap, f->d_vkey};
  if (f->d_qflag && f->placement == BMF_PLACE_QEF) {  // the wide adjoint reads the forward's QEF branches
    mo.qflag = f->d_qflag;
    mo.qlist = f->d_qlist;
    mo.qcount = f->d_qlist + f->vcap;
    mo.qseed = f->d_qseed;
  }
  int k = 4 + launch_emit(BMF_MODE_Q, f->placement, f->d_chunks, f->n, f->d_units, f->n * f->dim, f->d_words,
                          d_density, f->d_flags, f->ws, mo, f->d_totals, st);
  if (f->iters > 0) {
    StructuredAdj sa{BMF_MODE_Q, f->d_chunks, f->n, f->d_words, f->ws, f->d_vkey};
    if (f->n >= kChunkSweepMinChunks) {
      sa.tot = f->d_tot;
      sa.order = f->d_order;
      sa.queue = f->d_pqueue;
      sa.wide_adj = true;  // bmf_fit_backward's adjoint sweeps read it
    }
    k += launch_process(4, f->vcap, f->icap / 4, f->d_totals, d_pos, nullptr, f->d_boundary, f->d_valence, f->d_idxg,
                        f->iters, 0, 0, f->ps, &sa, st);
  }
  BMF_LAUNCHED(ctx, k);
  f->last_density = d_density;
  if (h_counts) {
    BMF_CUDA(ctx, cudaMemcpyAsync(f->h_pinned, f->d_totals, 2 * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    BMF_CUDA(ctx, cudaStreamSynchronize(st));
    h_counts[0] = f->h_pinned[0];
    h_counts[1] = f->h_pinned[1];
    if (h_counts[0] > f->vcap || h_counts[1] > f->icap)
      return fail(ctx, BMF_ERR_CAPACITY, "bmf_fit_forward: output capacity exceeded (needed totals reported)");
  }
  return BMF_OK;
}

bmf_status bmf_fit_loss_spheres(bmf_fit* f, const float* d_pos, const float* d_spheres, int32_t n_spheres,
                                float* d_loss, float* d_grad_pos, void* stream) {
  BMF_TRACE("bmf_fit_loss_spheres");
  if (!f) return BMF_ERR_INVALID_ARGUMENT;
  bmf_ctx* ctx = f->ctx;
  if (!d_pos || !d_spheres || n_spheres <= 0 || !d_loss || !d_grad_pos || !f->last_density || !f->d_lpart)
    return fail(ctx, BMF_ERR_INVALID_ARGUMENT, "bmf_fit_loss_spheres: null buffer, no spheres or no forward yet");
  BMF_LAUNCHED(ctx, launch_fit_loss_spheres(f->d_chunks, f->n, f->d_tot, f->d_totals, f->vcap, d_pos, d_spheres,
                                            n_spheres, d_grad_pos, f->d_lpart, kFitLossPartials, d_loss,
                                            (cudaStream_t)stream));
  BMF_CUDA(ctx, cudaPeekAtLastError());
  return BMF_OK;
}

bmf_status bmf_fit_adam(bmf_fit* f, float* d_param, const float* d_grad, float* d_m, float* d_v, int64_t n,
                        int32_t* d_step, float lr, float beta1, float beta2, float eps, void* stream) {
  BMF_TRACE("bmf_fit_adam");
  if (!f) return BMF_ERR_INVALID_ARGUMENT;
  bmf_ctx* ctx = f->ctx;
  if (!d_param || !d_grad || !d_m || !d_v || !d_step || n < 0 || !std::isfinite(lr) || !(beta1 >= 0.0f) ||
      !(beta1 < 1.0f) || !(beta2 >= 0.0f) || !(beta2 < 1.0f) || !(eps > 0.0f))
    return fail(ctx, BMF_ERR_INVALID_ARGUMENT, "bmf_fit_adam: null buffer, n < 0 or bad hyper-parameters");
  BMF_LAUNCHED(ctx, launch_adam(d_param, d_grad, d_m, d_v, n, d_step, lr, beta1, beta2, eps, (cudaStream_t)stream));
  BMF_CUDA(ctx, cudaPeekAtLastError());
  return BMF_OK;
}

bmf_status bmf_fit_backward(bmf_fit* f, const float* d_grad_pos, int64_t n_grad_verts, float* d_grad_density,
                            void* stream) {
  BMF_TRACE("bmf_fit_backward");
  if (!f) return BMF_ERR_INVALID_ARGUMENT;
  bmf_ctx* ctx = f->ctx;
  if (!d_grad_pos || !d_grad_density || !f->last_density || n_grad_verts < 0)
    return fail(ctx, BMF_ERR_INVALID_ARGUMENT, "bmf_fit_backward: null buffer or no forward yet");
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t ng = n_grad_verts < f->vcap ? n_grad_verts : f->vcap;
  BMF_CUDA(ctx, cudaMemsetAsync(f->d_g, 0, sizeof(float) * 3 * f->vcap, st));
  if (ng > 0)
    BMF_CUDA(ctx, cudaMemcpyAsync(f->d_g, d_grad_pos, sizeof(float) * 3 * ng, cudaMemcpyDeviceToDevice, st));
  // with enough chunks to fill the GPU the adjoint sweeps run chunk by chunk
  StructuredAdj sa{BMF_MODE_Q, f->d_chunks, f->n, f->d_words, f->ws, f->d_vkey};
  if (f->n >= kChunkSweepBwdMinChunks) {
    sa.tot = f->d_tot;
    sa.order = f->d_order;
    sa.queue = f->d_pqueue;
  }
  int k = launch_process_bwd(4, f->vcap, f->icap / 4, f->d_totals, f->d_boundary, f->d_valence, f->d_idxg, f->iters,
                             0, f->ps, f->d_g, &sa, st);
  BMF_CUDA(ctx, cudaMemsetAsync(d_grad_density, 0, sizeof(float) * (size_t)f->n * f->dim * f->dim * f->dim, st));
  const int wide = (f->flags & BMF_FIT_ADJOINT_F64) ? 1 : ((f->flags & BMF_FIT_ADJOINT_DF) ? 2 : 0);
  launch_place_bwd(f->placement, wide, f->d_chunks, f->n, f->d_words, f->last_density, f->d_vkey, f->d_totals,
                   f->vcap, f->d_g, d_grad_density, f->d_qlist, f->d_qlist + f->vcap, f->d_qseed, f->d_qflag, st);
  BMF_LAUNCHED(ctx, k + (wide && f->placement == BMF_PLACE_QEF ? 2 : 1));
  return BMF_OK;
}

bmf_status bmf_batch_destroy(bmf_batch* b) {
  if (!b) return BMF_ERR_INVALID_ARGUMENT;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  void* ptrs[] = {b->d_chunks, b->d_units, b->d_flags, b->d_tot, b->d_totals, b->d_dens, b->d_words,
                  b->ws.vcnt, b->ws.icnt, b->ws.gpl, b->ps.off, b->ps.cursor, b->ps.adj, b->ps.dual_p,
                  b->ps.dual_n, b->ps.tmp, b->d_idxg, b->d_valence, b->d_boundary, b->d_vkey,
                  b->d_fill_items, b->d_queue, b->d_order, b->d_pqueue, b->d_clist, b->d_exact, b->d_fix,
                  b->d_cols};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (b->h_pinned) cudaFreeHost(b->h_pinned);
  if (b->h_stage) cudaFreeHost(b->h_stage);
  if (b->stage_done) cudaEventDestroy(b->stage_done);
  if (b->run_done) cudaEventDestroy(b->run_done);
  if (b->extract_done) cudaEventDestroy(b->extract_done);
  if (b->aux) cudaStreamDestroy(b->aux);
  delete b;
  return BMF_OK;
}

}  // extern "C"
