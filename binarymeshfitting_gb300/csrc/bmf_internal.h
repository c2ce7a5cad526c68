// Host-side declarations shared by the library's translation units.
#pragma once

#include "../../include/bmf.h"
#include <atomic>
#include <cstdint>
#include <cuda_runtime.h>

namespace bmf {

// A launch constant worked out once per device (an occupancy-sized grid, a
// shared-memory opt-in done).  Host threads may race on the first call: each
// computes the same value, and the atomic slot makes the publication well
// defined.  compute(dev) must return a non-zero value.
template <class F>
inline int per_device_once(std::atomic<int> (&slot)[64], F compute) {
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return compute(dev);
  int v = slot[dev].load(std::memory_order_acquire);
  if (v == 0) {
    v = compute(dev);
    slot[dev].store(v, std::memory_order_release);
  }
  return v;
}

struct ChunkDev;
struct FieldDev;

// Output arena for one launch of the emit kernels (single chunk or batch).
struct MeshOut {
  float* pos;
  float* nrm;
  uint8_t* boundary;
  uint8_t* valence;
  uint32_t* idx;          // chunk-local vertex ids (one VerticesIndicesBlock per chunk)
  uint32_t* idx_global;   // optional: the same indices offset by the chunk's vertex base
  int64_t vcap, icap;
  // optional: where each vertex came from, (chunk-local linear sample index << 2) | k,
  // k = crossing axis (Mode R) or vertex group (Mode Q); the key the analytic
  // adjacency build starts from.
  uint32_t* vkey = nullptr;
  // optional (QEF placement with keys): the record the QEF adjoint reads --
  // per vertex whether it took the QEF branch, the list of those vertices
  // (count in *qcount) and their FP32 eigenvectors (9 floats per entry)
  uint8_t* qflag = nullptr;
  uint32_t* qlist = nullptr;
  uint32_t* qcount = nullptr;
  float* qseed = nullptr;
};

// Per-word scratch of the extraction kernels, indexed like the occupancy
// words (chunk.words + (x*dim + y)*zc + zb).
struct WordScratch {
  uint32_t* vcnt;   // vertices hosted by the word's 32 cells; scanned in place to the chunk-local base
  uint32_t* icnt;   // indices emitted by the word's cells; scanned in place
  uint32_t* gpl;    // 3 bit-planes of the per-cell triangle (Mode R) / vertex-group (Mode Q) count
  // Work list (nullable), in no particular order; *ccount (zeroed before the
  // count kernel) entries, at most clist_cap kept.  Mode R: every busy word
  // (one whose cells own a crossing or emit triangles) as {chunk, word index
  // in the chunk}; Mode Q: every cell that holds vertex groups or owns an
  // interior crossing, as {chunk, vertex_key(x, y, z, 0)}.  Either way its size
  // bound is vcap + icap / prim_size + 1.
  uint2* clist;
  uint32_t* ccount;
  int64_t clist_cap;
  // Band fill (Mode R, nullable): its exactness mask, and the list of samples
  // the count kernel finds at an end of a crossing with an inexact density,
  // as {chunk, sample index in the chunk}; *fcount (zeroed before the count
  // kernel) entries, at most fix_cap kept.  A crossing has two ends, so the
  // list holds at most twice the vertex count (2 vcap + 1 suffices).
  const uint32_t* exact = nullptr;
  uint2* fix = nullptr;
  uint32_t* fcount = nullptr;
  int64_t fix_cap = 0;
  // The 2D heightmap's column fill (Mode R batches, nullable): no densities
  // are stored; the emit computes a crossing end's density from its (x, z)
  // column height (at chunk.words + x * dim + z) as the full fill does,
  // -(py * g) - n * height with py = chunk.oy + y * scale.
  const float* cols2d = nullptr;
  float c2d_g = 0.0f, c2d_height = 0.0f;
};

// Fill + label.  A terrain field of a single chunk goes through the line
// kernel (k_fill_terrain) directly; batches pass their own item queue to
// launch_fill_terrain.
// cols (nullable, BMF_FIELD_TERRAIN_2D): the (x, z) column heights from
// launch_columns2d, stored at chunk.words + x * dim + z (a chunk's dim^2
// columns fit its words' span); without it the x-plane CTAs evaluate them.
void launch_sample_label(const ChunkDev* d_chunks, int n_chunks, const int* d_unit_start, int n_units, int max_dim,
                         const FieldDev& field, const float* dens_in, float* dens_out, uint32_t* words,
                         uint32_t* flags, cudaStream_t st, const float* cols = nullptr);
// The 2D heightmap's column heights of a batch into cols (layout above), over
// items {chunk, first column} of columns2d_item() columns each.
void launch_columns2d(const ChunkDev* d_chunks, const int2* d_items, int n_items, const FieldDev& field, float* cols,
                      cudaStream_t st);
int columns2d_item();
// The 2D heightmap's occupancy words and contains_mesh flags from the column
// heights alone (the column fill: no densities).
void launch_words2d(const ChunkDev* d_chunks, int n_chunks, const int* d_unit_start, int n_units,
                    const FieldDev& field, const float* cols, uint32_t* words, uint32_t* flags, cudaStream_t st);
// Terrain FBM fill over line items {chunk, first line} (kFillLines lines
// each; d_items null = chunk 0's items in order).  d_queue non-null: grid
// persistent CTAs take items from the queue (reset here); else one CTA per item.
// run = z-samples per step (4, 8, 16 or 32).
// exact (nullable): the band fill's exactness mask (words layout); with it
// the fill may leave decided samples inexact (see k_fill_terrain<RUN, true>)
void launch_fill_terrain(int run, const ChunkDev* d_chunks, const int2* d_items, int n_items, int* d_queue,
                         int grid, const FieldDev& field, float* dens_out, uint32_t* words, uint32_t* flags,
                         uint32_t* exact, cudaStream_t st);
// the band fill applies to fields of the form (py - h) - a * FBM with a > 0,
// and (as the column fill: words and column heights, no densities) to the 2D
// heightmap
bool fill_band_supported(const FieldDev& field);
// The batched-fitting loss (sum over chunks of the mean squared sphere-union
// distance of the chunk's vertices) into *loss and its position gradient into
// grad (vcap * 3, zero past the vertex total); n_partial per-block partial sums.
int launch_fit_loss_spheres(const ChunkDev* d_chunks, int n_chunks, const uint32_t* d_tot, const int64_t* d_totals,
                            int64_t vcap, const float* pos, const float* spheres, int k, float* grad, float* partial,
                            int n_partial, float* loss, cudaStream_t st);
// Adam over n parameters with the step count on the device (advanced after)
int launch_adam(float* p, const float* g, float* m, float* v, int64_t n, int* step, float lr, float b1, float b2,
                float eps, cudaStream_t st);
// exact densities for the samples the count kernel listed in ws.fix (the
// inexact ends of crossings; after launch_count, before launch_emit)
void launch_fill_fixup(const ChunkDev* d_chunks, const WordScratch& ws, const FieldDev& field, float* dens,
                       cudaStream_t st);
int fill_terrain_items(int dim);          // items of one chunk
int fill_terrain_lines();                 // lines per item
int fill_terrain_resident_ctas(int run, int octaves, bool band);  // persistent grid: SMs x resident CTAs per SM
void launch_cell_masks(int dim, const uint32_t* W, uint8_t* masks, cudaStream_t st);
// contains_mesh flags of chunks whose words were produced elsewhere.
void launch_word_flags(const ChunkDev* d_chunks, int n_chunks, const uint32_t* words, uint32_t* flags,
                       cudaStream_t st);

// Extraction: count -> per-chunk scan -> (chunk offsets) -> emit.
void launch_count(int mode, const ChunkDev* d_chunks, int n_chunks, const int* d_unit_start, int n_units,
                  const uint32_t* words, const uint32_t* flags, WordScratch ws, cudaStream_t st);
// Scans each chunk's word counts; writes chunk totals (vertices, indices) to
// d_tot[2c].  d_order (optional): a permutation of the chunks, largest first.
void launch_scan_chunks(const ChunkDev* d_chunks, int n_chunks, WordScratch ws, uint32_t* d_tot, cudaStream_t st,
                        const int* d_order = nullptr);
// Exclusive scan of the chunk totals into chunk.vout / chunk.iout, and the
// per-chunk info table {voff, vcount, ioff, icount, contains_mesh, status}.
void launch_chunk_offsets(ChunkDev* d_chunks, int n_chunks, const uint32_t* d_tot, const uint32_t* flags,
                          int64_t vcap, int64_t icap, int64_t* d_info, int64_t* d_totals, cudaStream_t st);
// Returns the kernels launched: Mode Q QEF placement with vertex keys and
// d_counts (total vertices on the device) adds the per-vertex k_place_qef.
int launch_emit(int mode, int placement, const ChunkDev* d_chunks, int n_chunks, const int* d_unit_start,
                int n_units, const uint32_t* words, const float* dens, const uint32_t* flags, WordScratch ws,
                MeshOut out, const int64_t* d_counts, cudaStream_t st);

// MeshProcessor: operates on one flat mesh (vertices [0, nv), prims of N).
struct ProcessScratch {
  uint32_t* off;      // nv + 1 CSR offsets
  uint32_t* cursor;   // nv fill cursors
  uint32_t* adj;      // sum of valences
  float* dual_p;      // 3 * n_prims
  float* dual_n;      // 3 * n_prims
  uint32_t* tmp;      // scan scratch (block totals)
  int block;          // threads per CTA of the dual / primal sweeps (0 = 256)
};
// nv / n_prims size the grids; when d_counts is given the actual vertex and
// index counts are read from d_counts[0] / d_counts[1] on the device (so the
// sequence can be captured in a CUDA graph before the counts are known).
// Scratch sizes: off nv+1, cursor nv, adj N*n_prims, dual_p/dual_n 3*n_prims,
// tmp ceil(nv / 4096) + 1.
// Where the vertex->primitive lists come from: a mesh this library extracted
// (grid structure known: built analytically per vertex) or any mesh (atomic
// scatter + per-vertex sort).
struct StructuredAdj {
  int mode;                  // BMF_MODE_R / BMF_MODE_Q
  const ChunkDev* chunks;    // with vout / iout set
  int n_chunks;
  const uint32_t* words;
  WordScratch ws;            // scanned counts + per-word bit-planes
  const uint32_t* vkey;      // per-vertex keys written by the emit kernel
  // optional (all three or none): the sweeps run chunk by chunk, one CTA per
  // chunk, taking chunks from queue in the given order
  const uint32_t* tot = nullptr;  // per chunk {vertices, indices}
  const int* order = nullptr;     // chunk indices, largest first
  int* queue = nullptr;           // one int, reset by launch_process
  // the chunk-by-chunk sweeps keep 16-bit chunk-relative adjacency lists for
  // chunks of at most 65535 primitives unless a later pass reads the
  // adjacency (the fit's adjoint sweeps want 32-bit mesh-wide ids)
  bool wide_adj = false;
};
void launch_adj_build(int mode, const ChunkDev* d_chunks, int n_chunks, const uint32_t* words, WordScratch ws,
                      const uint32_t* vkey, const uint32_t* off, const int64_t* d_counts, int64_t vcap,
                      uint32_t* adj, cudaStream_t st);
// The chunk-by-chunk form of launch_process for StructuredAdj with tot /
// order / queue set: CSR offsets, adjacency and all sweeps in one launch.
void launch_sweep_chunks(const StructuredAdj& sa, int N, int64_t nv, int64_t n_prims, const int64_t* d_counts,
                         float* pos, float* nrm, const uint8_t* boundary, const uint8_t* valence,
                         const uint32_t* idx, int iters, int process_boundary, int smooth_normals,
                         const ProcessScratch& s, cudaStream_t st);
// Returns the number of kernels launched.
int launch_process(int N, int64_t nv, int64_t n_prims, const int64_t* d_counts, float* pos, float* nrm,
                   const uint8_t* boundary, const uint8_t* valence, const uint32_t* idx, int iters,
                   int process_boundary, int smooth_normals, ProcessScratch s, const StructuredAdj* sa,
                   cudaStream_t st);
// Device-side LOD descriptor generation (bmf_lod.cu).  cap <= kLodMaxLeaves.
constexpr int kLodMaxLeaves = 16384;
size_t lod_scratch_bytes(int cap);
int lod_generate(const bmf_lod_params& p, bmf_chunk_desc* d_descs, int cap, int32_t* d_count, void* scratch,
                 cudaStream_t st);
// GLChunk::format_data: per-vertex p/n/c (unwind 0) or unwound quads with
// one normal each (unwind 1); d_chunks non-null resolves chunk-local indices
// of a batch arena.  Returns the kernels launched.
int launch_format(const ChunkDev* d_chunks, int n_chunks, int64_t nv, int64_t ni, const int64_t* d_counts,
                  const float* pos, const float* nrm, const uint32_t* idx, int unwind, int smooth, float* p, float* n,
                  float* c, int64_t cap, cudaStream_t st);
// Adjoint of the position sweeps of launch_process (needs its CSR in s.off /
// s.adj; uses s.dual_p as scratch).  g holds dL/d(final positions) on entry and
// dL/d(initial positions) on return.  Returns the number of kernels launched.
int launch_process_bwd(int N, int64_t nv, int64_t n_prims, const int64_t* d_counts, const uint8_t* boundary,
                       const uint8_t* valence, const uint32_t* idx, int iters, int process_boundary,
                       const ProcessScratch& s, float* g, const StructuredAdj* sa, cudaStream_t st);
// Adjoint of Mode Q placement (placement 1 mass point, 2 QEF; f64: the QEF
// derivative from an FP64 re-solve); accumulates into grad_dens (the caller
// clears it).
// The wide list pass of launch_place_bwd (bmf_adjoint64.cu): wide 1 = FP64,
// 2 = double-float.
void launch_place_bwd_wide_list(int wide, const ChunkDev* d_chunks, int n_chunks, const uint32_t* words,
                                const float* dens, const uint32_t* vkey, const int64_t* d_counts, int64_t vcap,
                                const float* grad_pos, float* grad_dens, uint32_t* qlist, uint32_t* qcount,
                                float* qseed, cudaStream_t st);
// qlist (vcap entries) + qcount + qseed (9 floats per entry: the first pass's
// FP32 eigenvectors of the listed vertex): scratch of the two-pass wide form
// (nullable: one pass, idle lanes in the wide code).  wide: 0 FP32 adjoint, 1 the QEF
// derivative from an FP64 re-solve, 2 from a double-float re-solve.
void launch_place_bwd(int placement, int wide, const ChunkDev* d_chunks, int n_chunks, const uint32_t* words,
                      const float* dens, const uint32_t* vkey, const int64_t* d_counts, int64_t vcap,
                      const float* grad_pos, float* grad_dens, uint32_t* qlist, uint32_t* qcount, float* qseed,
                      const uint8_t* qflag, cudaStream_t st);
void launch_exclusive_scan_u8_to_u32(const uint8_t* in, uint32_t* out, int64_t n, const int64_t* d_n,
                                     uint32_t* block_tmp, cudaStream_t st);

}  // namespace bmf
