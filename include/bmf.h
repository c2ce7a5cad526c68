/* bmf.h -- C ABI of the GB300-native chunk-extraction library (libbmf_gb300.so).
 *
 * The reference (BinaryMeshFitting) has no C ABI: its extraction surface is the
 * C++ Sampler functor triple, DMCChunk's stage methods, MeshProcessor<N> and
 * ChunkGenerator::process_queue.  Each entry point below replaces one of
 * those, as cited beside it.  Conventions:
 *   - every call returns a bmf_status; bmf_last_error() gives a message;
 *   - pointers named d_* are device pointers owned by the caller; h_* are host
 *     pointers; nothing is freed across the ABI;
 *   - `stream` is a cudaStream_t (0 = the legacy default stream);
 *   - outputs carry counts, and a capacity overflow is reported as
 *     BMF_ERR_CAPACITY with the needed counts filled in (nothing is written
 *     out of bounds);
 *   - a context is not thread-safe: use one per host thread (the reference
 *     gives each OpenMP worker its own chunk, ChunkGenerator.cpp:91).
 *
 * Grid conventions (as in the reference): a chunk has dim samples per axis and
 * dim-1 cells per axis; sample (x,y,z) sits at index x*dim*dim + y*dim + z
 * (z fastest) and at world position origin + (x,y,z)*scale; positions in the
 * output mesh are in sample-index units (the reference's shader applies
 * world = p*scale + origin, shaders/main_vs.glsl:34).
 */
#ifndef BMF_H
#define BMF_H

#include <stddef.h>
#include <stdint.h>

#include "bmf_fields.h"

#if defined(__GNUC__)
#define BMF_API __attribute__((visibility("default")))
#else
#define BMF_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum bmf_status {
  BMF_OK = 0,
  BMF_ERR_INVALID_ARGUMENT = 1,
  BMF_ERR_CUDA = 2,
  BMF_ERR_CAPACITY = 3,      /* output capacity too small; needed counts reported */
  BMF_ERR_TIMEOUT = 4,       /* a bounded host-side wait gave up (bmf_batch_wait); nothing was cancelled */
  BMF_ERR_OUT_OF_MEMORY = 5,
  BMF_ERR_NOT_SUPPORTED = 6
} bmf_status;

typedef struct bmf_ctx bmf_ctx;

typedef struct bmf_config {
  int32_t device;          /* CUDA device ordinal */
  int32_t flags;           /* reserved, 0 */
  size_t scratch_bytes;    /* initial scratch arena size (0 = grow on demand) */
} bmf_config;

/* One density source: the Sampler plugin (Sampler.hpp:20-34). */
typedef struct bmf_field {
  int32_t kind;                          /* BMF_FIELD_* (bmf_fields.h) */
  float params[BMF_FIELD_MAX_PARAMS];
} bmf_field;

/* One chunk: DMCChunk's pos/overlap/scale after label_grid set them
 * (DMCChunk.cpp:94-98): origin = overlap_pos, scale = delta.  Every entry
 * point that samples a chunk rejects, with BMF_ERR_INVALID_ARGUMENT, a dim
 * out of range, a non-finite origin, and a scale that is not finite and > 0;
 * field params must be finite too. */
typedef struct bmf_chunk_desc {
  float origin[3];
  float scale;
  int32_t dim;             /* samples per axis, 2..1024 */
  int32_t level;           /* LOD level (informational) */
} bmf_chunk_desc;

/* Topology modes. */
#define BMF_MODE_R 0   /* reference: Marching-Cubes triangles on edge crossings (DMCChunk::polygonize) */
#define BMF_MODE_Q 1   /* dual marching cubes quads, one vertex per Tables::EdgeTable group */

/* Mode Q vertex placement. */
#define BMF_PLACE_CENTER 0
#define BMF_PLACE_MASSPOINT 1
#define BMF_PLACE_QEF 2       /* qef_simd.h solve on hermite data (grid-gradient normals) */

typedef struct bmf_extract_opts {
  int32_t mode;             /* BMF_MODE_* */
  int32_t placement;        /* BMF_PLACE_* (Mode Q) */
  int32_t iters;            /* MeshProcessor iterations (0 = none), WorldProperties::process_iters */
  int32_t process_boundary; /* WorldProperties::boundary_processing */
  int32_t smooth_normals;   /* MeshProcessor smooth_normals (SMOOTH_NORMALS) */
  int32_t reserved;
} bmf_extract_opts;

/* A chunk mesh in caller-owned device buffers (VerticesIndicesBlock,
 * ChunkBlocks.hpp:161-179, as structure-of-arrays). */
typedef struct bmf_mesh {
  float* d_pos;        /* vcap * 3 */
  float* d_nrm;        /* vcap * 3, may be NULL (then normals are not produced) */
  uint8_t* d_boundary; /* vcap, may be NULL */
  uint8_t* d_valence;  /* vcap, may be NULL (init_valence) */
  uint32_t* d_idx;     /* icap */
  int64_t vcap, icap;
  /* outputs */
  int64_t n_verts, n_idx;
  int32_t contains_mesh;
  int32_t prim_size;   /* 3 (Mode R) or 4 (Mode Q) */
} bmf_mesh;

/* ---- context ---- */
BMF_API bmf_status bmf_create(const bmf_config* cfg, bmf_ctx** out);
BMF_API bmf_status bmf_destroy(bmf_ctx* ctx);
BMF_API const char* bmf_status_string(bmf_status s);
BMF_API const char* bmf_last_error(const bmf_ctx* ctx);
/* Number of kernels this context has launched (instrumentation). */
BMF_API int64_t bmf_launch_count(const bmf_ctx* ctx);

/* ---- stage entry points (per chunk) ---- */

/* Sampler::block (Sampler.hpp:21; ImplicitSampler.hpp:14-36,
 * NoiseSampler.cpp:148-263): fill d_density[dim^3] for the chunk. */
BMF_API bmf_status bmf_sample_block(bmf_ctx* ctx, const bmf_chunk_desc* desc, const bmf_field* field, float* d_density,
                            void* stream);

/* DMCChunk::label_grid binarisation (DMCChunk.cpp:113-162): d_words gets
 * dim*dim*ceil(dim/32) occupancy words (bit z%32 of word [x][y][z/32] set
 * when density < 0); *h_contains_mesh (may be NULL) gets the reference's
 * contains_mesh flag (synchronises the stream when non-NULL). */
BMF_API bmf_status bmf_label_grid(bmf_ctx* ctx, int32_t dim, const float* d_density, uint32_t* d_words,
                          int32_t* h_contains_mesh, void* stream);

/* Fused Sampler::block + label_grid: density (d_density may be NULL when only
 * the occupancy words are wanted) and words in one pass. */
BMF_API bmf_status bmf_sample_label(bmf_ctx* ctx, const bmf_chunk_desc* desc, const bmf_field* field, float* d_density,
                            uint32_t* d_words, int32_t* h_contains_mesh, void* stream);

/* DMCChunk::label_edges mask passes (DMCChunk.cpp:202-438): one byte per cell,
 * d_masks[(x*dim + y)*zpad + z], zpad = 32*ceil(dim/32); bit (4dx+2dy+dz) set
 * when corner (x+dx,y+dy,z+dz) exists and is inside.  For dim % 32 == 0 this
 * is byte-for-byte the reference's uint64 MasksBlock. */
BMF_API bmf_status bmf_cell_masks(bmf_ctx* ctx, int32_t dim, const uint32_t* d_words, uint8_t* d_masks, void* stream);

/* DMCChunk::label_edges enumeration + polygonize (DMCChunk.cpp:440-576) for
 * Mode R, or the DMC quad emitter for Mode Q.  Synchronises the stream to
 * report counts in *out. */
BMF_API bmf_status bmf_polygonize(bmf_ctx* ctx, int32_t dim, const float* d_density, const uint32_t* d_words,
                          int32_t mode, int32_t placement, bmf_mesh* out, void* stream);

/* Largest chunk (samples per axis) bmf_polygonize_noalloc accepts. */
#define BMF_NOALLOC_MAX_DIM 129

/* bmf_polygonize for callers that cannot allocate device memory.  No
 * counterpart in the reference (its extraction always takes blocks from its
 * allocator pools).  Meant for hosts that own all device memory through their
 * own pool or may not block on the driver's allocator (engines, real-time
 * threads): it needs no bmf_ctx and calls no cudaMalloc / cudaFree; its
 * scratch is a fixed ~1.7 MB device array that every GPU loading the library
 * holds until exit.  dim > BMF_NOALLOC_MAX_DIM returns BMF_ERR_NOT_SUPPORTED.
 * All calls share that array: calls that overlap on the GPU race, so
 * serialise them.  The first call on a device resolves the array's address
 * for that device; with CUDA's lazy module loading (the default) that first
 * call is also when the driver loads the library's device code on that device
 * and places the array, which allocates device memory once.  A host that
 * forbids any allocation later makes that first call at start-up (and before
 * any stream capture).  Inputs, outputs and results are those of
 * bmf_polygonize, including BMF_ERR_CAPACITY with the needed counts when
 * vcap / icap are too small (nothing is written past them); synchronises the
 * stream. */
BMF_API bmf_status bmf_polygonize_noalloc(int32_t dim, const float* d_density, const uint32_t* d_words,
                                          int32_t mode, int32_t placement, bmf_mesh* out, void* stream);

/* MeshProcessor<N>::init/optimize_dual_grid/optimize_primal_grid/flush
 * (MeshProcessor.cpp:26-306) in the order ChunkGenerator::extract_chunk uses
 * (ChunkGenerator.cpp:112-124).  Updates d_pos (and d_nrm when non-NULL) in
 * place; N = mesh->prim_size. */
BMF_API bmf_status bmf_process(bmf_ctx* ctx, bmf_mesh* mesh, int32_t iters, int32_t process_boundary,
                       int32_t smooth_normals, void* stream);

/* ChunkGenerator::extract_chunk for one chunk (ChunkGenerator.cpp:98-124):
 * sample -> label -> polygonize -> process.  d_density_scratch may be NULL
 * (the context then uses its own scratch). */
BMF_API bmf_status bmf_extract_chunk(bmf_ctx* ctx, const bmf_chunk_desc* desc, const bmf_field* field,
                             const bmf_extract_opts* opts, bmf_mesh* out, void* stream);

/* ---- batched form: ChunkGenerator::process_queue (ChunkGenerator.hpp:23) ----
 * A plan owns the device descriptor queue and the scratch for one batch shape
 * and records the whole update as a CUDA graph. */
typedef struct bmf_batch bmf_batch;

typedef struct bmf_batch_out {
  float* d_pos;          /* vcap * 3 */
  float* d_nrm;          /* vcap * 3 or NULL */
  uint8_t* d_boundary;   /* vcap or NULL */
  uint32_t* d_idx;       /* icap; indices are chunk-local (as each VerticesIndicesBlock) */
  int64_t vcap, icap;
  /* d_chunk_info[6*i + k], k: 0 vertex offset, 1 vertex count, 2 index
   * offset, 3 index count, 4 contains_mesh, 5 status (0 ok, 3 capacity) */
  int64_t* d_chunk_info;
  /* outputs (host) */
  int64_t n_verts, n_idx;
} bmf_batch_out;

BMF_API bmf_status bmf_batch_create(bmf_ctx* ctx, const bmf_chunk_desc* h_descs, int32_t n_chunks, const bmf_field* field,
                            const bmf_extract_opts* opts, bmf_batch** out);
/* Runs the update.  use_graph != 0 replays the captured CUDA graph.
 * sync != 0 waits and fills out->n_verts / n_idx. */
BMF_API bmf_status bmf_batch_run(bmf_batch* b, bmf_batch_out* out, int32_t use_graph, int32_t sync, void* stream);
BMF_API bmf_status bmf_batch_destroy(bmf_batch* b);
/* Waits on the host, for at most timeout_ms milliseconds (0 = poll once), for
 * the plan's last bmf_batch_run to finish on the GPU -- typically one launched
 * with sync == 0 -- then fills out->n_verts / n_idx as a synchronous run does
 * (BMF_ERR_CAPACITY when they exceed the arena).  Returns BMF_ERR_TIMEOUT when
 * the update is still running at the deadline: nothing is cancelled, the call
 * may be repeated, and plan and context stay usable.  A host thread that must
 * not block (the reference's watcher thread, WorldWatcher.cpp) polls with 0.
 * No counterpart in the reference (its extraction is synchronous). */
BMF_API bmf_status bmf_batch_wait(bmf_batch* b, bmf_batch_out* out, int32_t timeout_ms);
/* Makes `stream` wait, on the device (no host sync), until the extraction of
 * the plan's last enqueued run is done: the indices and the chunk table are
 * final there while the smoothing sweeps still run, so a caller can start
 * copying or consuming the topology early (the positions, normals and boundary
 * flags are final only when the run is).  An event recorded inside the run
 * (inside its graph too); a plan that has not run yet makes this a no-op.
 * No counterpart in the reference (its extraction is synchronous). */
BMF_API bmf_status bmf_batch_wait_extraction(bmf_batch* b, void* stream);
/* Replaces the plan's chunk descriptors with those of the next update (same
 * count and the same dim per slot, e.g. the next frame of a streaming world):
 * an asynchronous pinned host->device copy on `stream`, so the captured graph
 * replays on the new chunks.  The caller's array may be reused on return. */
BMF_API bmf_status bmf_batch_set_descs(bmf_batch* b, const bmf_chunk_desc* h_descs, int32_t n_chunks, void* stream);
/* Runs one update stage by stage (no graph) with CUDA events between the
 * stages on `stream` and returns the stage times in ms:
 * h_stage_ms[0] fill+label, [1] count, [2] scan, [3] offsets, [4] emit,
 * [5] mesh processing. */
BMF_API bmf_status bmf_batch_profile(bmf_batch* b, bmf_batch_out* out, float* h_stage_ms, void* stream);

/* ---- device-side descriptor generation: the WorldOctree LOD split policy ----
 * WorldOctree::split_leaves / node_needs_split (WorldOctree.cpp:129-161,
 * 237-247) from a root cube: a node splits while level < min_level, or while
 * level < max_level and |focus - middle| < size * split_multiplier +
 * size_modifier + size / 2; the leaves become chunk descriptors in the
 * reference's leaf order (its depth-first stack order), framed as
 * DMCChunk::label_grid frames them (DMCChunk.cpp:94-97) with the overlap rule
 * of ChunkGenerator::extract_chunk (ChunkGenerator.cpp:98). */
typedef struct {
  float root_pos[3];      /* root corner; WorldOctree::init(s) uses size 2s at -s per axis */
  float root_size;
  float focus[3];
  float split_multiplier; /* WorldProperties (WorldOctree.cpp:21-33) */
  float size_modifier;
  int32_t min_level;
  int32_t max_level;      /* <= 20 */
  int32_t dim;            /* samples per chunk axis (chunk_resolution) */
  float base_overlap;     /* WorldProperties::overlap */
  int32_t boundary_processing;
  int32_t iters;
} bmf_lod_params;
/* Writes at most `cap` (<= 16384) descriptors to d_descs (device) and their
 * count to *d_count (device int; -1 when the tree has more leaves than cap).
 * Asynchronous on `stream` (graph-capturable). */
BMF_API bmf_status bmf_lod_generate(bmf_ctx* ctx, const bmf_lod_params* p, bmf_chunk_desc* d_descs, int32_t cap,
                                    int32_t* d_count, void* stream);

/* ---- draw layout: GLChunk::format_data (GLChunk.cpp:278-335), headless ----
 * Writes 3 floats each of position, normal and colour per output vertex into
 * d_p, d_n, d_c (device, at least `cap` vertices).  unwind == 0: one output
 * vertex per mesh vertex (normal 0 when the mesh has none); unwind == 1: the
 * quads (prim_size 4) unwound to 4 vertices each, all four with one normal:
 * smooth_normals ? the mean of the 4 vertex normals (needs d_nrm) : the flat
 * normal -normalize((m0 + m1) / 2) of the quad's two corner triangles.  The
 * colour is white, the vertex colour of this path (DMCChunk.cpp:681, averaged
 * by the sweeps).  *h_count (nullable) receives the vertices written. */
BMF_API bmf_status bmf_format(bmf_ctx* ctx, const bmf_mesh* mesh, int32_t unwind, int32_t smooth_normals, float* d_p,
                              float* d_n, float* d_c, int64_t cap, int64_t* h_count, void* stream);
/* The same over a batch arena after bmf_batch_run (chunk-local indices are
 * resolved through the plan's chunk table; output in arena order; counts
 * read on the device, so it can follow the run without a sync). */
BMF_API bmf_status bmf_batch_format(bmf_batch* b, const bmf_batch_out* out, int32_t unwind, int32_t smooth_normals,
                                    float* d_p, float* d_n, float* d_c, int64_t cap, void* stream);

/* ---- launch tuning of a batch plan (no counterpart in the reference) ----
 * The knobs that change only speed, never results. */
typedef struct {
  int32_t fill_mode;   /* terrain fill: 0 x-plane kernel, 1 one CTA per line item, 2 persistent CTAs taking
                          line items (largest chunks first) from a device work queue */
  int32_t fill_run;    /* line kernel tile height: z-samples per thread step, 4, 8 or 16 */
  int32_t sweep_block; /* threads per CTA of the dual / primal sweeps: 128, 256 or 512 */
  int32_t fill_band;   /* 1: band fill (Mode R terrain plans, fill_mode 1 or 2): a run stops evaluating octaves
                          once the bound on the remaining octaves fixes every sample's sign, and only the ends of
                          sign-changing edges get exact densities (the mesh reads no others); for Mode R plans of
                          BMF_FIELD_TERRAIN_2D the column fill: each (x, z) column height is evaluated once, the
                          occupancy words come from the heights, and the emit computes the densities it reads
                          from them (no density is stored); 0: every sample's density exact.  Both give
                          bit-identical meshes.  Default 1 where supported. */
  int32_t reserved[4];
} bmf_batch_tuning;
BMF_API bmf_status bmf_batch_get_tuning(const bmf_batch* b, bmf_batch_tuning* t);
/* Invalidates the captured graph (the next graph run captures again). */
BMF_API bmf_status bmf_batch_set_tuning(bmf_batch* b, const bmf_batch_tuning* t);
/* Autotuner: times every fill candidate (terrain fields) and every sweep block
 * size (iters > 0) on this plan and output arena, `reps` runs each (median of
 * CUDA-event times on `stream`), keeps the fastest of each stage and returns
 * the choice in *chosen (nullable).  h_ms (nullable) receives the median
 * times in candidate order (fill candidates, then sweep candidates), at most
 * max_report of them; *n_report (nullable) their count.  Synchronises; on
 * return `out` holds a correct update made with the chosen tuning. */
BMF_API bmf_status bmf_batch_autotune(bmf_batch* b, bmf_batch_out* out, int32_t reps, void* stream,
                                      bmf_batch_tuning* chosen, float* h_ms, int32_t max_report, int32_t* n_report);

/* ---- differentiable extraction (no counterpart in the reference) ----
 * With the topology fixed by the signs, Mode Q vertex placement (mass point or
 * QEF on hermite data with grid-gradient normals, qef_simd.h:411-461) and the
 * MeshProcessor<4> position sweeps (MeshProcessor.cpp:130-306) are smooth
 * functions of the density samples.  A fit plan runs them for n_chunks
 * learnable dim^3 grids packed back to back and gives the exact adjoint
 * (discrete choices -- topology, QEF truncation pattern, mass-point fallback --
 * held fixed).  Boundary vertices stay frozen, as in the reference. */
typedef struct bmf_fit bmf_fit;
/* flags of bmf_fit_create */
#define BMF_FIT_ADJOINT_F64 1 /* QEF adjoint from an FP64 re-solve of the hermite data and eigen pairs */
/* QEF adjoint from a double-float re-solve (pairs of floats, ~48-bit
 * significands; FP64's accuracy for this adjoint at a fraction of its cost on
 * GPUs with a reduced FP64 rate).  Exclusive with BMF_FIT_ADJOINT_F64. */
#define BMF_FIT_ADJOINT_DF 2
BMF_API bmf_status bmf_fit_create(bmf_ctx* ctx, int32_t n_chunks, int32_t dim, int32_t placement, int32_t iters,
                                  int64_t vcap, int64_t icap, int32_t flags, bmf_fit** out);
/* Positions (vcap*3) and chunk-local quad indices (icap) of all chunks, with
 * the per-chunk table of bmf_batch_out.  h_counts (nullable) gets the totals
 * {vertices, indices} (synchronises).  Keeps d_density's address for the
 * backward: do not change the density between forward and backward. */
BMF_API bmf_status bmf_fit_forward(bmf_fit* f, const float* d_density, float* d_pos, uint32_t* d_idx,
                                   int64_t* d_chunk_info, int64_t* h_counts, void* stream);
/* The loss of the batched-fitting workload on the device (no counterpart in
 * the reference): for each chunk, the mean over its output vertices of the
 * squared signed distance to the nearest of its n_spheres spheres
 * (|p - c| - r), summed over the chunks, into *d_loss (one float); and
 * dL/d(positions) into d_grad_pos (vcap * 3 floats, zero past the vertex
 * total).  d_pos holds the last forward's positions; d_spheres is n_chunks *
 * n_spheres rows {centre xyz, radius} (park unused rows far away).  Reads the
 * vertex totals on the device: with bmf_fit_forward(h_counts = NULL) and
 * bmf_fit_backward(n_grad_verts = vcap) a whole fitting step runs without a
 * host sync.  The sum is reduced in a fixed order (reproducible). */
BMF_API bmf_status bmf_fit_loss_spheres(bmf_fit* f, const float* d_pos, const float* d_spheres, int32_t n_spheres,
                                        float* d_loss, float* d_grad_pos, void* stream);
/* One Adam step (Kingma & Ba; torch.optim.Adam's arithmetic without weight
 * decay or amsgrad) over n learnable values, the optimizer of the batched
 * fitting workload (no counterpart in the reference): d_m / d_v are the
 * moment buffers (zero before the first step), *d_step the step count on the
 * device (0 before the first step; advanced by the call), so a CUDA graph that
 * replays the call advances it.  One pass over the four arrays. */
BMF_API bmf_status bmf_fit_adam(bmf_fit* f, float* d_param, const float* d_grad, float* d_m, float* d_v, int64_t n,
                                int32_t* d_step, float lr, float beta1, float beta2, float eps, void* stream);
/* dL/d(density) (n_chunks*dim^3, overwritten) from dL/d(positions) of the
 * last forward; d_grad_pos holds n_grad_verts * 3 floats. */
BMF_API bmf_status bmf_fit_backward(bmf_fit* f, const float* d_grad_pos, int64_t n_grad_verts, float* d_grad_density,
                                    void* stream);
BMF_API bmf_status bmf_fit_destroy(bmf_fit* f);

#ifdef __cplusplus
}
#endif
#endif
