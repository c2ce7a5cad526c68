/* CPU oracle for the chunk-extraction hot path of BinaryMeshFitting.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference's
 * algorithm, used by tests/, by __graft_entry__.smoke() and by bench.py's CPU
 * baseline leg as the checker.  The product (binarymeshfitting_gb300 and its
 * CUDA library) never links, imports or calls it.
 *
 * Each function cites the reference file:line it follows
 * (paths relative to the reference project root).  Build: oracle/Makefile
 * (gcc -ffp-contract=off, so every float operation is separately rounded and
 * results are identical on x86-64 and aarch64).
 *
 * Pinning: the mask, enumeration, vertex and triangle restatement is proven
 * bit-identical to the reference's own DMCChunk.cpp at dim = 32/64/128 (the
 * sizes its mask layout supports) by tests/test_oracle_pinned.py against
 * fixtures generated from the compiled reference (tests/golden/make_golden.py).
 * MeshProcessor is pinned the same way.  Noise (FBM) and Mode Q have no
 * counterpart in the reference's live code: they are specified here.
 */
#ifndef BMF_ORACLE_H
#define BMF_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- deterministic scalar math shared bit-for-bit with the CUDA kernels ---- */
float bmfo_sin(float x);
void bmfo_perm_init(uint64_t seed, uint8_t perm[256]);
float bmfo_perlin(const uint8_t perm[256], float x, float y, float z);
/* the same noise in textbook evaluation order (precision yardstick) */
float bmfo_perlin_textbook(const uint8_t perm[256], float x, float y, float z);
float bmfo_fbm(const uint8_t perm[256], float x, float y, float z, int octaves, float freq, float lacunarity,
               float gain);

/* BMF_FIELD_TERRAIN_2D pieces: the height noise of an (x, z) column and the
 * 2D gradient / value noises it is built from. */
float bmfo_terrain2d_height(const uint8_t perm[256], const float* params, float px, float pz);
float bmfo_noise2_grad(const uint8_t perm[256], int c, float x, float z);
float bmfo_noise2_value(const uint8_t perm[256], float x, float z);

/* ---- density fields (Sampler::block equivalents) ----
 * out[x*dim*dim + y*dim + z] = f(origin + (x,y,z)*scale), z fastest
 * (ImplicitSampler.hpp:14-36).  params: see bmf.h (BMF_FIELD_*). */
void bmfo_fill_field(int kind, const float* params, int dim, const float origin[3], float scale, float* out);

/* ---- DMCChunk::label_grid (DMCChunk.cpp:79-166) ----
 * words: dim*dim*ceil(dim/32) u32.  Returns contains_mesh. */
int bmfo_label_grid(int dim, const float* density, uint32_t* words);

/* ---- DMCChunk::label_edges mask passes (DMCChunk.cpp:168-438) ----
 * masks: dim*dim*(4*ceil(dim/32)) u64 words (8 cells per word, cell z at
 * byte z%8 of word z/8 of its row), i.e. one byte per cell with the row padded
 * to 32*ceil(dim/32) cells.  Equal to the reference layout when dim%32 == 0. */
void bmfo_cell_masks(int dim, const uint32_t* words, uint64_t* masks);

/* ---- Mode R: cell enumeration + calculate_cell + polygonize
 * (DMCChunk.cpp:440-498, 514-576, 593-674).  Buffers may be NULL to count
 * only.  Returns 0, or -1 when a capacity is exceeded.  cell_lin/cell_mask
 * list the surface cells in enumeration order. */
typedef struct {
  int64_t n_cells, n_verts, n_idx;
} bmfo_counts;
int bmfo_extract_r(int dim, const float* density, const uint64_t* masks, int64_t vcap, int64_t icap, int64_t ccap,
                   float* vpos, uint8_t* vboundary, uint8_t* vvalence, uint32_t* idx, uint32_t* cell_lin,
                   uint16_t* cell_mask, bmfo_counts* counts);

/* ---- Mode Q: DMC / manifold dual contouring quads (Tables.hpp:76-354 groups).
 * placement: 0 cell centre, 1 mass point of the group's crossings, 2 QEF on
 * hermite data with central-difference grid-gradient normals (FP32 restatement
 * of qef_simd with exact 1/sqrt), 3 the same QEF in FP64. */
int bmfo_extract_q(int dim, const float* density, const uint32_t* words, int placement, int64_t vcap, int64_t icap,
                   float* vpos, uint8_t* vboundary, uint8_t* vvalence, uint32_t* idx, bmfo_counts* counts);

/* ---- MeshProcessor<N> (MeshProcessor.cpp:26-306) in the order
 * ChunkGenerator::extract_chunk uses (ChunkGenerator.cpp:112-124).  pos and
 * nrm are updated in place (nrm holds the starting normals, usually 0). */
/* WorldOctree::split_leaves + chunk framing: rows (origin xyz, scale, dim,
 * level) in the reference's leaf order; returns the leaf count. */
int64_t bmfo_lod_generate(const float* prm, int min_level, int max_level, int dim, int boundary_processing,
                          int iters, float* out, int64_t cap);
/* GLChunk::format_data: per vertex (unwind 0) or unwound quads with one
 * normal each (unwind 1); returns the vertices written. */
int64_t bmfo_format(int64_t nverts, const float* pos, const float* nrm, int64_t nidx, const uint32_t* idx, int unwind,
                    int smooth_normals, float* p, float* n, float* c);
void bmfo_process(int N, int64_t nverts, float* pos, float* nrm, const uint8_t* vboundary, const uint8_t* vvalence,
                  int64_t nidx, const uint32_t* idx, int iters, int process_boundary, int smooth_normals);

/* ---- QEF (qef_simd.h:411-579) ---- */
float bmfo_qef_f32(const float* pos, const float* nrm, int count, float* out);
double bmfo_qef_f64(const double* pos, const double* nrm, int count, double* out);

/* Mode Q QEF placement (placement 2) of group `group` of cell (x, y, z) with
 * cell mask `mask`, in float as bmfo_extract_q places it; returns 1 when the
 * QEF solution was used, 0 for the mass-point fallback. */
int bmfo_place_q_f32(int dim, const float* density, int x, int y, int z, int mask, int group, float out[3]);

/* ---- FP64 differentiable path (oracle/bmf_oracle_fit.c): Mode Q + QEF
 * placement + `iters` position sweeps + mean squared rounded-box SDF.  box =
 * {centre xyz, half extents xyz, corner radius}.  grad_density (nullable,
 * dim^3) receives dL/d(density) with the discrete choices held fixed;
 * out_counts (nullable) = {vertices, quads, vertices placed by QEF};
 * state_hash (nullable) fingerprints those discrete choices; near_branch
 * (nullable, dim^3) flags the samples read by vertices whose branch (QEF or
 * mass point, truncation pattern) a float32 forward may take differently. */
double bmfo_fit_loss_f64(int dim, const double* density, int iters, const double* box, double* grad_density,
                         int64_t* out_counts, uint64_t* state_hash, unsigned char* near_branch);
/* The same with the loss' target a union of n_spheres spheres (rows of centre
 * xyz, radius); the state hash also covers each vertex's nearest sphere. */
double bmfo_fit_loss_spheres_f64(int dim, const double* density, int iters, const double* spheres, int n_spheres,
                                 double* grad_density, int64_t* out_counts, uint64_t* state_hash,
                                 unsigned char* near_branch);

/* ---- CPU baseline driver: the whole per-chunk path for a batch of chunks,
 * OpenMP over chunks like ChunkGenerator::extract_chunk.  desc: per chunk
 * {origin.x, origin.y, origin.z, scale, dim(as float)}.  Returns total
 * vertices; per-chunk counts written to out_counts (3 per chunk). */
int64_t bmfo_extract_batch(int n_chunks, const float* desc, int field, const float* params, int mode, int placement,
                           int iters, int smooth_normals, int64_t* out_counts, int n_threads);
/* The same with MeshProcessor's process_boundary and, per chunk, four digests
 * (bmfo_digest64 of the indices, positions, boundary flags and normals) in
 * out_digest[4 * i ..] (nullable), for chunk-by-chunk parity checks of a
 * whole update without keeping its meshes. */
int64_t bmfo_extract_batch_digest(int n_chunks, const float* desc, int field, const float* params, int mode,
                                  int placement, int iters, int process_boundary, int smooth_normals,
                                  int64_t* out_counts, uint64_t* out_digest, int n_threads);
uint64_t bmfo_digest64(const void* data, int64_t n_bytes, int f32_canon);

#ifdef __cplusplus
}
#endif
#endif
