// Stage 1 + 2: density filling (Sampler::block) fused with the binary grid
// (DMCChunk::label_grid, DMCChunk.cpp:113-162), and the packed cell masks
// (DMCChunk::label_edges mask passes, DMCChunk.cpp:202-438).
//
// Work unit = one x-plane of one chunk (dim*dim samples).  Threads map densely
// onto samples (z fastest), so no lane idles on the ragged last z-word of
// 33/65/129-sample lines; each warp ballots its 32 inside bits and ORs each
// word-aligned run of them into the plane's occupancy words in shared memory,
// which are then stored with coalesced 32-bit writes.
#include "bmf_device.cuh"
#include "bmf_internal.h"

namespace bmf {

// Chunk lookup: unit u belongs to the chunk c with unit_start[c] <= u < unit_start[c+1].
__device__ __forceinline__ int find_chunk(const int* __restrict__ unit_start, int n_chunks, int u) {
  int lo = 0, hi = n_chunks - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(unit_start + mid) <= u) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// flags bits: 1 = a word that is neither empty nor full, 2 = a full word,
// 4 = an empty word.  contains_mesh = (f & 1) || ((f & 6) == 6), the
// reference's mesh / negative / positive logic (DMCChunk.cpp:141-162).
__global__ void __launch_bounds__(256) k_sample_label(const ChunkDev* __restrict__ chunks, int n_chunks,
                                                      const int* __restrict__ unit_start, FieldDev field,
                                                      const float* __restrict__ dens_in, float* __restrict__ dens_out,
                                                      uint32_t* __restrict__ words, uint32_t* __restrict__ flags) {
  extern __shared__ uint32_t sw[];
  __shared__ int perm2[512];
  __shared__ uint2 gcode[512];
  const int u = blockIdx.x;
  const int c = find_chunk(unit_start, n_chunks, u);
  const ChunkDev ch = chunks[c];
  const int x = u - __ldg(unit_start + c);
  const int dim = ch.dim, zc = ch.zc;
  const int nw = dim * zc;
  for (int i = threadIdx.x; i < 512; i += blockDim.x) {
    perm2[i] = field.perm[i & 255];
    gcode[i] = grad_code(field.perm[i & 255]);
  }
  for (int i = threadIdx.x; i < nw; i += blockDim.x) sw[i] = 0u;
  __syncthreads();

  // Work item = a run of kRun consecutive z-samples of one (x, y) line; runs
  // start at multiples of kRun (which divides 32), so a run's inside bits land
  // in a single occupancy word.
  const int plane = dim * dim;
  const int nruns = (dim + kRun - 1) / kRun;
  const float px = ch.ox + (float)x * ch.scale;
  const int64_t dbase = ch.dens + (int64_t)x * plane;
  for (int item = threadIdx.x; item < dim * nruns; item += blockDim.x) {
    const int y = item / nruns;
    const int z0 = (item - y * nruns) * kRun;
    const int n = min(kRun, dim - z0);
    const int64_t o = dbase + (int64_t)y * dim + z0;
    float v[kRun];
    if (field.kind == BMF_FIELD_GRID) {
#pragma unroll
      for (int k = 0; k < kRun; ++k)
        if (k < n) v[k] = __ldg(dens_in + o + k);
    } else {
      const float py = ch.oy + (float)y * ch.scale;
      float pz[kRun];
#pragma unroll
      for (int k = 0; k < kRun; ++k) pz[k] = ch.oz + (float)(z0 + k) * ch.scale;
      if (field.kind == BMF_FIELD_TERRAIN_FBM) {
        terrain_run(field, perm2, gcode, px, py, pz, n, v);
      } else {
#pragma unroll
        for (int k = 0; k < kRun; ++k)
          if (k < n) v[k] = eval_field(field, perm2, px, py, pz[k]);
      }
      if (dens_out) {
#pragma unroll
        for (int k = 0; k < kRun; ++k)
          if (k < n) dens_out[o + k] = v[k];
      }
    }
    uint32_t bits = 0u;
#pragma unroll
    for (int k = 0; k < kRun; ++k)
      if (k < n && v[k] < 0.0f) bits |= 1u << k;
    if (bits) atomicOr(&sw[y * zc + (z0 >> 5)], bits << (z0 & 31));
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  uint32_t f = 0;
  uint32_t* wout = words + ch.words + (int64_t)x * nw;
  for (int i = threadIdx.x; i < nw; i += blockDim.x) {
    const uint32_t w = sw[i];
    wout[i] = w;
    f |= (w != 0u && w != kFull) ? 1u : (w == kFull ? 2u : 4u);
  }
  f |= __shfl_xor_sync(kFull, f, 16);
  f |= __shfl_xor_sync(kFull, f, 8);
  f |= __shfl_xor_sync(kFull, f, 4);
  f |= __shfl_xor_sync(kFull, f, 2);
  f |= __shfl_xor_sync(kFull, f, 1);
  if (lane == 0 && f) atomicOr(flags + c, f);
}

// One byte per cell, padded rows of 32*zc cells (bmf_cell_masks).
__global__ void k_cell_masks(int dim, int zc, const uint32_t* __restrict__ W, uint8_t* __restrict__ masks) {
  const int zp = 32 * zc;
  const int64_t n = (int64_t)dim * dim * zp;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int z = (int)(i % zp);
    const int64_t line = i / zp;
    const int y = (int)(line % dim), x = (int)(line / dim);
    masks[i] = (uint8_t)cell_mask_at(W, dim, zc, x, y, z);
  }
}

// contains_mesh flags from existing words (one CTA per chunk).
__global__ void k_word_flags(const ChunkDev* __restrict__ chunks, const uint32_t* __restrict__ words,
                             uint32_t* __restrict__ flags) {
  const ChunkDev ch = chunks[blockIdx.x];
  const int64_t n = (int64_t)ch.dim * ch.dim * ch.zc;
  uint32_t f = 0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    const uint32_t w = words[ch.words + i];
    f |= (w != 0u && w != kFull) ? 1u : (w == kFull ? 2u : 4u);
  }
  f = __reduce_or_sync(kFull, f);
  if ((threadIdx.x & 31) == 0 && f) atomicOr(flags + blockIdx.x, f);
}

void launch_word_flags(const ChunkDev* d_chunks, int n_chunks, const uint32_t* words, uint32_t* flags,
                       cudaStream_t st) {
  cudaMemsetAsync(flags, 0, sizeof(uint32_t) * n_chunks, st);
  k_word_flags<<<n_chunks, 256, 0, st>>>(d_chunks, words, flags);
}

void launch_sample_label(const ChunkDev* d_chunks, int n_chunks, const int* d_unit_start, int n_units, int max_dim,
                         const FieldDev& field, const float* dens_in, float* dens_out, uint32_t* words,
                         uint32_t* flags, cudaStream_t st) {
  const int max_zc = (max_dim + 31) / 32;
  const size_t smem = (size_t)max_dim * max_zc * sizeof(uint32_t);
  k_sample_label<<<n_units, 256, smem, st>>>(d_chunks, n_chunks, d_unit_start, field, dens_in, dens_out, words,
                                             flags);
}

void launch_cell_masks(int dim, const uint32_t* W, uint8_t* masks, cudaStream_t st) {
  const int zc = (dim + 31) / 32;
  const int64_t n = (int64_t)dim * dim * 32 * zc;
  const int blocks = (int)((n + 255) / 256 < 152 * 16 ? (n + 255) / 256 : 152 * 16);
  k_cell_masks<<<blocks, 256, 0, st>>>(dim, zc, W, masks);
}

}  // namespace bmf
