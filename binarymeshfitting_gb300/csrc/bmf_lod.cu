// Device-side chunk-descriptor generation: the WorldOctree split policy
// (WorldOctree::split_leaves / node_needs_split, WorldOctree.cpp:129-161,
// 237-247; children at MCDX/MCDY/MCDZ offsets, WorldOctree.cpp:177-199;
// Tables.hpp:7-9) evaluated level by level on the GPU, so a batched update's
// descriptor queue is produced where it is consumed.
//
// Level l: every frontier node either splits (its 8 children join the next
// frontier) or becomes a leaf.  The reference walks the tree depth first with
// a stack (children pushed 0..7, so popped 7..0); its leaf order is the
// descending order of the left-aligned path of push indices, which one CTA restores
// with a bitonic sort in shared memory before writing the descriptors
// (DMCChunk.cpp:94-97 frame, ChunkGenerator.cpp:98 overlap rule).
#include <cstdint>

#include "../../include/bmf.h"
#include "bmf_device.cuh"
#include "bmf_internal.h"

namespace bmf {

struct LodNode {
  float px, py, pz, size;
  int level;
  int pad;
  unsigned long long code;  // path of child push indices (3 bits per level) below a leading 1
};

constexpr int kLodMaxLevel = 20;  // 3 bits per level below the leading 1 of a 64-bit path

struct LodState {
  int count[kLodMaxLevel + 2];  // frontier size of each level
  int leaves;                   // leaves found
  int overflow;                 // a frontier or the leaf list exceeded the capacity
};

__device__ __forceinline__ bool lod_needs_split(const bmf_lod_params& p, const LodNode& n) {
  if (n.level >= p.max_level) return false;
  if (n.level < p.min_level) return true;
  // glm::distance(middle, focus) = length(focus - middle), middle = pos + size / 2
  const float mx = n.px + n.size * 0.5f, my = n.py + n.size * 0.5f, mz = n.pz + n.size * 0.5f;
  const float dx = p.focus[0] - mx, dy = p.focus[1] - my, dz = p.focus[2] - mz;
  const float d = sqrtf((dx * dx + dy * dy) + dz * dz);
  return d < (n.size * p.split_multiplier + p.size_modifier) + n.size * 0.5f;
}

__global__ void k_lod_root(bmf_lod_params p, LodNode* front, LodState* st) {
  LodNode r;
  r.px = p.root_pos[0];
  r.py = p.root_pos[1];
  r.pz = p.root_pos[2];
  r.size = p.root_size;
  r.level = 0;
  r.pad = 0;
  r.code = 1ull;
  front[0] = r;
  for (int l = 0; l < kLodMaxLevel + 2; ++l) st->count[l] = l == 0 ? 1 : 0;
  st->leaves = 0;
  st->overflow = 0;
}

// One level: the frontier of `level` -> the next level's frontier + leaves.
__global__ void k_lod_level(bmf_lod_params p, int level, const LodNode* __restrict__ in, LodNode* __restrict__ out,
                            LodNode* __restrict__ leaves, int cap, LodState* st) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= min(st->count[level], cap)) return;
  const LodNode n = in[i];
  if (!lod_needs_split(p, n)) {
    const int k = atomicAdd(&st->leaves, 1);
    if (k < cap) leaves[k] = n;
    else st->overflow = 1;
    return;
  }
  const int base = atomicAdd(&st->count[level + 1], 8);
  if (base + 8 > cap) {
    st->overflow = 1;
    return;
  }
  const float cs = n.size * 0.5f;
  const int dx[8] = {0, 1, 1, 0, 0, 1, 1, 0}, dy[8] = {0, 0, 0, 0, 1, 1, 1, 1}, dz[8] = {0, 0, 1, 1, 0, 0, 1, 1};
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    LodNode ch;
    ch.px = n.px + (float)dx[c] * cs;
    ch.py = n.py + (float)dy[c] * cs;
    ch.pz = n.pz + (float)dz[c] * cs;
    ch.size = n.size * 0.5f;
    ch.level = n.level + 1;
    ch.pad = 0;
    ch.code = (n.code << 3) | (unsigned long long)c;
    out[base + c] = ch;
  }
}

constexpr int kLodSortThreads = 1024;
static_assert(sizeof(LodState) <= 512, "LodState fits its scratch slot");

// Sorts the leaves by left-aligned push-index path, descending (= the
// reference's stack order), and writes their descriptors.
__global__ void __launch_bounds__(kLodSortThreads) k_lod_emit(bmf_lod_params p, const LodNode* __restrict__ leaves,
                                                              int cap, int n_pow2, const LodState* st,
                                                              bmf_chunk_desc* __restrict__ descs,
                                                              int32_t* __restrict__ d_count) {
  extern __shared__ unsigned long long s_key[];
  int* s_idx = (int*)(s_key + n_pow2);
  const int n = min(st->leaves, cap);
  const int depth_bits = 3 * p.max_level;
  for (int i = threadIdx.x; i < n_pow2; i += blockDim.x) {
    if (i < n) {
      const LodNode& l = leaves[i];
      s_key[i] = l.code << (depth_bits - 3 * l.level);
    } else {
      s_key[i] = 0ull;  // padding sorts last
    }
    s_idx[i] = i;
  }
  __syncthreads();
  for (int k = 2; k <= n_pow2; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < n_pow2; i += blockDim.x) {
        const int ij = i ^ j;
        if (ij > i) {
          const bool desc = (i & k) == 0;
          const unsigned long long a = s_key[i], b = s_key[ij];
          if (desc ? (a < b) : (a > b)) {
            s_key[i] = b;
            s_key[ij] = a;
            const int t = s_idx[i];
            s_idx[i] = s_idx[ij];
            s_idx[ij] = t;
          }
        }
      }
      __syncthreads();
    }
  }
  for (int r = threadIdx.x; r < n; r += blockDim.x) {
    const LodNode& l = leaves[s_idx[r]];
    // ChunkGenerator.cpp:98 overlap; DMCChunk.cpp:94-97 frame
    const float overlap = (l.level == p.max_level && (!p.boundary_processing || p.iters == 0))
                              ? 0.0f
                              : p.base_overlap + 0.005f * (float)p.iters;
    const float delta = l.size * (1.0f + overlap * 2.0f) / (float)(p.dim - 1);
    const float shift = l.size * overlap;
    bmf_chunk_desc d;
    d.origin[0] = l.px - shift;
    d.origin[1] = l.py - shift;
    d.origin[2] = l.pz - shift;
    d.scale = delta;
    d.dim = p.dim;
    d.level = l.level;
    descs[r] = d;
  }
  if (threadIdx.x == 0 && d_count) *d_count = st->overflow ? -1 : n;
}

size_t lod_scratch_bytes(int cap) { return 512 + 3 * sizeof(LodNode) * (size_t)cap + 256; }

int lod_generate(const bmf_lod_params& p, bmf_chunk_desc* d_descs, int cap, int32_t* d_count, void* scratch,
                 cudaStream_t st) {
  char* base = (char*)scratch;
  LodState* s = (LodState*)base;
  LodNode* f0 = (LodNode*)(base + 512);
  LodNode* f1 = f0 + cap;
  LodNode* leaves = f1 + cap;
  int n_pow2 = 1;
  while (n_pow2 < cap) n_pow2 <<= 1;
  k_lod_root<<<1, 1, 0, st>>>(p, f0, s);
  const int blocks = (cap + 255) / 256;
  for (int l = 0; l <= p.max_level; ++l) {
    const bool odd = l & 1;
    k_lod_level<<<blocks, 256, 0, st>>>(p, l, odd ? f1 : f0, odd ? f0 : f1, leaves, cap, s);
  }
  const size_t smem = (size_t)n_pow2 * (sizeof(unsigned long long) + sizeof(int));
  static std::atomic<int> attr_set[64] = {};  // the shared-memory opt-in, once per device
  per_device_once(attr_set, [](int) {
    cudaFuncSetAttribute(k_lod_emit, cudaFuncAttributeMaxDynamicSharedMemorySize, kLodMaxLeaves * 12);
    return 1;
  });
  k_lod_emit<<<1, kLodSortThreads, smem, st>>>(p, leaves, cap, n_pow2, s, d_descs, d_count);
  return p.max_level + 3;
}

}  // namespace bmf
