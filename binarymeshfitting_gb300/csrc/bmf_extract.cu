// Stage 3 + 4: surface-cell enumeration, vertex / primitive compaction and
// emission (DMCChunk::label_edges enumeration + calculate_cell +
// calculate_isovertex + polygonize, DMCChunk.cpp:440-674), and the DMC quad
// emitter with mass-point / QEF placement (qef_simd.h).
//
// The reference numbers vertices in one sequential scan: cells in linear
// (x, y, z) order, and inside a cell its x-, y-, z-edge crossings
// (DMCChunk.cpp:449-474, 599-654).  Here every 32-bit occupancy word W[x][y][zb]
// stands for the 32 cells (x, y, 32zb..32zb+31), and the crossings those cells
// own are three bit words:
//     X = W[x][y] ^ W[x+1][y],  Y = W[x][y] ^ W[x][y+1],  Z = W ^ (W >> 1 | next << 31)
// so a word hosts popc(X)+popc(Y)+popc(Z) vertices, and the vertex id of cell z's
// axis-a crossing is   base(word) + popc((X|Y|Z bits of cells < z)) + (own earlier axes).
// base(word) is an exclusive scan of the per-word counts in (x, y, zb) order,
// which is exactly the reference's sequential order.  Triangles are counted
// and placed the same way, so vertex and index buffers come out bit-identical
// to the reference without any per-cell index volume (IndexesBlock) or cell
// list (DMC_CellsBlock).
#include "bmf_device.cuh"
#include "bmf_internal.h"

namespace bmf {

__device__ __forceinline__ int find_chunk_e(const int* __restrict__ unit_start, int n_chunks, int u) {
  int lo = 0, hi = n_chunks - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(unit_start + mid) <= u) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ bool contains_mesh(uint32_t f) { return (f & 1u) || ((f & 6u) == 6u); }

// EDGE_V offsets (DMCChunk.cpp:32, 543-565): edge e of a cell is the axis-a
// crossing owned by the cell at offset (ox, oy, oz).
static __constant__ int8_t c_edge_owner[12][4] = {{0, 0, 0, 0}, {0, 0, 1, 0}, {0, 1, 0, 0}, {0, 1, 1, 0},
                                                  {0, 0, 0, 1}, {0, 0, 1, 1}, {1, 0, 0, 1}, {1, 0, 1, 1},
                                                  {0, 0, 0, 2}, {0, 1, 0, 2}, {1, 0, 0, 2}, {1, 1, 0, 2}};

// Mask of cell (x, y, 32zb + lane) from the four line words around it and the
// four next-block words (for corner z + 1 of the block's last cell).
__device__ __forceinline__ int mask_from_lines(uint32_t w00, uint32_t w01, uint32_t w10, uint32_t w11, uint32_t n00,
                                               uint32_t n01, uint32_t n10, uint32_t n11, int lane) {
  const uint64_t q00 = ((uint64_t)n00 << 32) | w00, q01 = ((uint64_t)n01 << 32) | w01;
  const uint64_t q10 = ((uint64_t)n10 << 32) | w10, q11 = ((uint64_t)n11 << 32) | w11;
  return (int)(((q00 >> lane) & 3u) | (((q01 >> lane) & 3u) << 2) | (((q10 >> lane) & 3u) << 4) |
               (((q11 >> lane) & 3u) << 6));
}

struct LineWords {
  uint32_t w00, w01, w10, w11, n00, n01, n10, n11;
  __device__ __forceinline__ void load(const uint32_t* W, int dim, int zc, int x, int y, int zb) {
    w00 = word_at(W, dim, zc, x, y, zb);
    w01 = word_at(W, dim, zc, x, y + 1, zb);
    w10 = word_at(W, dim, zc, x + 1, y, zb);
    w11 = word_at(W, dim, zc, x + 1, y + 1, zb);
    n00 = word_at(W, dim, zc, x, y, zb + 1);
    n01 = word_at(W, dim, zc, x, y + 1, zb + 1);
    n10 = word_at(W, dim, zc, x + 1, y, zb + 1);
    n11 = word_at(W, dim, zc, x + 1, y + 1, zb + 1);
  }
  __device__ __forceinline__ int mask(int lane) const {
    return mask_from_lines(w00, w01, w10, w11, n00, n01, n10, n11, lane);
  }
};

constexpr int kWordBlock = 256;  // threads per CTA of the count / emit kernels

// The case tables staged in shared memory: per-lane lookups with different
// masks serialise on the constant cache, not on shared memory.
struct SmemTabs {
  uint64_t tri[256];
  uint64_t uses[256];
  uint64_t grp[256];
};
__device__ __forceinline__ void load_tabs(SmemTabs& t) {
  for (int i = threadIdx.x; i < 256; i += blockDim.x) {
    t.tri[i] = __ldg(g_tri_cases + i);
    t.uses[i] = __ldg(g_edge_uses + i);
    t.grp[i] = __ldg(g_group_cases + i);
  }
  __syncthreads();
}
__device__ __forceinline__ int tab_uses(const SmemTabs& t, int mask, int e) { return (int)((t.uses[mask] >> (4 * e)) & 0xF); }

// A word is quiet when its 32 cells can neither own a crossing nor have a
// mixed corner mask: the four line words around it are identical, so are the
// four next-block words, and the line has no z-crossing.  Then X = Y = Z = 0
// and every cell with all corners inside the chunk has mask 0 or 255, so the
// word contributes no vertex, triangle or quad in either mode.
__device__ __forceinline__ bool word_is_quiet(const uint32_t* W, int dim, int zc, int x, int y, int zb) {
  const uint32_t w = word_at(W, dim, zc, x, y, zb);
  if (word_at(W, dim, zc, x, y + 1, zb) != w || word_at(W, dim, zc, x + 1, y, zb) != w ||
      word_at(W, dim, zc, x + 1, y + 1, zb) != w)
    return false;
  const uint32_t n = word_at(W, dim, zc, x, y, zb + 1);
  if (word_at(W, dim, zc, x, y + 1, zb + 1) != n || word_at(W, dim, zc, x + 1, y, zb + 1) != n ||
      word_at(W, dim, zc, x + 1, y + 1, zb + 1) != n)
    return false;
  return zcross_word(W, dim, zc, x, y, zb) == 0u;
}

// Interior-edge test of Mode Q: the grid edge from sample s along axis a has
// all four surrounding cells.
__device__ __forceinline__ bool q_edge_interior(int dim, int sx, int sy, int sz, int a) {
  const int s[3] = {sx, sy, sz};
  const int b = (a + 1) % 3, c = (a + 2) % 3;
  return s[a] <= dim - 2 && s[b] >= 1 && s[b] <= dim - 2 && s[c] >= 1 && s[c] <= dim - 2;
}

// Interior crossing words of Mode Q (quads) for line (x, y) block zb.
__device__ __forceinline__ void q_quad_words(const uint32_t* W, int dim, int zc, int x, int y, int zb, uint32_t& Xi,
                                             uint32_t& Yi, uint32_t& Zi) {
  // z in [1, dim-2]
  uint32_t zint = kFull;
  const int lo = 1 - 32 * zb, hi = dim - 2 - 32 * zb;  // valid bit range [lo, hi]
  if (hi < 0 || lo > 31) zint = 0u;
  else {
    if (hi < 31) zint &= (2u << hi) - 1u;
    if (lo > 0) zint &= ~((1u << lo) - 1u);
  }
  Xi = (y >= 1 && y <= dim - 2) ? (xcross_word(W, dim, zc, x, y, zb) & zint) : 0u;
  Yi = (x >= 1 && x <= dim - 2) ? (ycross_word(W, dim, zc, x, y, zb) & zint) : 0u;
  Zi = (x >= 1 && x <= dim - 2 && y >= 1 && y <= dim - 2) ? zcross_word(W, dim, zc, x, y, zb) : 0u;
}

// ---------------------------------------------------------------------------
// K2: per-word counts
// ---------------------------------------------------------------------------
template <int MODE>
__global__ void __launch_bounds__(256) k_count(const ChunkDev* __restrict__ chunks, int n_chunks,
                                               const int* __restrict__ unit_start, const uint32_t* __restrict__ words,
                                               const uint32_t* __restrict__ flags, WordScratch ws) {
  const int u = blockIdx.x;
  const int c = find_chunk_e(unit_start, n_chunks, u);
  const ChunkDev ch = chunks[c];
  const int x = u - __ldg(unit_start + c);
  const int dim = ch.dim, zc = ch.zc, nw = dim * zc;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const uint32_t* W = words + ch.words;
  const bool cm = contains_mesh(__ldg(flags + c));
  __shared__ SmemTabs T;
  load_tabs(T);
  __shared__ int s_busy[kWordBlock];
  __shared__ int s_nbusy;
  __shared__ uint32_t s_act[kWordBlock];  // Mode R work list: active cells of each busy word
  __shared__ uint32_t s_apos[kWordBlock];
  __shared__ uint32_t s_acnt, s_abase;
  const bool listing = MODE == 0 && ws.clist != nullptr;
  for (int base = 0; base < nw; base += kWordBlock) {
    // level 1: one thread per word; quiet words get zero counts right away
    if (threadIdx.x == 0) {
      s_nbusy = 0;
      s_acnt = 0;
    }
    __syncthreads();
    if (base + (int)threadIdx.x < nw) {
      const int wi = base + threadIdx.x;
      const int y = wi / zc, zb = wi - y * zc;
      if (cm && !word_is_quiet(W, dim, zc, x, y, zb)) {
        s_busy[atomicAdd(&s_nbusy, 1)] = wi;
      } else {
        const int64_t o = ch.words + (int64_t)x * nw + wi;
        ws.vcnt[o] = 0u;
        ws.icnt[o] = 0u;
        if (ws.gpl) { ws.gpl[3 * o] = 0u; ws.gpl[3 * o + 1] = 0u; ws.gpl[3 * o + 2] = 0u; }
      }
    }
    __syncthreads();
    // level 2: one warp per busy word, one lane per cell
    const int nbusy = s_nbusy;
    for (int li = warp; li < nbusy; li += nwarps) {
    const int wi = s_busy[li];
    const int y = wi / zc, zb = wi - y * zc;
    const int64_t o = ch.words + (int64_t)x * nw + wi;
    const int z = 32 * zb + lane;
    LineWords lw;
    lw.load(W, dim, zc, x, y, zb);
    uint32_t vc, ic;
    if (MODE == 0) {
      const uint32_t X = (x + 1 < dim) ? (lw.w00 ^ lw.w10) : 0u;
      const uint32_t Y = (y + 1 < dim) ? (lw.w00 ^ lw.w01) : 0u;
      const uint32_t Z = zcross_word(W, dim, zc, x, y, zb);
      vc = __popc(X) + __popc(Y) + __popc(Z);
      const bool interior = x < dim - 1 && y < dim - 1 && z < dim - 1;
      const int nt = interior ? (int)(T.tri[lw.mask(lane)] >> 60) : 0;
      if (listing) {
        const uint32_t act = __ballot_sync(kFull, nt != 0 || (((X | Y | Z) >> lane) & 1u));
        if (lane == 0) {
          s_act[li] = act;
          s_apos[li] = act ? atomicAdd(&s_acnt, (uint32_t)__popc(act)) : 0u;
        }
      }
      int t = 3 * nt;
      // bit-planes of the per-cell triangle count (0..5): a cell's first
      // primitive is ibase + 3 * (popc(p0 & lt) + 2 popc(p1 & lt) + 4 popc(p2 & lt))
      const uint32_t p0 = __ballot_sync(kFull, nt & 1), p1 = __ballot_sync(kFull, nt & 2),
                     p2 = __ballot_sync(kFull, nt & 4);
      if (lane == 0 && ws.gpl) { ws.gpl[3 * o] = p0; ws.gpl[3 * o + 1] = p1; ws.gpl[3 * o + 2] = p2; }
      t += __shfl_xor_sync(kFull, t, 16);
      t += __shfl_xor_sync(kFull, t, 8);
      t += __shfl_xor_sync(kFull, t, 4);
      t += __shfl_xor_sync(kFull, t, 2);
      t += __shfl_xor_sync(kFull, t, 1);
      ic = (uint32_t)t;
    } else {
      const bool interior = x <= dim - 2 && y <= dim - 2 && z <= dim - 2;
      const int ng = interior ? (int)((T.grp[lw.mask(lane)] >> 48) & 0xF) : 0;
      const uint32_t g0 = __ballot_sync(kFull, ng & 1), g1 = __ballot_sync(kFull, ng & 2),
                     g2 = __ballot_sync(kFull, ng & 4);
      vc = __popc(g0) + 2 * __popc(g1) + 4 * __popc(g2);
      uint32_t Xi, Yi, Zi;
      q_quad_words(W, dim, zc, x, y, zb, Xi, Yi, Zi);
      ic = 4u * (__popc(Xi) + __popc(Yi) + __popc(Zi));
      if (lane == 0) { ws.gpl[3 * o] = g0; ws.gpl[3 * o + 1] = g1; ws.gpl[3 * o + 2] = g2; }
    }
    if (lane == 0) {
      ws.vcnt[o] = vc;
      ws.icnt[o] = ic;
    }
    }
    __syncthreads();
    if (listing) {
      // one global reservation per block of words, then each busy word's
      // active cells in lane order
      if (threadIdx.x == 0) s_abase = s_acnt ? atomicAdd(ws.ccount, s_acnt) : 0u;
      __syncthreads();
      for (int li = warp; li < nbusy; li += nwarps) {
        const uint32_t act = s_act[li];
        if (!((act >> lane) & 1u)) continue;
        const int wi = s_busy[li];
        const int y = wi / zc, zb = wi - y * zc;
        const int64_t slot = (int64_t)s_abase + s_apos[li] + __popc(act & lane_lt(lane));
        if (slot < ws.clist_cap)
          ws.clist[slot] = make_uint2((uint32_t)c, (uint32_t)(((int64_t)x * dim + y) * dim + 32 * zb + lane));
      }
      __syncthreads();
    }
  }
}

// ---------------------------------------------------------------------------
// K3: exclusive scan of each chunk's per-word counts (one CTA per chunk).
// ---------------------------------------------------------------------------
template <int NT>
__device__ __forceinline__ void block_excl_scan2(uint32_t& a, uint32_t& b, uint32_t& tot_a, uint32_t& tot_b) {
  __shared__ uint32_t sa[NT / 32], sb[NT / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t ia = a, ib = b;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t na = __shfl_up_sync(kFull, ia, o), nb = __shfl_up_sync(kFull, ib, o);
    if (lane >= o) { ia += na; ib += nb; }
  }
  if (lane == 31) { sa[warp] = ia; sb[warp] = ib; }
  __syncthreads();
  if (warp == 0) {
    uint32_t va = lane < NT / 32 ? sa[lane] : 0u, vb = lane < NT / 32 ? sb[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t na = __shfl_up_sync(kFull, va, o), nb = __shfl_up_sync(kFull, vb, o);
      if (lane >= o) { va += na; vb += nb; }
    }
    if (lane < NT / 32) { sa[lane] = va; sb[lane] = vb; }
  }
  __syncthreads();
  const uint32_t wa = warp ? sa[warp - 1] : 0u, wb = warp ? sb[warp - 1] : 0u;
  tot_a = sa[NT / 32 - 1];
  tot_b = sb[NT / 32 - 1];
  a = wa + ia - a;
  b = wb + ib - b;
  __syncthreads();
}

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;

__global__ void __launch_bounds__(kScanThreads) k_scan_chunks(const ChunkDev* __restrict__ chunks, WordScratch ws,
                                                            uint32_t* __restrict__ tot) {
  const ChunkDev ch = chunks[blockIdx.x];
  const int64_t n = (int64_t)ch.dim * ch.dim * ch.zc;
  uint32_t* v = ws.vcnt + ch.words;
  uint32_t* ic = ws.icnt + ch.words;
  uint32_t carry_v = 0, carry_i = 0;
  for (int64_t base = 0; base < n; base += (int64_t)kScanThreads * kScanItems) {
    const int64_t i0 = base + (int64_t)threadIdx.x * kScanItems;
    uint32_t lv[kScanItems], li[kScanItems], sv = 0, si = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
      lv[k] = (i0 + k < n) ? v[i0 + k] : 0u;
      li[k] = (i0 + k < n) ? ic[i0 + k] : 0u;
      sv += lv[k];
      si += li[k];
    }
    uint32_t ev = sv, ei = si, tv, ti;
    block_excl_scan2<kScanThreads>(ev, ei, tv, ti);
    ev += carry_v;
    ei += carry_i;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
      if (i0 + k < n) {
        v[i0 + k] = ev;
        ic[i0 + k] = ei;
      }
      ev += lv[k];
      ei += li[k];
    }
    carry_v += tv;
    carry_i += ti;
  }
  if (threadIdx.x == 0) {
    tot[2 * blockIdx.x] = carry_v;
    tot[2 * blockIdx.x + 1] = carry_i;
  }
}

// Chunk offsets in the output arena + per-chunk info (single CTA).
__global__ void __launch_bounds__(1024) k_chunk_offsets(ChunkDev* __restrict__ chunks, int n, const uint32_t* tot,
                                                        const uint32_t* flags, int64_t vcap, int64_t icap,
                                                        int64_t* info, int64_t* totals) {
  __shared__ int64_t s_v[1024], s_i[1024];
  int64_t carry_v = 0, carry_i = 0;
  for (int base = 0; base < n; base += 1024) {
    const int c = base + threadIdx.x;
    const int64_t v = c < n ? (int64_t)tot[2 * c] : 0, i = c < n ? (int64_t)tot[2 * c + 1] : 0;
    s_v[threadIdx.x] = v;
    s_i[threadIdx.x] = i;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
      const int64_t av = threadIdx.x >= o ? s_v[threadIdx.x - o] : 0, ai = threadIdx.x >= o ? s_i[threadIdx.x - o] : 0;
      __syncthreads();
      s_v[threadIdx.x] += av;
      s_i[threadIdx.x] += ai;
      __syncthreads();
    }
    if (c < n) {
      const int64_t vo = carry_v + s_v[threadIdx.x] - v, io = carry_i + s_i[threadIdx.x] - i;
      chunks[c].vout = vo;
      chunks[c].iout = io;
      if (info) {
        info[6 * c + 0] = vo;
        info[6 * c + 1] = v;
        info[6 * c + 2] = io;
        info[6 * c + 3] = i;
        info[6 * c + 4] = contains_mesh(flags[c]) ? 1 : 0;
        info[6 * c + 5] = (vo + v > vcap || io + i > icap) ? 3 : 0;
      }
    }
    carry_v += s_v[1023];
    carry_i += s_i[1023];
    __syncthreads();
  }
  if (threadIdx.x == 0 && totals) {
    totals[0] = carry_v;
    totals[1] = carry_i;
  }
}

// ---------------------------------------------------------------------------
// K4: emission
// ---------------------------------------------------------------------------

// Vertex id (chunk-local) of the axis-a crossing owned by sample (x, y, z).
__device__ __forceinline__ uint32_t r_vertex_id(const uint32_t* W, const uint32_t* vbase, int dim, int zc, int x, int y,
                                                int z, int a) {
  const int zb = z >> 5, l = z & 31;
  const uint32_t X = xcross_word(W, dim, zc, x, y, zb), Y = ycross_word(W, dim, zc, x, y, zb);
  const uint32_t Z = zcross_word(W, dim, zc, x, y, zb);
  const uint32_t lt = lane_lt(l);
  uint32_t id = __ldg(vbase + ((int64_t)x * dim + y) * zc + zb) + __popc(X & lt) + __popc(Y & lt) + __popc(Z & lt);
  if (a >= 1) id += (X >> l) & 1u;
  if (a >= 2) id += (Y >> l) & 1u;
  return id;
}

// Per-warp staging of a busy word's neighbourhood (Mode R emit): the
// occupancy words of lines (x-1+i, y-1+j), i, j in 0..3, for blocks zb-1, zb,
// zb+1, and the scanned vertex bases of lines (x+i, y+j), i, j in 0..1, for
// blocks zb, zb+1.  Every valence and every neighbour vertex id of the word's
// 32 cells is then computed from shared memory.
struct NbCache {
  uint32_t w[48];  // [i][j][b], b = block - (zb - 1)
  uint32_t vb[8];  // [i][j][b], b = block - zb
};

__device__ __forceinline__ void nb_load(NbCache& c, const uint32_t* W, const uint32_t* vbase, int dim, int zc, int x,
                                        int y, int zb, int lane) {
  __syncwarp();  // every lane is done with the previous word's cache
  for (int k = lane; k < 48; k += 32) {
    const int i = k / 12, j = (k / 3) & 3, b = k % 3;
    c.w[k] = word_at(W, dim, zc, x - 1 + i, y - 1 + j, zb - 1 + b);
  }
  if (lane < 8) {
    const int xx = x + (lane >> 2), yy = y + ((lane >> 1) & 1), bb = zb + (lane & 1);
    c.vb[lane] = (xx < dim && yy < dim && bb < zc) ? __ldg(vbase + ((int64_t)xx * dim + yy) * zc + bb) : 0u;
  }
  __syncwarp();
}

// Inside bit of sample (x-1+i, y-1+j, 32*(zb-1) + zr), zr in [0, 96).
__device__ __forceinline__ int nb_bit(const NbCache& c, int i, int j, int zr) {
  return (int)((c.w[(i * 4 + j) * 3 + (zr >> 5)] >> (zr & 31)) & 1u);
}

// Reference mask of cell (x-1+ci, y-1+cj, 32*(zb-1) + zr).
__device__ __forceinline__ int nb_mask(const NbCache& c, int ci, int cj, int zr) {
  int m = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) m |= nb_bit(c, ci + ((k >> 2) & 1), cj + ((k >> 1) & 1), zr + (k & 1)) << k;
  return m;
}

// r_vertex_id from the cache: the axis-a crossing owned by sample
// (x+i, y+j, zabs), i, j in {0, 1}, zabs in [32zb, 32zb+32].
__device__ __forceinline__ uint32_t nb_vertex_id(const NbCache& c, int dim, int x, int y, int zb, int i, int j,
                                                 int zabs, int a) {
  const int b = (zabs >> 5) - zb, l = zabs & 31;
  const uint32_t wc = c.w[((i + 1) * 4 + (j + 1)) * 3 + b + 1];
  const uint32_t X = (x + i + 1 < dim) ? wc ^ c.w[((i + 2) * 4 + (j + 1)) * 3 + b + 1] : 0u;
  const uint32_t Y = (y + j + 1 < dim) ? wc ^ c.w[((i + 1) * 4 + (j + 2)) * 3 + b + 1] : 0u;
  const uint32_t lt = lane_lt(l);
  uint32_t id = c.vb[i * 4 + j * 2 + b] + __popc(X & lt) + __popc(Y & lt);
  if (l > 0) {  // then b == 0 and the next block is cached
    uint32_t Z = wc ^ ((wc >> 1) | (c.w[((i + 1) * 4 + (j + 1)) * 3 + 2] << 31));
    const int valid = dim - 1 - 32 * zb;
    if (valid < 32) Z &= valid <= 0 ? 0u : ((1u << valid) - 1u);
    id += __popc(Z & lt);
  }
  if (a >= 1) id += (X >> l) & 1u;
  if (a >= 2) id += (Y >> l) & 1u;
  return id;
}

// Mode Q vertex base of cell (x, y, z).
__device__ __forceinline__ uint32_t q_vertex_base(const uint32_t* vbase, const uint32_t* gpl, int dim, int zc, int x,
                                                  int y, int z) {
  const int64_t wi = ((int64_t)x * dim + y) * zc + (z >> 5);
  const uint32_t lt = lane_lt(z & 31);
  return __ldg(vbase + wi) + __popc(__ldg(gpl + 3 * wi) & lt) + 2 * __popc(__ldg(gpl + 3 * wi + 1) & lt) +
         4 * __popc(__ldg(gpl + 3 * wi + 2) & lt);
}

__device__ __forceinline__ float dens_at(const float* D, int dim, int x, int y, int z) {
  return __ldg(D + ((int64_t)x * dim + y) * dim + z);
}

// Central-difference grid gradient, one-sided at the chunk faces.
__device__ __forceinline__ void grid_gradient(const float* D, int dim, int x, int y, int z, float g[3]) {
  const int c[3] = {x, y, z};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    int lo[3] = {x, y, z}, hi[3] = {x, y, z};
    float h = 0.5f;
    if (c[a] > 0) lo[a]--; else h = 1.0f;
    if (c[a] < dim - 1) hi[a]++; else h = 1.0f;
    g[a] = (dens_at(D, dim, hi[0], hi[1], hi[2]) - dens_at(D, dim, lo[0], lo[1], lo[2])) * h;
  }
}

// QEF solve, restating qef_simd.h:150-579 lane by lane in FP32 with the exact
// 1/sqrt in place of _mm_rsqrt_ps.
__device__ __forceinline__ float dot4(const float a[4], const float b[4]) {
  const float m0 = a[0] * b[0], m1 = a[1] * b[1], m2 = a[2] * b[2], m3 = a[3] * b[3];
  return (m0 + m1) + (m3 + m2);
}
__device__ __forceinline__ void vec_mul_m4(const float a[4], const float B[4][4], float out[4]) {
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    float r = a[0] * B[0][k];
    r = r + a[1] * B[1][k];
    r = r + a[2] * B[2][k];
    r = r + a[3] * B[3][k];
    out[k] = r;
  }
}

// What the QEF adjoint needs from a solve: the eigen decomposition the
// Jacobi sweeps produced, the kept reciprocals, the mass point and the
// centred right-hand side r = ATb - ATA * masspoint.
struct QefSolveInfo {
  float V[3][3];
  float sigma[3];
  float inv[3];
  float mp[3];
  float r[3];
};

struct QefAccum {
  float ata[4][4];
  float atb[4];
  float acc[4];
  int count;
  __device__ __forceinline__ void init() {
#pragma unroll
    for (int r = 0; r < 4; ++r) {
#pragma unroll
      for (int k = 0; k < 4; ++k) ata[r][k] = 0.0f;
      atb[r] = 0.0f;
      acc[r] = 0.0f;
    }
    count = 0;
  }
  // qef_simd_add, qef_simd.h:411-430
  __device__ __forceinline__ void add(const float pp[3], const float nn[3]) {
    const float p[4] = {pp[0], pp[1], pp[2], 1.0f};
    const float n[4] = {nn[0], nn[1], nn[2], 0.0f};
#pragma unroll
    for (int r = 0; r < 3; ++r) {
#pragma unroll
      for (int k = 0; k < 4; ++k) ata[r][k] = ata[r][k] + n[r] * n[k];
    }
    const float d = dot4(p, n);
    const float dd[4] = {d, d, d, 0.0f};
#pragma unroll
    for (int k = 0; k < 4; ++k) atb[k] = atb[k] + dd[k] * n[k];
#pragma unroll
    for (int k = 0; k < 4; ++k) acc[k] = acc[k] + p[k];
    ++count;
  }
  // qef_simd_solve + svd_solve_ATA_ATb (qef_simd.h:304-461); returns false
  // for fewer than 2 or more than 12 inputs (qef_simd.h:556-560).
  __device__ bool solve(float out[3], QefSolveInfo* info = nullptr) const {
    if (count < 2 || count > 12) {
      out[0] = out[1] = out[2] = 0.0f;
      return false;
    }
    float mp[4], pr[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) mp[k] = acc[k] / acc[3];
    vec_mul_m4(mp, ata, pr);
#pragma unroll
    for (int k = 0; k < 4; ++k) pr[k] = atb[k] - pr[k];
    float V[4][4] = {{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 0}};
    float vt[4][4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
#pragma unroll
      for (int k = 0; k < 4; ++k) vt[r][k] = ata[r][k];
    }
#pragma unroll 1
    for (int sweep = 0; sweep < 5; ++sweep) {
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        const int a = q == 2 ? 1 : 0, b = q == 0 ? 1 : 2;
        if (vt[a][b] != 0.0f) {
          // givens_coeffs_sym
          const float pp = vt[a][a], pq = vt[a][b], qq = vt[b][b];
          const float tau = (qq - pp) / (pq * 2.0f);
          const float stt = sqrtf(tau * tau + 1.0f);
          const float tn = 1.0f / ((tau >= 0.0f) ? (tau + stt) : (tau - stt));
          float cc = 1.0f / sqrtf(1.0f + tn * tn);
          float ss = tn * cc;
          if (pq == 0.0f) { cc = 1.0f; ss = 0.0f; }
          // rotateq_xy
          const float c2 = cc * cc, s2 = ss * ss;
          const float mx = ((2.0f * cc) * ss) * pq;
          const float nx = (c2 * pp - mx) + s2 * qq;
          const float ny = (s2 * pp + mx) + c2 * qq;
          vt[a][a] = nx;
          vt[b][b] = ny;
          // rotate_xy
          const float u3 = vt[0][3 - b], v3 = vt[1 - a][2];
#pragma unroll
          for (int r = 0; r < 3; ++r) {
            const float uu = V[r][a], vv = V[r][b];
            V[r][a] = cc * uu - ss * vv;
            V[r][b] = ss * uu + cc * vv;
          }
          vt[0][3 - b] = cc * u3 - ss * v3;
          vt[1 - a][2] = ss * u3 + cc * v3;
          vt[a][b] = 0.0f;
        }
      }
    }
    const float sigma[4] = {vt[0][0], vt[1][1], vt[2][2], 0.0f};
    float invdet[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {  // svd_invdet
      const float oo = 1.0f / sigma[k];
      const float a1 = fabsf(sigma[k]), a2 = fabsf(oo);
      const float mn = (a1 < a2) ? a1 : a2;
      invdet[k] = (mn >= 0.001f) ? oo : 0.0f;
    }
    float mm[3][4], o[4][4];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
#pragma unroll
      for (int k = 0; k < 4; ++k) mm[r][k] = V[r][k] * invdet[k];
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
#pragma unroll
      for (int k = 0; k < 4; ++k) o[r][k] = (r < 3 && k < 3) ? dot4(mm[k], V[r]) : 0.0f;
    }
    float xq[4];
    vec_mul_m4(pr, o, xq);
    out[0] = xq[0] + mp[0];
    out[1] = xq[1] + mp[1];
    out[2] = xq[2] + mp[2];
    if (info) {
#pragma unroll
      for (int r = 0; r < 3; ++r) {
#pragma unroll
        for (int k = 0; k < 3; ++k) info->V[r][k] = V[r][k];
        info->sigma[r] = sigma[r];
        info->inv[r] = invdet[r];
        info->mp[r] = mp[r];
        info->r[r] = pr[r];
      }
    }
    return true;
  }
};

// Crossing point (and hermite normal) of edge e of cell (x, y, z).
__device__ __forceinline__ void hermite(const float* D, int dim, int x, int y, int z, int e, bool want_n, float p[3],
                                        float n[3]) {
  const int ca = edge_c0(e), cb = edge_c1(e);
  const int a0[3] = {x + ((ca >> 2) & 1), y + ((ca >> 1) & 1), z + (ca & 1)};
  const int a1[3] = {x + ((cb >> 2) & 1), y + ((cb >> 1) & 1), z + (cb & 1)};
  const float s0 = dens_at(D, dim, a0[0], a0[1], a0[2]), s1 = dens_at(D, dim, a1[0], a1[1], a1[2]);
  const float mu = (0.0f - s0) / (s1 - s0);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float dv = ((float)a1[k] - (float)a0[k]) * mu;
    p[k] = dv + (float)a0[k];
  }
  if (want_n) {
    float g0[3], g1[3], g[3];
    grid_gradient(D, dim, a0[0], a0[1], a0[2], g0);
    grid_gradient(D, dim, a1[0], a1[1], a1[2], g1);
#pragma unroll
    for (int k = 0; k < 3; ++k) g[k] = g0[k] + (g1[k] - g0[k]) * mu;
    const float l2 = (g[0] * g[0] + g[1] * g[1]) + g[2] * g[2];
    const float inv = 1.0f / sqrtf(l2);
#pragma unroll
    for (int k = 0; k < 3; ++k) n[k] = g[k] * inv;
  }
}

template <int PLACE>
__device__ __forceinline__ void q_place(const float* D, int dim, int x, int y, int z, int mask, int g, float out[3]) {
  if (PLACE == 0) {
    out[0] = (float)x + 0.5f;
    out[1] = (float)y + 0.5f;
    out[2] = (float)z + 0.5f;
    return;
  }
  float mp[3] = {0.0f, 0.0f, 0.0f};
  int cnt = 0;
  QefAccum q;
  if (PLACE == 2) q.init();
  for (int e = 0; e < 12; ++e) {
    if (group_of(mask, e) != g) continue;
    float p[3], n[3];
    hermite(D, dim, x, y, z, e, PLACE == 2, p, n);
#pragma unroll
    for (int k = 0; k < 3; ++k) mp[k] = mp[k] + p[k];
    ++cnt;
    if (PLACE == 2) q.add(p, n);
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) mp[k] = mp[k] / (float)cnt;
  if (PLACE == 2) {
    float s[3];
    q.solve(s);
    const bool ok = s[0] >= (float)x && s[0] <= (float)(x + 1) && s[1] >= (float)y && s[1] <= (float)(y + 1) &&
                    s[2] >= (float)z && s[2] <= (float)(z + 1);
    if (ok) {
      out[0] = s[0]; out[1] = s[1]; out[2] = s[2];
      return;
    }
  }
  out[0] = mp[0]; out[1] = mp[1]; out[2] = mp[2];
}

template <int MODE, int PLACE>
__global__ void __launch_bounds__(256) k_emit(const ChunkDev* __restrict__ chunks, int n_chunks,
                                              const int* __restrict__ unit_start, const uint32_t* __restrict__ words,
                                              const float* __restrict__ dens, const uint32_t* __restrict__ flags,
                                              WordScratch ws, MeshOut out) {
  const int u = blockIdx.x;
  const int c = find_chunk_e(unit_start, n_chunks, u);
  if (!contains_mesh(__ldg(flags + c))) return;
  const ChunkDev ch = chunks[c];
  const int x = u - __ldg(unit_start + c);
  const int dim = ch.dim, zc = ch.zc, nw = dim * zc;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const uint32_t* W = words + ch.words;
  const uint32_t* vbase = ws.vcnt + ch.words;
  const uint32_t* ibase = ws.icnt + ch.words;
  const float* D = dens + ch.dens;
  const uint32_t lt = lane_lt(lane);
  __shared__ int s_busy[kWordBlock];
  __shared__ int s_nbusy;
  __shared__ NbCache s_nb[kWordBlock / 32];
  for (int base = 0; base < nw; base += kWordBlock) {
    // level 1: one thread per word; quiet words emit nothing
    if (threadIdx.x == 0) s_nbusy = 0;
    __syncthreads();
    if (base + (int)threadIdx.x < nw) {
      const int wi = base + threadIdx.x;
      const int y = wi / zc, zb = wi - y * zc;
      if (!word_is_quiet(W, dim, zc, x, y, zb)) s_busy[atomicAdd(&s_nbusy, 1)] = wi;
    }
    __syncthreads();
    // level 2: one warp per busy word, one lane per cell
    const int nbusy = s_nbusy;
    for (int li = warp; li < nbusy; li += nwarps) {
    const int wi = s_busy[li];
    const int y = wi / zc, zb = wi - y * zc;
    const int z = 32 * zb + lane;
    const int64_t wo = (int64_t)x * nw + wi;
    LineWords lw;
    lw.load(W, dim, zc, x, y, zb);
    if (MODE == 0) {
      NbCache& nb = s_nb[warp];
      nb_load(nb, W, vbase, dim, zc, x, y, zb, lane);
      // ---- vertices: calculate_cell / calculate_isovertex order ----
      const uint32_t X = (x + 1 < dim) ? (lw.w00 ^ lw.w10) : 0u;
      const uint32_t Y = (y + 1 < dim) ? (lw.w00 ^ lw.w01) : 0u;
      const uint32_t Z = zcross_word(W, dim, zc, x, y, zb);
      if ((X | Y | Z) != 0u) {
        uint32_t vid = __ldg(vbase + wo) + __popc(X & lt) + __popc(Y & lt) + __popc(Z & lt);
        const uint32_t own = ((X >> lane) & 1u) | (((Y >> lane) & 1u) << 1) | (((Z >> lane) & 1u) << 2);
        for (int a = 0; a < 3; ++a) {
          if (!((own >> a) & 1u)) continue;
          const int x1 = x + (a == 0), y1 = y + (a == 1), z1 = z + (a == 2);
          const int64_t gv = ch.vout + vid;
          ++vid;
          if (gv >= out.vcap) continue;
          const float s0 = dens_at(D, dim, x, y, z), s1 = dens_at(D, dim, x1, y1, z1);
          const float mu = (0.0f - s0) / (s1 - s0);
          const float q0[3] = {(float)x, (float)y, (float)z};
          const float dl[3] = {(float)(x1 - x), (float)(y1 - y), (float)(z1 - z)};
          float* P = out.pos + 3 * gv;
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            const float dv = dl[k] * mu;
            P[k] = dv + q0[k];
          }
          if (out.boundary)
            out.boundary[gv] = (x == 0 || y == 0 || z == 0 || x == dim - 1 || y == dim - 1 || z == dim - 1 ||
                                x1 == dim - 1 || y1 == dim - 1 || z1 == dim - 1);
          if (out.nrm) { out.nrm[3 * gv] = 0.0f; out.nrm[3 * gv + 1] = 0.0f; out.nrm[3 * gv + 2] = 0.0f; }
          if (out.vkey) out.vkey[gv] = ((uint32_t)(((int64_t)x * dim + y) * dim + z) << 2) | (uint32_t)a;
          if (out.valence) {
            // init_valence: uses of this edge by the (up to) four interior
            // cells around it (polygonize skips far-face cells, DMCChunk.cpp:528).
            int val = 0;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              const int d1 = k >> 1, d2 = k & 1;
              int cx = x, cy = y, cz = z, e;
              if (a == 0) { cy -= d1; cz -= d2; e = 2 * d1 + d2; }
              else if (a == 1) { cx -= d1; cz -= d2; e = 4 + 2 * d1 + d2; }
              else { cx -= d1; cy -= d2; e = 8 + 2 * d1 + d2; }
              if (cx < 0 || cy < 0 || cz < 0 || cx > dim - 2 || cy > dim - 2 || cz > dim - 2) continue;
              val += edge_uses(nb_mask(nb, cx - x + 1, cy - y + 1, cz - 32 * (zb - 1)), e);
            }
            out.valence[gv] = (uint8_t)val;
          }
        }
      }
      // ---- triangles: polygonize_cell order ----
      const bool interior = x < dim - 1 && y < dim - 1 && z < dim - 1;
      const int mask = interior ? lw.mask(lane) : 0;
      const uint64_t tw = c_tri_cases[mask];
      const int t3 = 3 * (int)(tw >> 60);
      if (__ballot_sync(kFull, t3 != 0) == 0u) continue;
      const int incl = warp_incl_scan(t3);
      int64_t gi = ch.iout + (int64_t)__ldg(ibase + wo) + (incl - t3);
      for (int i = 0; i < t3; ++i, ++gi) {
        const int e = tri_edge(tw, i);
        const uint32_t vid = nb_vertex_id(nb, dim, x, y, zb, c_edge_owner[e][0], c_edge_owner[e][1],
                                          z + c_edge_owner[e][2], c_edge_owner[e][3]);
        if (gi < out.icap) {
          out.idx[gi] = vid;
          if (out.idx_global) out.idx_global[gi] = (uint32_t)(ch.vout + vid);
        }
      }
    } else {
      // ---- Mode Q vertices: one per vertex group of each interior surface cell ----
      const bool interior = x <= dim - 2 && y <= dim - 2 && z <= dim - 2;
      const int mask = interior ? lw.mask(lane) : 0;
      const int ng = group_count(mask);
      const int64_t gpo = 3 * (ch.words + wo);
      if (ng) {
        uint32_t vid = __ldg(vbase + wo) + __popc(__ldg(ws.gpl + gpo) & lt) +
                       2 * __popc(__ldg(ws.gpl + gpo + 1) & lt) + 4 * __popc(__ldg(ws.gpl + gpo + 2) & lt);
        const int nc = dim - 1;
        const uint8_t bnd = (x == 0 || y == 0 || z == 0 || x == nc - 1 || y == nc - 1 || z == nc - 1);
        for (int g = 0; g < ng; ++g, ++vid) {
          const int64_t gv = ch.vout + vid;
          if (gv >= out.vcap) continue;
          // QEF positions come from k_place_qef (thread per vertex) when the
          // vertex keys are kept; only here on the few lanes of surface cells
          // otherwise
          if (PLACE != 2 || !out.vkey) {
            float P[3];
            q_place<PLACE>(D, dim, x, y, z, mask, g, P);
            out.pos[3 * gv] = P[0];
            out.pos[3 * gv + 1] = P[1];
            out.pos[3 * gv + 2] = P[2];
          }
          if (out.nrm) { out.nrm[3 * gv] = 0.0f; out.nrm[3 * gv + 1] = 0.0f; out.nrm[3 * gv + 2] = 0.0f; }
          if (out.boundary) out.boundary[gv] = bnd;
          if (out.vkey) out.vkey[gv] = ((uint32_t)(((int64_t)x * dim + y) * dim + z) << 2) | (uint32_t)g;
          if (out.valence) {
            int val = 0;
            for (int e = 0; e < 12; ++e) {
              if (group_of(mask, e) != g) continue;
              const int c0 = edge_c0(e);
              val += q_edge_interior(dim, x + ((c0 >> 2) & 1), y + ((c0 >> 1) & 1), z + (c0 & 1), e >> 2);
            }
            out.valence[gv] = (uint8_t)val;
          }
        }
      }
      // ---- quads: one per interior sign-changing grid edge ----
      uint32_t Xi, Yi, Zi;
      q_quad_words(W, dim, zc, x, y, zb, Xi, Yi, Zi);
      const int own = (int)(((Xi >> lane) & 1u) | (((Yi >> lane) & 1u) << 1) | (((Zi >> lane) & 1u) << 2));
      const int nq = __popc(own);
      if (__ballot_sync(kFull, nq != 0) == 0u) continue;
      const int incl = warp_incl_scan(4 * nq);
      int64_t gi = ch.iout + (int64_t)__ldg(ibase + wo) + (incl - 4 * nq);
      const bool in0 = ((lw.w00 >> lane) & 1u) != 0u;
      for (int a = 0; a < 3; ++a) {
        if (!((own >> a) & 1)) continue;
        const int b = (a + 1) % 3, cax = (a + 2) % 3;
        uint32_t q[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const int ob = (k == 0 || k == 3) ? -1 : 0, oc = (k < 2) ? -1 : 0;
          int cc[3] = {x, y, z};
          cc[b] += ob;
          cc[cax] += oc;
          int lo[3] = {0, 0, 0};
          lo[b] = -ob;
          lo[cax] = -oc;
          const int e = a == 0 ? 2 * lo[1] + lo[2] : (a == 1 ? 4 + 2 * lo[0] + lo[2] : 8 + 2 * lo[0] + lo[1]);
          const int cm = cell_mask_at(W, dim, zc, cc[0], cc[1], cc[2]);
          q[k] = q_vertex_base(vbase, ws.gpl + 3 * ch.words, dim, zc, cc[0], cc[1], cc[2]) + (uint32_t)group_of(cm, e);
        }
        if (!in0) {
          const uint32_t t = q[1];
          q[1] = q[3];
          q[3] = t;
        }
#pragma unroll
        for (int k = 0; k < 4; ++k, ++gi)
          if (gi < out.icap) {
            out.idx[gi] = q[k];
            if (out.idx_global) out.idx_global[gi] = (uint32_t)(ch.vout + q[k]);
          }
      }
    }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Adjoint of the Mode Q vertex placement with respect to the density.
// Per vertex the forward's branch (QEF solution inside the cell, or the mass
// point) is replayed exactly as k_emit took it (same hermite data, same FP32
// QEF).  The incoming position gradient then goes through the QEF -- x = m +
// V f(S) V^T r, r = ATb - ATA m, differentiated with the truncation pattern
// held fixed (Daleckii-Krein: F_ij = (f_i - f_j)/(s_i - s_j), F_ii = f'(s_i))
// -- or through the mass point, then through every hermite pair: the normal
// n = G/|G| of the lerped central-difference gradients and the crossing
// p = a0 + (a1 - a0) mu, mu = -s0 / (s1 - s0), into the density samples
// (float atomics).
//
// T = float differentiates with the forward's own FP32 eigen decomposition.
// T = double recomputes the hermite data and the eigen decomposition (cyclic
// Jacobi to convergence) in FP64 from the same samples: the derivative of
// the exact-arithmetic placement.  It matters because 1/s^2 amplifies the
// ~1e-6 absolute FP32 error of a small kept eigenvalue (s in [1e-3, 0.05] is
// common on smooth surfaces, where a cell's normals are nearly parallel).
// ---------------------------------------------------------------------------
__device__ __forceinline__ int find_chunk_by_vertex(const ChunkDev* __restrict__ chunks, int n, int64_t v);

template <typename T>
struct QefAdj {
  T A[3][3];    // ATA
  T V[3][3];    // eigenvectors (columns)
  T sigma[3];   // eigenvalues
  T inv[3];     // kept reciprocals (0 = truncated)
  T mp[3];      // mass point
  T r[3];       // ATb - ATA mp
};

template <typename T>
__device__ __forceinline__ T dens_t(const float* D, int dim, int x, int y, int z) {
  return (T)dens_at(D, dim, x, y, z);
}

template <typename T>
__device__ __forceinline__ void grid_gradient_t(const float* D, int dim, int x, int y, int z, T g[3]) {
  const int c[3] = {x, y, z};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    int lo[3] = {x, y, z}, hi[3] = {x, y, z};
    T h = (T)0.5;
    if (c[a] > 0) lo[a]--; else h = (T)1;
    if (c[a] < dim - 1) hi[a]++; else h = (T)1;
    g[a] = (dens_t<T>(D, dim, hi[0], hi[1], hi[2]) - dens_t<T>(D, dim, lo[0], lo[1], lo[2])) * h;
  }
}

// Hermite pair of edge e in precision T (the crossing, the lerped gradient,
// its length and the unit normal).
template <typename T>
struct HermiteT {
  int a0[3], a1[3];
  T s0, s1, mu, p[3], g0[3], g1[3], n[3], glen;
};

template <typename T>
__device__ __forceinline__ void hermite_t(const float* D, int dim, int x, int y, int z, int e, bool want_n,
                                          HermiteT<T>& h) {
  const int ca = edge_c0(e), cb = edge_c1(e);
  h.a0[0] = x + ((ca >> 2) & 1); h.a0[1] = y + ((ca >> 1) & 1); h.a0[2] = z + (ca & 1);
  h.a1[0] = x + ((cb >> 2) & 1); h.a1[1] = y + ((cb >> 1) & 1); h.a1[2] = z + (cb & 1);
  h.s0 = dens_t<T>(D, dim, h.a0[0], h.a0[1], h.a0[2]);
  h.s1 = dens_t<T>(D, dim, h.a1[0], h.a1[1], h.a1[2]);
  h.mu = ((T)0 - h.s0) / (h.s1 - h.s0);
#pragma unroll
  for (int k = 0; k < 3; ++k) h.p[k] = ((T)h.a1[k] - (T)h.a0[k]) * h.mu + (T)h.a0[k];
  h.glen = (T)1;
  if (want_n) {
    grid_gradient_t<T>(D, dim, h.a0[0], h.a0[1], h.a0[2], h.g0);
    grid_gradient_t<T>(D, dim, h.a1[0], h.a1[1], h.a1[2], h.g1);
    T G[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) G[k] = h.g0[k] + (h.g1[k] - h.g0[k]) * h.mu;
    h.glen = sqrt((G[0] * G[0] + G[1] * G[1]) + G[2] * G[2]);
#pragma unroll
    for (int k = 0; k < 3; ++k) h.n[k] = G[k] / h.glen;
  }
}

// Symmetric 3x3 eigen decomposition in FP64, A = V diag(w) V^T, refined from
// the forward's FP32 eigenvectors: V0 is re-orthonormalised (Gram-Schmidt),
// A is rotated into that basis (nearly diagonal, off-diagonals ~1e-6 |A|)
// and cyclic Jacobi rotations finish it; convergence is quadratic, so one or
// two sweeps reach the 1e-17 |A| stopping point instead of five or six from
// the identity.
__device__ void eig3_refine(const double A[3][3], const float V0[3][3], double w[3], double V[3][3]) {
  // columns of V0, orthonormalised
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    double v[3] = {(double)V0[0][c], (double)V0[1][c], (double)V0[2][c]};
#pragma unroll
    for (int k = 0; k < c; ++k) {
      const double d = v[0] * V[0][k] + v[1] * V[1][k] + v[2] * V[2][k];
#pragma unroll
      for (int r = 0; r < 3; ++r) v[r] -= d * V[r][k];
    }
    const double il = 1.0 / sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
#pragma unroll
    for (int r = 0; r < 3; ++r) V[r][c] = v[r] * il;
  }
  // B = V^T A V
  double AV[3][3], B[3][3];
#pragma unroll
  for (int r = 0; r < 3; ++r) {
#pragma unroll
    for (int c = 0; c < 3; ++c) AV[r][c] = A[r][0] * V[0][c] + A[r][1] * V[1][c] + A[r][2] * V[2][c];
  }
#pragma unroll
  for (int r = 0; r < 3; ++r) {
#pragma unroll
    for (int c = 0; c < 3; ++c) B[r][c] = V[0][r] * AV[0][c] + V[1][r] * AV[1][c] + V[2][r] * AV[2][c];
  }
#pragma unroll
  for (int r = 0; r < 3; ++r) {
#pragma unroll
    for (int c = 0; c < r; ++c) B[r][c] = B[c][r] = 0.5 * (B[r][c] + B[c][r]);
  }
  const double tol = 1e-17 * (fabs(B[0][0]) + fabs(B[1][1]) + fabs(B[2][2]));
#pragma unroll 1
  for (int sweep = 0; sweep < 16; ++sweep) {
    if (fabs(B[0][1]) + fabs(B[0][2]) + fabs(B[1][2]) <= tol) break;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const int p = q == 2 ? 1 : 0, r = q == 0 ? 1 : 2;
      if (fabs(B[p][r]) <= tol) continue;
      const double tau = (B[r][r] - B[p][p]) / (2.0 * B[p][r]);
      const double t = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
      const double c = 1.0 / sqrt(1.0 + t * t), s = t * c;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const double bkp = B[k][p], bkr = B[k][r];
        B[k][p] = c * bkp - s * bkr;
        B[k][r] = s * bkp + c * bkr;
      }
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const double bpk = B[p][k], brk = B[r][k];
        B[p][k] = c * bpk - s * brk;
        B[r][k] = s * bpk + c * brk;
      }
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const double vkp = V[k][p], vkr = V[k][r];
        V[k][p] = c * vkp - s * vkr;
        V[k][r] = s * vkp + c * vkr;
      }
    }
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) w[i] = B[i][i];
}

// LIST = 0: every vertex; 1: every vertex, but QEF-placed ones are only
// appended to qlist (for a dense second pass); 2: the vertices of qlist.
template <int PLACE, typename T, int LIST>
__global__ void __launch_bounds__(128) k_place_bwd(const ChunkDev* __restrict__ chunks, int n_chunks,
                                                   const uint32_t* __restrict__ words, const float* __restrict__ dens,
                                                   const uint32_t* __restrict__ vkey,
                                                   const int64_t* __restrict__ d_counts, int64_t vcap,
                                                   const float* __restrict__ grad_pos, float* __restrict__ grad_dens,
                                                   uint32_t* __restrict__ qlist, uint32_t* __restrict__ qcount) {
  int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (LIST == 2) {
    if (v >= (int64_t)*qcount) return;
    v = qlist[v];
  }
  if (v >= (d_counts ? min(vcap, d_counts[0]) : vcap)) return;
  const int c = find_chunk_by_vertex(chunks, n_chunks, v);
  const ChunkDev ch = chunks[c];
  const int dim = ch.dim, zc = ch.zc;
  const uint32_t* W = words + ch.words;
  const float* D = dens + ch.dens;
  float* GD = grad_dens + ch.dens;
  const uint32_t key = vkey[v];
  const int lin = (int)(key >> 2), g = (int)(key & 3u);
  const int z = lin % dim, y = (lin / dim) % dim, x = lin / (dim * dim);
  const int mask = cell_mask_at(W, dim, zc, x, y, z);
  const T gx[3] = {(T)grad_pos[3 * v], (T)grad_pos[3 * v + 1], (T)grad_pos[3 * v + 2]};
  // the forward's branch: replay of q_place in FP32
  int cnt = 0;
  QefAccum q;
  if (PLACE == 2) q.init();
  for (int e = 0; e < 12; ++e) {
    if (group_of(mask, e) != g) continue;
    float p[3], n[3];
    hermite(D, dim, x, y, z, e, PLACE == 2, p, n);
    ++cnt;
    if (PLACE == 2) q.add(p, n);
  }
  if (cnt == 0) return;
  bool use_qef = false;
  QefAdj<T> Q;
  if (PLACE == 2) {
    float s[3];
    QefSolveInfo info;
    if (q.solve(s, &info))
      use_qef = s[0] >= (float)x && s[0] <= (float)(x + 1) && s[1] >= (float)y && s[1] <= (float)(y + 1) &&
                s[2] >= (float)z && s[2] <= (float)(z + 1);
    if (LIST == 1 && use_qef) {
      qlist[atomicAdd(qcount, 1u)] = (uint32_t)v;
      return;
    }
    if (use_qef) {
      if (sizeof(T) == sizeof(float)) {
#pragma unroll
        for (int r = 0; r < 3; ++r) {
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            Q.A[r][k] = (T)q.ata[r][k];
            Q.V[r][k] = (T)info.V[r][k];
          }
          Q.sigma[r] = (T)info.sigma[r];
          Q.inv[r] = (T)info.inv[r];
          Q.mp[r] = (T)info.mp[r];
          Q.r[r] = (T)info.r[r];
        }
      } else {
        // the same QEF in FP64: ATA, ATb, mass point, converged eigen pairs
        double A[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, b[3] = {0, 0, 0}, m[3] = {0, 0, 0};
        for (int e = 0; e < 12; ++e) {
          if (group_of(mask, e) != g) continue;
          HermiteT<double> h;
          hermite_t<double>(D, dim, x, y, z, e, true, h);
          const double d = h.n[0] * h.p[0] + h.n[1] * h.p[1] + h.n[2] * h.p[2];
#pragma unroll
          for (int r = 0; r < 3; ++r) {
#pragma unroll
            for (int k = 0; k < 3; ++k) A[r][k] += h.n[r] * h.n[k];
            b[r] += d * h.n[r];
            m[r] += h.p[r];
          }
        }
#pragma unroll
        for (int r = 0; r < 3; ++r) {
          m[r] /= (double)cnt;
#pragma unroll
          for (int k = 0; k < 3; ++k) Q.A[r][k] = (T)A[r][k];
        }
#pragma unroll
        for (int r = 0; r < 3; ++r) {
          Q.mp[r] = (T)m[r];
          Q.r[r] = (T)(b[r] - (A[r][0] * m[0] + A[r][1] * m[1] + A[r][2] * m[2]));
        }
        double w[3], V[3][3];
        eig3_refine(A, info.V, w, V);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          const double oo = 1.0 / w[i];
          const double mn = fabs(w[i]) < fabs(oo) ? fabs(w[i]) : fabs(oo);
          Q.sigma[i] = (T)w[i];
          Q.inv[i] = (T)(mn >= 0.001 ? oo : 0.0);
#pragma unroll
          for (int k = 0; k < 3; ++k) Q.V[k][i] = (T)V[k][i];
        }
      }
    }
  }
  // QEF adjoint down to gA (symmetric), gr, gm
  T gA[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, gr[3] = {0, 0, 0}, gm[3] = {gx[0], gx[1], gx[2]};
  if (use_qef) {
    T Pm[3][3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
#pragma unroll
      for (int k = 0; k < 3; ++k)
        Pm[r][k] = Q.V[r][0] * Q.inv[0] * Q.V[k][0] + Q.V[r][1] * Q.inv[1] * Q.V[k][1] + Q.V[r][2] * Q.inv[2] * Q.V[k][2];
    }
#pragma unroll
    for (int r = 0; r < 3; ++r) gr[r] = Pm[r][0] * gx[0] + Pm[r][1] * gx[1] + Pm[r][2] * gx[2];
    T Gs[3][3], M[3][3], F[3][3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
#pragma unroll
      for (int k = 0; k < 3; ++k) Gs[r][k] = (T)0.5 * (gx[r] * Q.r[k] + gx[k] * Q.r[r]);
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        T s = (T)0;
#pragma unroll
        for (int r = 0; r < 3; ++r) {
#pragma unroll
          for (int k = 0; k < 3; ++k) s += Q.V[r][a] * Gs[r][k] * Q.V[k][b];
        }
        M[a][b] = s;
        // f(s) = 1/s: (f_a - f_b) / (s_a - s_b) = -f_a f_b (no cancellation for
        // close eigenvalues) and f'(s) = -f^2; a truncated eigenvalue (f = 0)
        // beside a kept one takes the quotient
        const T fa = Q.inv[a], fb = Q.inv[b], sa = Q.sigma[a], sb = Q.sigma[b];
        if (fa != (T)0 && fb != (T)0)
          F[a][b] = -fa * fb;
        else if (a == b || fabs(sa - sb) <= (T)1e-6 * (fabs(sa) + fabs(sb)))
          F[a][b] = (T)0;
        else
          F[a][b] = (fa - fb) / (sa - sb);
      }
    }
#pragma unroll
    for (int r = 0; r < 3; ++r) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        T s = (T)0;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
#pragma unroll
          for (int b = 0; b < 3; ++b) s += Q.V[r][a] * F[a][b] * M[a][b] * Q.V[k][b];
        }
        gA[r][k] = s - (T)0.5 * (gr[r] * Q.mp[k] + gr[k] * Q.mp[r]);
      }
    }
#pragma unroll
    for (int r = 0; r < 3; ++r) gm[r] -= Q.A[r][0] * gr[0] + Q.A[r][1] * gr[1] + Q.A[r][2] * gr[2];
  }
  const T inv_cnt = (T)1 / (T)cnt;
  // per hermite pair: g_p, g_n, then into the density
  for (int e = 0; e < 12; ++e) {
    if (group_of(mask, e) != g) continue;
    HermiteT<T> h;
    hermite_t<T>(D, dim, x, y, z, e, PLACE == 2, h);
    const int ax = e >> 2;
    T gp[3], gn[3] = {(T)0, (T)0, (T)0};
    if (!use_qef) {
#pragma unroll
      for (int k = 0; k < 3; ++k) gp[k] = gx[k] * inv_cnt;
    } else {
      const T d = h.n[0] * h.p[0] + h.n[1] * h.p[1] + h.n[2] * h.p[2];
      const T gd = gr[0] * h.n[0] + gr[1] * h.n[1] + gr[2] * h.n[2];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        gn[k] = (T)2 * (gA[k][0] * h.n[0] + gA[k][1] * h.n[1] + gA[k][2] * h.n[2]) + d * gr[k] + gd * h.p[k];
        gp[k] = gd * h.n[k] + gm[k] * inv_cnt;
      }
    }
    T gmu = gp[ax];
    if (use_qef) {
      const T nd = h.n[0] * gn[0] + h.n[1] * gn[1] + h.n[2] * gn[2];
      T gG[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        gG[k] = (gn[k] - h.n[k] * nd) / h.glen;
        gmu += gG[k] * (h.g1[k] - h.g0[k]);
      }
      // central differences at both endpoints: g[a] = (s[hi] - s[lo]) * h
#pragma unroll
      for (int a = 0; a < 3; ++a) {
#pragma unroll
        for (int end = 0; end < 2; ++end) {
          const int* q0 = end ? h.a1 : h.a0;
          const T w = gG[a] * (end ? h.mu : (T)1 - h.mu);
          int lo[3] = {q0[0], q0[1], q0[2]}, hi[3] = {q0[0], q0[1], q0[2]};
          T hh = (T)0.5;
          if (q0[a] > 0) lo[a]--; else hh = (T)1;
          if (q0[a] < dim - 1) hi[a]++; else hh = (T)1;
          atomicAdd(GD + ((int64_t)hi[0] * dim + hi[1]) * dim + hi[2], (float)(w * hh));
          atomicAdd(GD + ((int64_t)lo[0] * dim + lo[1]) * dim + lo[2], (float)(-w * hh));
        }
      }
    }
    const T den = (h.s1 - h.s0) * (h.s1 - h.s0);
    atomicAdd(GD + ((int64_t)h.a0[0] * dim + h.a0[1]) * dim + h.a0[2], (float)(gmu * (-h.s1 / den)));
    atomicAdd(GD + ((int64_t)h.a1[0] * dim + h.a1[1]) * dim + h.a1[2], (float)(gmu * (h.s0 / den)));
  }
}

void launch_place_bwd(int placement, int f64, const ChunkDev* d_chunks, int n_chunks, const uint32_t* words,
                      const float* dens, const uint32_t* vkey, const int64_t* d_counts, int64_t vcap,
                      const float* grad_pos, float* grad_dens, uint32_t* qlist, uint32_t* qcount, cudaStream_t st) {
  const int blocks = (int)((vcap + 127) / 128);
  if (blocks == 0) return;
#define BMF_PLACE_BWD(P, T, L)                                                                                     \
  k_place_bwd<P, T, L><<<blocks, 128, 0, st>>>(d_chunks, n_chunks, words, dens, vkey, d_counts, vcap, grad_pos, \
                                               grad_dens, qlist, qcount)
  if (placement == 2 && f64 && qlist && qcount) {
    // float pass for the mass-point vertices, then the FP64 QEF adjoint over
    // the compacted list of QEF-placed ones (no idle lanes in FP64 code)
    cudaMemsetAsync(qcount, 0, sizeof(uint32_t), st);
    BMF_PLACE_BWD(2, float, 1);
    BMF_PLACE_BWD(2, double, 2);
  } else if (placement == 2) {
    if (f64) BMF_PLACE_BWD(2, double, 0); else BMF_PLACE_BWD(2, float, 0);
  } else {
    BMF_PLACE_BWD(1, float, 0);
  }
#undef BMF_PLACE_BWD
}

// ---------------------------------------------------------------------------
// K5: vertex -> primitive adjacency (the CSR of MeshProcessor::init /
// init_primitives, MeshProcessor.cpp:26-128), built per vertex from the grid
// structure instead of by scattering primitives: a Mode R vertex on the axis-a
// edge of sample s is used by the (up to) four interior cells around that
// edge, whose primitive ids are ascending in linear cell order and, inside a
// cell, in triangle-list order -- exactly the ascending-prim order
// init_primitives produces.  A Mode Q vertex is used by one quad per interior
// crossing edge of its group; those quad ids are sorted.  No atomics, no sort
// pass, deterministic.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int find_chunk_by_vertex(const ChunkDev* __restrict__ chunks, int n, int64_t v) {
  int lo = 0, hi = n - 1;  // last chunk whose vout <= v (empty chunks share the next one's offset)
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (chunks[mid].vout <= v) lo = mid; else hi = mid - 1;
  }
  return lo;
}

template <int MODE>
__global__ void __launch_bounds__(256) k_adj_build(const ChunkDev* __restrict__ chunks, int n_chunks,
                                                   const uint32_t* __restrict__ words, WordScratch ws,
                                                   const uint32_t* __restrict__ vkey, const uint32_t* __restrict__ off,
                                                   const int64_t* __restrict__ d_counts, int64_t vcap,
                                                   uint32_t* __restrict__ adj) {
  __shared__ SmemTabs T;
  load_tabs(T);
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= (d_counts ? min(vcap, d_counts[0]) : vcap)) return;
  const int c = find_chunk_by_vertex(chunks, n_chunks, v);
  const ChunkDev ch = chunks[c];
  const int dim = ch.dim, zc = ch.zc;
  const uint32_t* W = words + ch.words;
  const uint32_t* vbase = ws.vcnt + ch.words;
  const uint32_t* ibase = ws.icnt + ch.words;
  const uint32_t* pl = ws.gpl + 3 * ch.words;
  const uint32_t key = vkey[v];
  const int lin = (int)(key >> 2), k = (int)(key & 3u);
  const int z = lin % dim, y = (lin / dim) % dim, x = lin / (dim * dim);
  uint32_t* out = adj + off[v];
  // the vertex's CSR range (the exclusive scan of init_valence): never write past it
  const int room = (int)(off[v + 1] - off[v]);
  int n = 0;
  if (MODE == 0) {
    const int a = k;
#pragma unroll
    for (int q = 0; q < 4; ++q) {  // cells around the edge, ascending linear order
      const int d1 = (q >> 1) ^ 1, d2 = (q & 1) ^ 1;
      int cx = x, cy = y, cz = z, e;
      if (a == 0) { cy -= d1; cz -= d2; e = 2 * d1 + d2; }
      else if (a == 1) { cx -= d1; cz -= d2; e = 4 + 2 * d1 + d2; }
      else { cx -= d1; cy -= d2; e = 8 + 2 * d1 + d2; }
      if (cx < 0 || cy < 0 || cz < 0 || cx > dim - 2 || cy > dim - 2 || cz > dim - 2) continue;
      const int m = cell_mask_at(W, dim, zc, cx, cy, cz);
      if (!tab_uses(T, m, e)) continue;
      const uint64_t tw = T.tri[m];
      const int nt = (int)(tw >> 60);
      const int64_t wi = ((int64_t)cx * dim + cy) * zc + (cz >> 5);
      const uint32_t lt = lane_lt(cz & 31);
      const uint32_t pre = __popc(__ldg(pl + 3 * wi) & lt) + 2 * __popc(__ldg(pl + 3 * wi + 1) & lt) +
                           4 * __popc(__ldg(pl + 3 * wi + 2) & lt);
      const int64_t first = (ch.iout + (int64_t)__ldg(ibase + wi)) / 3 + pre;
      for (int t = 0; t < nt; ++t)
        if ((tri_edge(tw, 3 * t) == e || tri_edge(tw, 3 * t + 1) == e || tri_edge(tw, 3 * t + 2) == e) && n < room)
          out[n++] = (uint32_t)(first + t);
    }
  } else {
    const int g = k;
    const int m = cell_mask_at(W, dim, zc, x, y, z);
    uint32_t ids[12];
    const uint64_t gw = T.grp[m];
    for (int e = 0; e < 12; ++e) {
      if ((int)((gw >> (4 * e)) & 0xF) != g) continue;
      const int c0 = edge_c0(e), a = e >> 2;
      const int sx = x + ((c0 >> 2) & 1), sy = y + ((c0 >> 1) & 1), sz = z + (c0 & 1);
      if (!q_edge_interior(dim, sx, sy, sz, a)) continue;
      uint32_t Xi, Yi, Zi;
      q_quad_words(W, dim, zc, sx, sy, sz >> 5, Xi, Yi, Zi);
      const int l = sz & 31;
      const uint32_t lt = lane_lt(l);
      uint32_t pre = __popc(Xi & lt) + __popc(Yi & lt) + __popc(Zi & lt);
      if (a >= 1) pre += (Xi >> l) & 1u;
      if (a >= 2) pre += (Yi >> l) & 1u;
      const int64_t wi = ((int64_t)sx * dim + sy) * zc + (sz >> 5);
      uint32_t id = (uint32_t)((ch.iout + (int64_t)__ldg(ibase + wi)) / 4 + pre);
      int j = n++;  // insertion into the sorted prefix
      while (j > 0 && ids[j - 1] > id) { ids[j] = ids[j - 1]; --j; }
      ids[j] = id;
    }
    for (int i = 0; i < n && i < room; ++i) out[i] = ids[i];
  }
  (void)vbase;
}

void launch_adj_build(int mode, const ChunkDev* d_chunks, int n_chunks, const uint32_t* words, WordScratch ws,
                      const uint32_t* vkey, const uint32_t* off, const int64_t* d_counts, int64_t vcap,
                      uint32_t* adj, cudaStream_t st) {
  const int blocks = (int)((vcap + 255) / 256);
  if (blocks == 0) return;
  if (mode == 0) k_adj_build<0><<<blocks, 256, 0, st>>>(d_chunks, n_chunks, words, ws, vkey, off, d_counts, vcap, adj);
  else k_adj_build<1><<<blocks, 256, 0, st>>>(d_chunks, n_chunks, words, ws, vkey, off, d_counts, vcap, adj);
}

void launch_count(int mode, const ChunkDev* d_chunks, int n_chunks, const int* d_unit_start, int n_units,
                  const uint32_t* words, const uint32_t* flags, WordScratch ws, cudaStream_t st) {
  if (mode == 0 && ws.clist) cudaMemsetAsync(ws.ccount, 0, sizeof(uint32_t), st);
  if (mode == 0) k_count<0><<<n_units, 256, 0, st>>>(d_chunks, n_chunks, d_unit_start, words, flags, ws);
  else k_count<1><<<n_units, 256, 0, st>>>(d_chunks, n_chunks, d_unit_start, words, flags, ws);
}

void launch_scan_chunks(const ChunkDev* d_chunks, int n_chunks, WordScratch ws, uint32_t* d_tot, cudaStream_t st) {
  k_scan_chunks<<<n_chunks, kScanThreads, 0, st>>>(d_chunks, ws, d_tot);
}

void launch_chunk_offsets(ChunkDev* d_chunks, int n_chunks, const uint32_t* d_tot, const uint32_t* flags,
                          int64_t vcap, int64_t icap, int64_t* d_info, int64_t* d_totals, cudaStream_t st) {
  k_chunk_offsets<<<1, 1024, 0, st>>>(d_chunks, n_chunks, d_tot, flags, vcap, icap, d_info, d_totals);
}

// Mode R emission over the work list, one thread per active cell (the
// warp-per-word form runs most lanes idle: a busy word holds a few surface
// cells).  Per cell it writes exactly what k_emit<0,0> writes for the cell's
// lane: its owned vertices (ids from the scanned word base and the crossing
// words, calculate_isovertex positions, boundary, key, init_valence) and its
// triangles (slot from the word's index base and the triangle-count planes).
__global__ void __launch_bounds__(256, 3) k_emit_cells_r(const ChunkDev* __restrict__ chunks,
                                                      const uint32_t* __restrict__ words,
                                                      const float* __restrict__ dens, WordScratch ws, MeshOut out) {
  __shared__ SmemTabs T;
  load_tabs(T);
  const int64_t n = min((int64_t)*ws.ccount, ws.clist_cap);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const uint2 ent = ws.clist[i];
    const ChunkDev ch = chunks[ent.x];
    const int dim = ch.dim, zc = ch.zc;
    const int lin = (int)ent.y;
    const int z = lin % dim, y = (lin / dim) % dim, x = lin / (dim * dim);
    const int zb = z >> 5, lane = z & 31;
    const uint32_t lt = lane_lt(lane);
    const uint32_t* W = words + ch.words;
    const uint32_t* vbase = ws.vcnt + ch.words;
    const float* D = dens + ch.dens;
    const int64_t wo = ((int64_t)x * dim + y) * zc + zb;
    const uint32_t w00 = word_at(W, dim, zc, x, y, zb);
    const uint32_t X = (x + 1 < dim) ? (w00 ^ word_at(W, dim, zc, x + 1, y, zb)) : 0u;
    const uint32_t Y = (y + 1 < dim) ? (w00 ^ word_at(W, dim, zc, x, y + 1, zb)) : 0u;
    const uint32_t Z = zcross_word(W, dim, zc, x, y, zb);
    const uint32_t own = ((X >> lane) & 1u) | (((Y >> lane) & 1u) << 1) | (((Z >> lane) & 1u) << 2);
    if (own) {
      uint32_t vid = __ldg(vbase + wo) + __popc(X & lt) + __popc(Y & lt) + __popc(Z & lt);
      for (int a = 0; a < 3; ++a) {
        if (!((own >> a) & 1u)) continue;
        const int x1 = x + (a == 0), y1 = y + (a == 1), z1 = z + (a == 2);
        const int64_t gv = ch.vout + vid;
        ++vid;
        if (gv >= out.vcap) continue;
        const float s0 = dens_at(D, dim, x, y, z), s1 = dens_at(D, dim, x1, y1, z1);
        const float mu = (0.0f - s0) / (s1 - s0);
        const float q0[3] = {(float)x, (float)y, (float)z};
        const float dl[3] = {(float)(x1 - x), (float)(y1 - y), (float)(z1 - z)};
        float* P = out.pos + 3 * gv;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const float dv = dl[k] * mu;
          P[k] = dv + q0[k];
        }
        if (out.boundary)
          out.boundary[gv] = (x == 0 || y == 0 || z == 0 || x == dim - 1 || y == dim - 1 || z == dim - 1 ||
                              x1 == dim - 1 || y1 == dim - 1 || z1 == dim - 1);
        if (out.nrm) { out.nrm[3 * gv] = 0.0f; out.nrm[3 * gv + 1] = 0.0f; out.nrm[3 * gv + 2] = 0.0f; }
        if (out.vkey) out.vkey[gv] = ((uint32_t)lin << 2) | (uint32_t)a;
        if (out.valence) {
          int val = 0;
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const int d1 = k >> 1, d2 = k & 1;
            int cx = x, cy = y, cz = z, e;
            if (a == 0) { cy -= d1; cz -= d2; e = 2 * d1 + d2; }
            else if (a == 1) { cx -= d1; cz -= d2; e = 4 + 2 * d1 + d2; }
            else { cx -= d1; cy -= d2; e = 8 + 2 * d1 + d2; }
            if (cx < 0 || cy < 0 || cz < 0 || cx > dim - 2 || cy > dim - 2 || cz > dim - 2) continue;
            val += tab_uses(T, cell_mask_at(W, dim, zc, cx, cy, cz), e);
          }
          out.valence[gv] = (uint8_t)val;
        }
      }
    }
    const bool interior = x < dim - 1 && y < dim - 1 && z < dim - 1;
    const int mask = interior ? cell_mask_at(W, dim, zc, x, y, z) : 0;
    const uint64_t tw = T.tri[mask];
    const int t3 = 3 * (int)(tw >> 60);
    if (t3 == 0) continue;
    const uint32_t* pl = ws.gpl + 3 * (ch.words + wo);
    const int before = __popc(__ldg(pl) & lt) + 2 * __popc(__ldg(pl + 1) & lt) + 4 * __popc(__ldg(pl + 2) & lt);
    int64_t gi = ch.iout + (int64_t)__ldg(ws.icnt + ch.words + wo) + 3 * before;
    for (int k = 0; k < t3; ++k, ++gi) {
      const int e = tri_edge(tw, k);
      const uint32_t vid = r_vertex_id(W, vbase, dim, zc, x + c_edge_owner[e][0], y + c_edge_owner[e][1],
                                       z + c_edge_owner[e][2], c_edge_owner[e][3]);
      if (gi < out.icap) {
        out.idx[gi] = vid;
        if (out.idx_global) out.idx_global[gi] = (uint32_t)(ch.vout + vid);
      }
    }
  }
}

// Mode Q QEF placement, one thread per vertex (dense lanes, unlike the
// warp-per-word emit where only surface cells' lanes work): the same
// q_place<2> on the vertex's cell and group, decoded from its key.
__global__ void __launch_bounds__(128) k_place_qef(const ChunkDev* __restrict__ chunks, int n_chunks,
                                                   const uint32_t* __restrict__ words, const float* __restrict__ dens,
                                                   const uint32_t* __restrict__ vkey,
                                                   const int64_t* __restrict__ d_counts, int64_t vcap,
                                                   float* __restrict__ pos) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= min(vcap, d_counts[0])) return;
  const int c = find_chunk_by_vertex(chunks, n_chunks, v);
  const ChunkDev ch = chunks[c];
  const int dim = ch.dim;
  const uint32_t key = vkey[v];
  const int lin = (int)(key >> 2), g = (int)(key & 3u);
  const int z = lin % dim, y = (lin / dim) % dim, x = lin / (dim * dim);
  const int mask = cell_mask_at(words + ch.words, dim, ch.zc, x, y, z);
  float P[3];
  q_place<2>(dens + ch.dens, dim, x, y, z, mask, g, P);
  pos[3 * v] = P[0];
  pos[3 * v + 1] = P[1];
  pos[3 * v + 2] = P[2];
}

int launch_emit(int mode, int placement, const ChunkDev* d_chunks, int n_chunks, const int* d_unit_start,
                int n_units, const uint32_t* words, const float* dens, const uint32_t* flags, WordScratch ws,
                MeshOut out, const int64_t* d_counts, cudaStream_t st) {
  if (mode == 0 && ws.clist) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    k_emit_cells_r<<<sms * 8, 256, 0, st>>>(d_chunks, words, dens, ws, out);
  } else if (mode == 0) {
    k_emit<0, 0><<<n_units, 256, 0, st>>>(d_chunks, n_chunks, d_unit_start, words, dens, flags, ws, out);
  } else if (placement == 0) {
    k_emit<1, 0><<<n_units, 256, 0, st>>>(d_chunks, n_chunks, d_unit_start, words, dens, flags, ws, out);
  } else if (placement == 1) {
    k_emit<1, 1><<<n_units, 256, 0, st>>>(d_chunks, n_chunks, d_unit_start, words, dens, flags, ws, out);
  } else {
    if (!out.vkey || !d_counts) out.vkey = nullptr;  // no keys: the emit places in place
    k_emit<1, 2><<<n_units, 256, 0, st>>>(d_chunks, n_chunks, d_unit_start, words, dens, flags, ws, out);
    if (out.vkey && out.vcap > 0) {
      k_place_qef<<<(int)((out.vcap + 127) / 128), 128, 0, st>>>(d_chunks, n_chunks, words, dens, out.vkey, d_counts,
                                                                out.vcap, out.pos);
      return 2;
    }
  }
  return 1;
}

}  // namespace bmf
