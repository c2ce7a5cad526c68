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
#include "bmf_qef.cuh"
#include "bmf_sweep.cuh"

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
  uint64_t etris[256];  // per case and edge e: bits [5 e, 5 e + 5) mark the triangles that use e
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
// K2: per-word counts, one thread per occupancy word.
//
// Everything a word contributes is bit arithmetic on the eight line words
// around it (lines (x..x+1, y..y+1), blocks zb and zb + 1): its owned
// crossings X / Y / Z (vertex count by popc, Mode R), its interior quad edges
// (Mode Q), and the set of its cells whose corner mask is mixed (neither 0 nor
// 255).  Only mixed cells can emit triangles or hold vertex groups, so the
// per-cell table lookup runs over the set bits of that mask alone; the
// counts go into three bit-planes (a cell's first primitive / vertex is
// base + popc(p0 & lt) + 2 popc(p1 & lt) + 4 popc(p2 & lt)).
// ---------------------------------------------------------------------------

// Per corner mask: Mode R triangle count (low nibble) and Mode Q vertex-group
// count (high nibble), four masks per word.
struct CaseCounts {
  uint32_t w[64];
};
constexpr CaseCounts make_case_counts() {
  constexpr uint64_t tri[256] = BMF_TRI_CASES_INIT;
  constexpr uint64_t grp[256] = BMF_GROUP_CASES_INIT;
  CaseCounts c{};
  for (int m = 0; m < 256; ++m)
    c.w[m >> 2] |= (uint32_t)((tri[m] >> 60) | (((grp[m] >> 48) & 0xF) << 4)) << (8 * (m & 3));
  return c;
}
static __device__ const CaseCounts g_case_counts = make_case_counts();

// Per corner mask and edge e: which of the case's triangles (bit t, t < 5)
// use edge e, at bits [5 e, 5 e + 5) -- derived from the triangle table.
struct EdgeTris {
  uint64_t w[256];
};
constexpr EdgeTris make_edge_tris() {
  constexpr uint64_t tri[256] = BMF_TRI_CASES_INIT;
  EdgeTris r{};
  for (int m = 0; m < 256; ++m) {
    const int nt = (int)(tri[m] >> 60);
    for (int t = 0; t < nt; ++t)
      for (int i = 0; i < 3; ++i) r.w[m] |= 1ull << (5 * (int)((tri[m] >> (4 * (3 * t + i))) & 0xFu) + t);
  }
  return r;
}
static __device__ const EdgeTris g_edge_tris = make_edge_tris();

constexpr int kCountThreads = 64;

// Cells z of block zb with z <= hi (bits [0, hi - 32 zb]).
__device__ __forceinline__ uint32_t zbits_upto(int hi, int zb) {
  const int n = hi - 32 * zb + 1;
  return n >= 32 ? kFull : (n <= 0 ? 0u : ((1u << n) - 1u));
}

template <int MODE>
__global__ void __launch_bounds__(kCountThreads) k_count(const ChunkDev* __restrict__ chunks, int n_chunks,
                                                         const int* __restrict__ unit_start,
                                                         const uint32_t* __restrict__ words,
                                                         const uint32_t* __restrict__ flags, WordScratch ws) {
  __shared__ uint32_t s_cnt[64];
  __shared__ int s_c;
  const int u = blockIdx.x;
  for (int i = threadIdx.x; i < 64; i += blockDim.x) s_cnt[i] = g_case_counts.w[i];
  if (threadIdx.x == 0) s_c = find_chunk_e(unit_start, n_chunks, u);
  __syncthreads();
  const int c = s_c;
  const ChunkDev ch = chunks[c];
  const int x = u - __ldg(unit_start + c);
  const int dim = ch.dim, zc = ch.zc, nw = dim * zc;
  const uint32_t* W = words + ch.words;
  const bool cm = contains_mesh(__ldg(flags + c));
  const int lane = threadIdx.x & 31;
  const bool listing = ws.clist != nullptr;
  const bool xin = x + 1 < dim;  // line x + 1 exists (cells and x-crossings of this plane)
  // a word's y is its index times the rounded-up 2^32 / zc, high half: exact
  // while index * zc < 2^32
  const uint64_t zmagic = ((1ull << 32) + (uint64_t)zc - 1u) / (uint64_t)zc;
  const uint32_t* Wx = W + (int64_t)x * nw;  // the plane's words
  for (int base = 0; base < nw; base += kCountThreads) {
    const int wi = base + threadIdx.x;
    const int y = (int)(((uint64_t)(uint32_t)wi * zmagic) >> 32), zb = wi - y * zc;
    uint32_t vc = 0u, ic = 0u, p0 = 0u, p1 = 0u, p2 = 0u, act = 0u;
    uint32_t f00 = 0u, f10 = 0u, f01 = 0u, fnx = 0u;  // band fill: samples to make exact
    if (wi < nw && cm) {
      const bool yin = y + 1 < dim, nin = zb + 1 < zc;
      const uint32_t* L00 = Wx + wi;  // the word (x, y, zb)
      const uint32_t w00 = __ldg(L00), n00 = nin ? __ldg(L00 + 1) : 0u;
      const uint32_t w01 = yin ? __ldg(L00 + zc) : 0u, n01 = (yin && nin) ? __ldg(L00 + zc + 1) : 0u;
      const uint32_t* L10 = L00 + (int64_t)dim * zc;
      const uint32_t w10 = xin ? __ldg(L10) : 0u, n10 = (xin && nin) ? __ldg(L10 + 1) : 0u;
      const uint32_t w11 = (xin && yin) ? __ldg(L10 + zc) : 0u, n11 = (xin && yin && nin) ? __ldg(L10 + zc + 1) : 0u;
      // corner words: bit l = corner (dx, dy, dz) of cell 32 zb + l
      const uint32_t a0 = w00, a1 = (w00 >> 1) | (n00 << 31), b0 = w01, b1 = (w01 >> 1) | (n01 << 31);
      const uint32_t c0 = w10, c1 = (w10 >> 1) | (n10 << 31), d0 = w11, d1 = (w11 >> 1) | (n11 << 31);
      const uint32_t any = a0 | a1 | b0 | b1 | c0 | c1 | d0 | d1, all = a0 & a1 & b0 & b1 & c0 & c1 & d0 & d1;
      const uint32_t zint = zbits_upto(dim - 2, zb);  // cells z <= dim - 2
      const uint32_t interior = (xin && yin) ? zint : 0u;
      const uint32_t mixed = interior & any & ~all;
      uint32_t t = 0u;
      for (uint32_t m = mixed; m; m &= m - 1u) {
        const int l = __ffs(m) - 1;
        const int mask = (int)(((w00 >> l) & 1u) | (((a1 >> l) & 1u) << 1) | (((w01 >> l) & 1u) << 2) |
                               (((b1 >> l) & 1u) << 3) | (((w10 >> l) & 1u) << 4) | (((c1 >> l) & 1u) << 5) |
                               (((w11 >> l) & 1u) << 6) | (((d1 >> l) & 1u) << 7));
        const uint32_t k = (s_cnt[mask >> 2] >> (8 * (mask & 3))) >> (MODE == 0 ? 0 : 4);
        const uint32_t n = k & 0xFu;
        t += n;
        p0 |= (n & 1u) << l;
        p1 |= ((n >> 1) & 1u) << l;
        p2 |= ((n >> 2) & 1u) << l;
      }
      if (MODE == 0) {
        const uint32_t X = xin ? (w00 ^ w10) : 0u;
        const uint32_t Y = yin ? (w00 ^ w01) : 0u;
        const uint32_t Z = (w00 ^ a1) & zbits_upto(dim - 2, zb);
        vc = __popc(X) + __popc(Y) + __popc(Z);
        ic = 3u * t;
        act = p0 | p1 | p2 | X | Y | Z;
        if (ws.exact && (X | Y | Z)) {
          // the band fill's inexact samples at the ends of this word's crossings:
          // own samples (X, Y, Z starts, Z ends), line x + 1 (X), line y + 1 (Y),
          // and bit 0 of the next word (the end of a crossing from bit 31)
          const uint32_t* E = ws.exact + ch.words + ((int64_t)x * dim + y) * zc + zb;
          f00 = (X | Y | Z | (Z << 1)) & ~__ldg(E);
          f10 = X ? (X & ~__ldg(E + (int64_t)dim * zc)) : 0u;
          f01 = Y ? (Y & ~__ldg(E + zc)) : 0u;
          fnx = (Z >> 31) ? (~__ldg(E + 1) & 1u) : 0u;
        }
      } else {
        // interior quad edges: the four cells around the edge exist
        const bool yi = y >= 1 && y <= dim - 2, xi = x >= 1 && x <= dim - 2;
        const uint32_t zlo = zb == 0 ? ~1u : kFull;  // with zint: z in [1, dim - 2]
        const uint32_t Xi = (yi && xin) ? ((w00 ^ w10) & zint & zlo) : 0u;
        const uint32_t Yi = (xi && yin) ? ((w00 ^ w01) & zint & zlo) : 0u;
        const uint32_t Zi = (xi && yi) ? ((w00 ^ a1) & zbits_upto(dim - 2, zb)) : 0u;
        vc = t;
        ic = 4u * (__popc(Xi) + __popc(Yi) + __popc(Zi));
        act = p0 | p1 | p2 | Xi | Yi | Zi;
      }
    }
    if (wi < nw) {
      const int64_t o = ch.words + (int64_t)x * nw + wi;
      ws.vcnt[o] = vc;
      ws.icnt[o] = ic;
      if (ws.gpl) {
        ws.gpl[3 * o] = p0;
        ws.gpl[3 * o + 1] = p1;
        ws.gpl[3 * o + 2] = p2;
      }
    }
    if (MODE == 0 && ws.exact && __any_sync(kFull, (f00 | f10 | f01 | fnx) != 0u)) {
      // one global reservation per warp for the samples to make exact
      const int nf = __popc(f00) + __popc(f10) + __popc(f01) + __popc(fnx);
      int incl = nf;
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        const int v = __shfl_up_sync(kFull, incl, off);
        if (lane >= off) incl += v;
      }
      const int tot = __shfl_sync(kFull, incl, 31);
      if (tot) {
        uint32_t fbase = 0u;
        if (lane == 31) fbase = atomicAdd(ws.fcount, (uint32_t)tot);
        fbase = __shfl_sync(kFull, fbase, 31);
        if (nf) {
          int64_t slot = (int64_t)fbase + incl - nf;
          const uint32_t s00 = (uint32_t)((((int64_t)x * dim + y) * dim) + 32 * zb);
          auto put = [&](uint32_t m, uint32_t sbase) {
            for (; m; m &= m - 1u, ++slot)
              if (slot < ws.fix_cap) ws.fix[slot] = make_uint2((uint32_t)c, sbase + (uint32_t)(__ffs(m) - 1));
          };
          put(f00, s00);
          put(f10, s00 + (uint32_t)dim * (uint32_t)dim);
          put(f01, s00 + (uint32_t)dim);
          put(fnx, s00 + 32u);
        }
      }
    }
    if (listing && __any_sync(kFull, act != 0u)) {
      // one global reservation per warp; Mode R lists busy words, Mode Q
      // each word's active cells in bit order
      const int na = MODE == 0 ? (act != 0u ? 1 : 0) : __popc(act);
      int incl = na;
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        const int v = __shfl_up_sync(kFull, incl, off);
        if (lane >= off) incl += v;
      }
      const int tot = __shfl_sync(kFull, incl, 31);
      uint32_t wbase = 0u;
      if (lane == 31 && tot) wbase = atomicAdd(ws.ccount, (uint32_t)tot);
      wbase = __shfl_sync(kFull, wbase, 31);
      if (act) {
        int64_t slot = (int64_t)wbase + incl - na;
        if (MODE == 0) {
          if (slot < ws.clist_cap) ws.clist[slot] = make_uint2((uint32_t)c, (uint32_t)(x * nw + wi));
        } else {
          const uint32_t key0 = vertex_key(x, y, 32 * zb, 0);  // the cell as a vertex key (k = 0)
          for (uint32_t m = act; m; m &= m - 1u, ++slot)
            if (slot < ws.clist_cap)
              ws.clist[slot] = make_uint2((uint32_t)c, key0 + ((uint32_t)(__ffs(m) - 1) << 2));
        }
      }
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
constexpr int kScanItems = 2;

// order (nullable): CTA i scans chunk order[i] -- largest chunks first, so the
// longest scans do not start last.
__global__ void __launch_bounds__(kScanThreads) k_scan_chunks(const ChunkDev* __restrict__ chunks, WordScratch ws,
                                                            uint32_t* __restrict__ tot, const int* __restrict__ order) {
  const int cid = order ? __ldg(order + blockIdx.x) : (int)blockIdx.x;
  const ChunkDev ch = chunks[cid];
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
    tot[2 * cid] = carry_v;
    tot[2 * cid + 1] = carry_i;
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
          if (out.vkey) out.vkey[gv] = vertex_key(x, y, z, a);
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
          if (out.vkey) out.vkey[gv] = vertex_key(x, y, z, g);
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

void launch_place_bwd(int placement, int wide, const ChunkDev* d_chunks, int n_chunks, const uint32_t* words,
                      const float* dens, const uint32_t* vkey, const int64_t* d_counts, int64_t vcap,
                      const float* grad_pos, float* grad_dens, uint32_t* qlist, uint32_t* qcount, float* qseed,
                      const uint8_t* qflag, cudaStream_t st) {
  const int blocks = (int)((vcap + 127) / 128);
  if (blocks == 0) return;
#define BMF_PLACE_BWD(P, T, L)                                                                                     \
  k_place_bwd<P, T, L><<<blocks, 128, 0, st>>>(d_chunks, n_chunks, words, dens, vkey, d_counts, vcap, grad_pos, \
                                               grad_dens, qlist, qcount, qseed, qflag)
  if (placement == 2 && wide && qlist && qcount && qseed && qflag) {
    // the forward recorded the branch and built the list: float pass over the
    // mass-point vertices, then the wide QEF adjoint over the list
    BMF_PLACE_BWD(2, float, 3);
    launch_place_bwd_wide_list(wide, d_chunks, n_chunks, words, dens, vkey, d_counts, vcap, grad_pos, grad_dens,
                               qlist, qcount, qseed, st);
  } else if (placement == 2 && wide && qlist && qcount && qseed) {
    // float pass for the mass-point vertices, then the wide QEF adjoint over
    // the compacted list of QEF-placed ones (no idle lanes in the wide code;
    // its own translation unit, compiled with FMA contraction)
    cudaMemsetAsync(qcount, 0, sizeof(uint32_t), st);
    BMF_PLACE_BWD(2, float, 1);
    launch_place_bwd_wide_list(wide, d_chunks, n_chunks, words, dens, vkey, d_counts, vcap, grad_pos, grad_dens,
                               qlist, qcount, qseed, st);
  } else if (placement == 2) {
    if (wide) BMF_PLACE_BWD(2, double, 0); else BMF_PLACE_BWD(2, float, 0);
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

// Three consecutive inside bits z0..z0+2 of line (x, y) (zero outside the
// chunk); W is the chunk's words, 32-bit offsets.
__device__ __forceinline__ uint32_t line_bits3(const uint32_t* __restrict__ W, int dim, int zc, int x, int y, int z0) {
  if (x < 0 || y < 0 || x >= dim || y >= dim) return 0u;
  const int b0 = z0 >> 5, s = z0 & 31;  // arithmetic shift: block -1 for z0 = -1
  const uint32_t* L = W + (x * dim + y) * zc;
  uint32_t bits = (b0 >= 0 && b0 < zc) ? __ldg(L + b0) >> s : 0u;
  if (s > 29 && b0 + 1 < zc) bits |= __ldg(L + b0 + 1) << (32 - s);  // the three bits cross into the next word
  return bits & 7u;
}

// Which case tables a kernel stages in shared memory.
template <bool TRI, bool USES, bool GRP, bool ETRIS = false>
__device__ __forceinline__ void load_tabs_some(SmemTabs& t) {
  for (int i = threadIdx.x; i < 256; i += blockDim.x) {
    if (TRI) t.tri[i] = __ldg(g_tri_cases + i);
    if (USES) t.uses[i] = __ldg(g_edge_uses + i);
    if (GRP) t.grp[i] = __ldg(g_group_cases + i);
    if (ETRIS) t.etris[i] = g_edge_tris.w[i];
  }
  __syncthreads();
}

// The adjacency list of one vertex (key: its packed grid position) of chunk
// ch, at most room entries, into out.
// OUT = uint16_t with rel = the chunk's first primitive: the list holds
// chunk-relative ids (the chunk-by-chunk sweeps, for chunks of at most 65535
// primitives: half the bytes in the gathers' working set).
template <int MODE, typename OUT = uint32_t>
__device__ __forceinline__ void adj_vertex(const SmemTabs& T, const ChunkDev& ch, const uint32_t* __restrict__ words,
                                           const WordScratch& ws, uint32_t key, OUT* __restrict__ out,
                                           int room, int64_t rel = 0) {
  const int dim = ch.dim, zc = ch.zc;
  const int64_t iout = ch.iout;
  const uint32_t* W = words + ch.words;
  const uint32_t* ibase = ws.icnt + ch.words;
  const uint32_t* pl = ws.gpl + 3 * ch.words;
  int x, y, z, k;
  vertex_key_decode(key, x, y, z, k);
  // the chunk's first primitive (its index offset and word bases are
  // multiples of the primitive size)
  const int64_t pbase = iout / (MODE == 0 ? 3 : 4);
  int n = 0;
  if (MODE == 0) {
    const int a = k;
    // inside bits of lines (x-1+i, y-1+j), samples z-1..z+1, packed 3 bits per
    // line at bit 3 (3i + j): every corner of the four cells around the edge
    uint32_t nbits = 0u;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j)
        if (a == 0 ? i >= 1 : (a == 1 ? j >= 1 : true))
          nbits |= line_bits3(W, dim, zc, x - 1 + i, y - 1 + j, z - 1) << (3 * (3 * i + j));
#pragma unroll
    for (int q = 0; q < 4; ++q) {  // cells around the edge, ascending linear order
      const int d1 = (q >> 1) ^ 1, d2 = (q & 1) ^ 1;
      int ox = 0, oy = 0, oz = 0;
      if (a == 0) { oy = -d1; oz = -d2; }
      else if (a == 1) { ox = -d1; oz = -d2; }
      else { ox = -d1; oy = -d2; }
      const int e = 4 * a + 2 * d1 + d2;
      const int cx = x + ox, cy = y + oy, cz = z + oz;
      if (cx < 0 || cy < 0 || cz < 0 || cx > dim - 2 || cy > dim - 2 || cz > dim - 2) continue;
      // corner (dx, dy, dz): line (1 + ox + dx, 1 + oy + dy), bit 1 + oz + dz
      const uint32_t base = nbits >> (3 * (3 * (1 + ox) + (1 + oy)) + 1 + oz);
      const int m = (int)((base & 3u) | (((base >> 3) & 3u) << 2) | (((base >> 9) & 3u) << 4) |
                          (((base >> 12) & 3u) << 6));
      // the cell's triangles that use edge e, ascending (polygonize_cell order)
      uint32_t tm = (uint32_t)(T.etris[m] >> (5 * e)) & 31u;
      if (!tm) continue;
      const int wi = (cx * dim + cy) * zc + (cz >> 5);
      const uint32_t lt = lane_lt(cz & 31);
      const uint32_t pre = __popc(__ldg(pl + 3 * wi) & lt) + 2 * __popc(__ldg(pl + 3 * wi + 1) & lt) +
                           4 * __popc(__ldg(pl + 3 * wi + 2) & lt);
      const int64_t first = pbase + __ldg(ibase + wi) / 3u + pre;
      for (; tm && n < room; tm &= tm - 1u) out[n++] = (OUT)(first + __ffs(tm) - 1 - rel);
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
      const int wi = (sx * dim + sy) * zc + (sz >> 5);
      uint32_t id = (uint32_t)(pbase + __ldg(ibase + wi) / 4u + pre);
      int j = n++;  // insertion into the sorted prefix
      while (j > 0 && ids[j - 1] > id) { ids[j] = ids[j - 1]; --j; }
      ids[j] = id;
    }
    for (int i = 0; i < n && i < room; ++i) out[i] = (OUT)(ids[i] - rel);
  }
}

template <int MODE>
__global__ void __launch_bounds__(256) k_adj_build(const ChunkDev* __restrict__ chunks, int n_chunks,
                                                   const uint32_t* __restrict__ words, WordScratch ws,
                                                   const uint32_t* __restrict__ vkey, const uint32_t* __restrict__ off,
                                                   const int64_t* __restrict__ d_counts, int64_t vcap,
                                                   uint32_t* __restrict__ adj) {
  __shared__ SmemTabs T;
  load_tabs_some<false, false, MODE != 0, MODE == 0>(T);
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= (d_counts ? min(vcap, d_counts[0]) : vcap)) return;
  const int c = find_chunk_by_vertex(chunks, n_chunks, v);
  // the vertex's CSR range (the exclusive scan of init_valence): never write past it
  adj_vertex<MODE>(T, chunks[c], words, ws, vkey[v], adj + off[v], (int)(off[v + 1] - off[v]));
}

void launch_adj_build(int mode, const ChunkDev* d_chunks, int n_chunks, const uint32_t* words, WordScratch ws,
                      const uint32_t* vkey, const uint32_t* off, const int64_t* d_counts, int64_t vcap,
                      uint32_t* adj, cudaStream_t st) {
  const int blocks = (int)((vcap + 255) / 256);
  if (blocks == 0) return;
  if (mode == 0) k_adj_build<0><<<blocks, 256, 0, st>>>(d_chunks, n_chunks, words, ws, vkey, off, d_counts, vcap, adj);
  else k_adj_build<1><<<blocks, 256, 0, st>>>(d_chunks, n_chunks, words, ws, vkey, off, d_counts, vcap, adj);
}

// ---------------------------------------------------------------------------
// K5+K6 chunk by chunk (batches): one CTA per chunk, from a queue ordered
// largest first, runs the chunk's CSR offsets, its adjacency and every
// dual / primal sweep with block barriers in between.  A chunk's vertices
// only touch its own primitives, and the sum of its vertices' valences is its
// index count, so the chunk's offsets are its index offset plus the exclusive
// scan of its own valences -- the global scan's values.  Per primitive and
// vertex the operations are those of k_adj_build, k_dual and k_primal, so
// the results are identical.
// ---------------------------------------------------------------------------
template <int MODE, int N>
__global__ void __launch_bounds__(chunk_sweep_threads<MODE>(), chunk_sweep_min_ctas<MODE>()) k_sweep_chunks(
    const ChunkDev* __restrict__ chunks, const uint32_t* __restrict__ tot, const int* __restrict__ order,
    int n_chunks, int* __restrict__ queue, const uint32_t* __restrict__ words, WordScratch ws,
    const uint32_t* __restrict__ vkey, int64_t nv, int64_t n_prims, int64_t adj_cap,
    const int64_t* __restrict__ d_counts, uint32_t* __restrict__ off, const uint8_t* __restrict__ valence,
    uint32_t* __restrict__ adj, const uint8_t* __restrict__ boundary, const uint32_t* __restrict__ idx,
    float* __restrict__ pos, float* __restrict__ nrm, float* __restrict__ dual_p, float* __restrict__ dual_n,
    int iters, int process_boundary, int sn, int wide_adj) {
  constexpr int kThreads = chunk_sweep_threads<MODE>(), kWarps = kThreads / 32;
  __shared__ SmemTabs T;
  __shared__ uint32_t s_warp[kWarps];
  __shared__ uint32_t s_total;
  __shared__ int s_item;
  load_tabs_some<false, false, MODE != 0, MODE == 0>(T);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t nvb = d_counts ? min(nv, d_counts[0]) : nv;
  const int64_t npb = d_counts ? min(n_prims, d_counts[1] / N) : n_prims;
  const int hard_norm_max = 10;
  const int max_norms = (iters / 2 - 3 < hard_norm_max ? iters / 2 - 3 : hard_norm_max);
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(queue, 1);
    __syncthreads();
    const int it = s_item;
    __syncthreads();  // everyone has read s_item before thread 0 takes the next
    if (it >= n_chunks) break;
    const int c = order[it];
    const ChunkDev& ch = chunks[c];
    const int64_t v0 = ch.vout, v1 = min(v0 + (int64_t)tot[2 * c], nvb);
    const int64_t p0 = ch.iout / N, p1 = min((ch.iout + (int64_t)tot[2 * c + 1]) / N, npb);
    // CSR offsets (MeshProcessor.cpp:32-40), blockDim vertices per pass;
    // vertex v is always handled by the same thread below
    uint32_t carry = (uint32_t)ch.iout;
    for (int64_t b = v0; b < v1; b += kThreads) {
      const int64_t v = b + threadIdx.x;
      const uint32_t x = v < v1 ? (uint32_t)__ldg(valence + v) : 0u;
      uint32_t incl = x;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += y;
      }
      if (lane == 31) s_warp[warp] = incl;
      __syncthreads();
      if (warp == 0) {
        const uint32_t w = lane < kWarps ? s_warp[lane] : 0u;
        uint32_t wi = w;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
          const uint32_t y = __shfl_up_sync(0xffffffffu, wi, d);
          if (lane >= d) wi += y;
        }
        if (lane < kWarps) s_warp[lane] = wi - w;  // exclusive over warps
        if (lane == kWarps - 1) s_total = wi;
      }
      __syncthreads();
      if (v < v1) off[v] = carry + s_warp[warp] + incl - x;
      carry += s_total;
      __syncthreads();
    }
    // adjacency, in each vertex's own CSR range and inside adj
    // a chunk of at most 65535 primitives keeps 16-bit chunk-relative ids, in
    // the first half of its own span of adj (its lists hold as many entries
    // as it has indices)
    const bool compact = !wide_adj && p1 - p0 <= 65535;
    uint16_t* adj16 = reinterpret_cast<uint16_t*>(adj + ch.iout);
    for (int64_t v = v0 + threadIdx.x; v < v1; v += kThreads) {
      const uint32_t o = off[v];
      const int room = (int)max((int64_t)0, min((int64_t)__ldg(valence + v), adj_cap - (int64_t)o));
      if (compact)
        adj_vertex<MODE, uint16_t>(T, ch, words, ws, __ldg(vkey + v), adj16 + (o - (uint32_t)ch.iout), room, p0);
      else
        adj_vertex<MODE>(T, ch, words, ws, __ldg(vkey + v), adj + o, room);
    }
    __syncthreads();
    // the sweeps in 32-bit chunk-relative indices over chunk-based pointers
    // (vertex ids, primitive ids and adjacency offsets stay mesh-wide)
    const uint32_t np_c = (uint32_t)max((int64_t)0, p1 - p0), nv_c = (uint32_t)max((int64_t)0, v1 - v0);
    const uint32_t nvb32 = (uint32_t)min(nvb, (int64_t)UINT32_MAX);
    const uint32_t npl32 = (uint32_t)min(n_prims, (int64_t)UINT32_MAX);
    const uint32_t* idx_c = idx + N * p0;
    float* dp_c = dual_p + 4 * p0;
    float* dn_c = dual_n + 2 * p0;
    const uint32_t* off_c = off + v0;
    const uint8_t* val_c = valence + v0;
    const uint8_t* bnd_c = boundary + v0;
    float* pos_c = pos + 3 * v0;
    float* nrm_c = nrm ? nrm + 3 * v0 : nullptr;
    for (int m = 0; m < iters; ++m) {
      const int normal_mode = !sn ? 0 : ((m == 0 || m < max_norms || m < 3) ? 1 : 2);
      const int set_colors = (m < iters - 1) ? ((m == 3) || (m == 0 && iters <= 3)) : 0;
      for (uint32_t t = threadIdx.x; t < np_c; t += kThreads)
        dual_prim<N, true, true>(t, nvb32, idx_c, pos, nrm, dp_c, dn_c, normal_mode);
      __syncthreads();
      if (compact) {
        for (uint32_t v = threadIdx.x; v < nv_c; v += kThreads)
          primal_vertex<true, true, uint32_t, uint16_t>(v, np_c, adj_cap, off_c, nullptr, val_c, adj, bnd_c, dp_c, dn_c,
                                                        pos_c, nrm_c, process_boundary, sn, set_colors, ch.iout);
      } else {
        for (uint32_t v = threadIdx.x; v < nv_c; v += kThreads)
          primal_vertex<true, true>(v, npl32, adj_cap, off_c, nullptr, val_c, adj, bnd_c, dual_p, dual_n, pos_c, nrm_c,
                                    process_boundary, sn, set_colors);
      }
      __syncthreads();
    }
  }
}

template <int MODE, int N>
static int sweep_chunks_grid() {
  static std::atomic<int> grid[64] = {};
  return per_device_once(grid, [](int dev) {
    int sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sweep_chunks<MODE, N>, chunk_sweep_threads<MODE>(), 0);
    return (sms > 0 ? sms : 1) * (per_sm > 0 ? per_sm : 1);
  });
}

void launch_sweep_chunks(const StructuredAdj& sa, int N, int64_t nv, int64_t n_prims, const int64_t* d_counts,
                         float* pos, float* nrm, const uint8_t* boundary, const uint8_t* valence,
                         const uint32_t* idx, int iters, int process_boundary, int smooth_normals,
                         const ProcessScratch& s, cudaStream_t st) {
  cudaMemsetAsync(sa.queue, 0, sizeof(int), st);
  const int64_t adj_cap = n_prims * N;
#define BMF_SWEEP_CHUNKS(M, NN)                                                                                 \
  k_sweep_chunks<M, NN><<<sweep_chunks_grid<M, NN>(), chunk_sweep_threads<M>(), 0, st>>>(                     \
      sa.chunks, sa.tot, sa.order, sa.n_chunks, sa.queue, sa.words, sa.ws, sa.vkey, nv, n_prims, adj_cap,        \
      d_counts, s.off, valence, s.adj, boundary, idx, pos, nrm, s.dual_p, s.dual_n, iters, process_boundary,      \
      smooth_normals, sa.wide_adj ? 1 : 0)
  if (sa.mode == 0) {
    if (N == 3) BMF_SWEEP_CHUNKS(0, 3); else BMF_SWEEP_CHUNKS(0, 4);
  } else {
    if (N == 3) BMF_SWEEP_CHUNKS(1, 3); else BMF_SWEEP_CHUNKS(1, 4);
  }
#undef BMF_SWEEP_CHUNKS
}

void launch_count(int mode, const ChunkDev* d_chunks, int n_chunks, const int* d_unit_start, int n_units,
                  const uint32_t* words, const uint32_t* flags, WordScratch ws, cudaStream_t st) {
  if (ws.clist) cudaMemsetAsync(ws.ccount, 0, sizeof(uint32_t), st);
  if (ws.exact) cudaMemsetAsync(ws.fcount, 0, sizeof(uint32_t), st);
  if (mode == 0) k_count<0><<<n_units, kCountThreads, 0, st>>>(d_chunks, n_chunks, d_unit_start, words, flags, ws);
  else k_count<1><<<n_units, kCountThreads, 0, st>>>(d_chunks, n_chunks, d_unit_start, words, flags, ws);
}

void launch_scan_chunks(const ChunkDev* d_chunks, int n_chunks, WordScratch ws, uint32_t* d_tot, cudaStream_t st,
                        const int* d_order) {
  k_scan_chunks<<<n_chunks, kScanThreads, 0, st>>>(d_chunks, ws, d_tot, d_order);
}

void launch_chunk_offsets(ChunkDev* d_chunks, int n_chunks, const uint32_t* d_tot, const uint32_t* flags,
                          int64_t vcap, int64_t icap, int64_t* d_info, int64_t* d_totals, cudaStream_t st) {
  k_chunk_offsets<<<1, 1024, 0, st>>>(d_chunks, n_chunks, d_tot, flags, vcap, icap, d_info, d_totals);
}

// k-th set bit (from 0) of m; m must have more than k set bits.
__device__ __forceinline__ int nth_set_bit(uint32_t m, int k) {
  int pos = 0, c = __popc(m & 0xFFFFu);
  if (k >= c) { k -= c; m >>= 16; pos += 16; }
  c = __popc(m & 0xFFu);
  if (k >= c) { k -= c; m >>= 8; pos += 8; }
  c = __popc(m & 0xFu);
  if (k >= c) { k -= c; m >>= 4; pos += 4; }
  c = __popc(m & 0x3u);
  if (k >= c) { k -= c; m >>= 2; pos += 2; }
  if (k >= (int)(m & 1u)) pos += 1;
  return pos;
}

// Corner mask of the cell at offset (ox, oy, oz) in {-1, 0} from sample
// (x, y, z), from the inside bits of lines (x-1+i, y-1+j) at samples z-1..z+1
// packed 3 bits per line at bit 3 (3i + j): corner (dx, dy, dz) is bit
// 3 (3 (1 + ox + dx) + 1 + oy + dy) + 1 + oz + dz.
__device__ __forceinline__ int packed_mask(uint32_t nbits, int ox, int oy, int oz) {
  const uint32_t b = nbits >> (3 * (3 * (1 + ox) + (1 + oy)) + 1 + oz);
  return (int)((b & 3u) | (((b >> 3) & 3u) << 2) | (((b >> 9) & 3u) << 4) | (((b >> 12) & 3u) << 6));
}

// Mode R emission over the busy-word list.  Each warp takes kTileWords list
// entries at a time and stages, per word, its neighbourhood (NbCache: the
// occupancy words of lines (x-1..x+2, y-1..y+2) in blocks zb-1..zb+1 and the
// scanned vertex bases of lines (x..x+1, y..y+1) in blocks zb..zb+1), its
// index base and its triangle-count planes in shared memory.  Then the tile's
// output is written in two flattened lists, so that every lane does the same
// work: one lane per vertex (the k-th vertex of a word is found from the
// popcounts of its crossing words; calculate_isovertex position, boundary,
// key, init_valence), then one lane per triangle (the k-th triangle of a word
// from its count planes; the cell's Marching-Cubes case and its three vertex
// ids, polygonize_cell order).  Ids and slots come from the scanned counts, so
// the output is exactly the reference's.  Every mask, valence and neighbour
// vertex id is read from shared memory; only the two endpoint densities of a
// vertex come from global memory.  Warps work on their own tiles with no
// block-wide barrier, so one warp's staging loads overlap the others' work.
constexpr int kTileWords = 16;
constexpr int kEmitWarps = 8;

// One 4-byte global -> shared copy in flight (cp.async; the staged pieces are
// 4-byte words of scattered lines, below the 16-byte unit of bulk copies), and
// the wait for all of a thread's copies.  BMF_EMIT_ASYNC 0 keeps plain loads.
#ifndef BMF_EMIT_ASYNC
#define BMF_EMIT_ASYNC 1
#endif
__device__ __forceinline__ void stage_async(uint32_t* dst, const uint32_t* src) {
#if BMF_EMIT_ASYNC
  const unsigned sa = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(src) : "memory");
#else
  *dst = __ldg(src);
#endif
}
__device__ __forceinline__ void stage_wait() {
#if BMF_EMIT_ASYNC
  asm volatile("cp.async.wait_all;\n" ::: "memory");
#endif
}

struct RTile {
  NbCache nb[kTileWords];
  uint32_t ib[kTileWords], p0[kTileWords], p1[kTileWords], p2[kTileWords];
  uint32_t X[kTileWords], Y[kTileWords], Z[kTileWords];
  int x[kTileWords], y[kTileWords], zb[kTileWords], dim[kTileWords], zc[kTileWords];
  int64_t cw[kTileWords], dens[kTileWords], vout[kTileWords], iout[kTileWords];
  float oy[kTileWords], sc[kTileWords];  // the chunk's y origin and scale (2D column fill)
  // per word, the crossing words of the owner lines (x + i, y + j), i, j in
  // {0, 1}: X and Y in blocks zb, zb + 1 ([i][j][b]) and Z in block zb -- what
  // a triangle's three vertex ids are counted from (tile_vertex_id)
  uint32_t ox_[kTileWords][8], oy_[kTileWords][8], oz_[kTileWords][4];
  int voff[kTileWords + 1], toff[kTileWords + 1];  // exclusive vertex / triangle offsets of the tile's words
};

// A crossing end's density: read from the fill's densities, or (2D heightmap
// column fill) computed from the sample's column height with the full fill's
// operations.
__device__ __forceinline__ float end_density(const WordScratch& ws, const float* D, int64_t cw, float oy, float sc,
                                             int dim, int x, int y, int z) {
  if (ws.cols2d) {
    const float py = oy + (float)y * sc;
    const float dy = py * ws.c2d_g;
    return -dy - __ldg(ws.cols2d + cw + (int64_t)x * dim + z) * ws.c2d_height;
  }
  return dens_at(D, dim, x, y, z);
}

// The tile word holding flattened item j: the last t < nt with off[t] <= j.
__device__ __forceinline__ int tile_word(const int* off, int nt, int j) {
  int t = 0;
#pragma unroll
  for (int s = kTileWords / 2; s > 0; s >>= 1)
    if (t + s < nt && off[t + s] <= j) t += s;
  return t;
}

// Chunk-local id of the vertex on the axis-a crossing owned by sample
// (x + i, y + j, zabs), i, j in {0, 1}, zabs in blocks zb, zb + 1 of tile word
// t: nb_vertex_id's count, from the word's staged owner-line crossing words.
__device__ __forceinline__ uint32_t tile_vertex_id(const RTile& R, int t, int i, int j, int zabs, int a) {
  const int b = (zabs >> 5) - R.zb[t], l = zabs & 31;
  const int q = i * 2 + j;
  const uint32_t X = R.ox_[t][q * 2 + b], Y = R.oy_[t][q * 2 + b], lt = lane_lt(l);
  uint32_t id = R.nb[t].vb[i * 4 + j * 2 + b] + __popc(X & lt) + __popc(Y & lt);
  if (l > 0) id += __popc(R.oz_[t][q] & lt);  // then b == 0
  if (a >= 1) id += (X >> l) & 1u;
  if (a >= 2) id += (Y >> l) & 1u;
  return id;
}

__global__ void __launch_bounds__(32 * kEmitWarps, 4) k_emit_words_r(const ChunkDev* __restrict__ chunks,
                                                                 const uint32_t* __restrict__ words,
                                                                 const float* __restrict__ dens, WordScratch ws,
                                                                 MeshOut out) {
  __shared__ uint64_t s_tri[256], s_uses[256];
  __shared__ RTile s_tiles[kEmitWarps];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) {
    s_tri[i] = __ldg(g_tri_cases + i);
    s_uses[i] = __ldg(g_edge_uses + i);
  }
  __syncthreads();
  const int64_t n = min((int64_t)*ws.ccount, ws.clist_cap);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  RTile& R = s_tiles[warp];
  const int64_t nwarps = (int64_t)gridDim.x * kEmitWarps;
  for (int64_t t0 = ((int64_t)blockIdx.x * kEmitWarps + warp) * kTileWords; t0 < n; t0 += nwarps * kTileWords) {
    const int nt = (int)min((int64_t)kTileWords, n - t0);
    // 1. the tile's words
    if (lane < nt) {
      const uint2 e = ws.clist[t0 + lane];
      const ChunkDev& ch = chunks[e.x];
      const int dim = ch.dim, zc = ch.zc, wi = (int)e.y;
      const int xy = wi / zc;
      R.zb[lane] = wi - xy * zc;
      R.y[lane] = xy % dim;
      R.x[lane] = xy / dim;
      R.dim[lane] = dim;
      R.zc[lane] = zc;
      R.cw[lane] = ch.words;
      R.dens[lane] = ch.dens;
      R.vout[lane] = ch.vout;
      R.iout[lane] = ch.iout;
      R.oy[lane] = ch.oy;
      R.sc[lane] = ch.scale;
    }
    __syncwarp();
    // 2. stage the neighbourhoods (zeros outside the chunk): one item per
    // (word, neighbour line) loads the line's blocks zb-1..zb+1; one item per
    // (word, owner line) its vertex bases in blocks zb, zb+1; one per word its
    // index base and count planes -- three loops, so a warp's lanes take the
    // same branch
    // (asynchronous global -> shared copies: a lane issues every copy of its
    // items and waits once, instead of a load-then-store per item)
    for (int k = lane; k < nt * 16; k += 32) {
      const int t = k >> 4, i = (k >> 2) & 3, j = k & 3;
      const int dim = R.dim[t], zc = R.zc[t], zb = R.zb[t];
      const int xx = R.x[t] - 1 + i, yy = R.y[t] - 1 + j;
      uint32_t* dst = R.nb[t].w + (i * 4 + j) * 3;
      if (xx < 0 || yy < 0 || xx >= dim || yy >= dim) {
        dst[0] = dst[1] = dst[2] = 0u;
      } else {
        const uint32_t* L = words + R.cw[t] + (xx * dim + yy) * zc + zb;
        if (zb > 0) stage_async(dst, L - 1); else dst[0] = 0u;
        stage_async(dst + 1, L);
        if (zb + 1 < zc) stage_async(dst + 2, L + 1); else dst[2] = 0u;
      }
    }
    for (int k = lane; k < nt * 4; k += 32) {
      const int t = k >> 2, l = k & 3;
      const int dim = R.dim[t], zc = R.zc[t], zb = R.zb[t];
      const int xx = R.x[t] + (l >> 1), yy = R.y[t] + (l & 1);
      uint32_t* dst = R.nb[t].vb + (l >> 1) * 4 + (l & 1) * 2;
      if (xx < dim && yy < dim) {
        const uint32_t* V = ws.vcnt + R.cw[t] + (xx * dim + yy) * zc + zb;
        stage_async(dst, V);
        if (zb + 1 < zc) stage_async(dst + 1, V + 1); else dst[1] = 0u;
      } else {
        dst[0] = dst[1] = 0u;
      }
    }
    if (lane < nt) {
      const int64_t wi = R.cw[lane] + (R.x[lane] * R.dim[lane] + R.y[lane]) * R.zc[lane] + R.zb[lane];
      stage_async(&R.ib[lane], ws.icnt + wi);
      stage_async(&R.p0[lane], ws.gpl + 3 * wi);
      stage_async(&R.p1[lane], ws.gpl + 3 * wi + 1);
      stage_async(&R.p2[lane], ws.gpl + 3 * wi + 2);
    }
    stage_wait();
    __syncwarp();
    // 3. per word: owned crossings, vertex count and triangle count (count
    // planes), scanned over the tile in one word (vertices low, triangles high)
    {
      uint32_t packed = 0u;
      if (lane < nt) {
        const NbCache& nb = R.nb[lane];
        const int dim = R.dim[lane], x = R.x[lane], y = R.y[lane], zb = R.zb[lane];
        const uint32_t wc = nb.w[(1 * 4 + 1) * 3 + 1];
        const uint32_t X = (x + 1 < dim) ? wc ^ nb.w[(2 * 4 + 1) * 3 + 1] : 0u;
        const uint32_t Y = (y + 1 < dim) ? wc ^ nb.w[(1 * 4 + 2) * 3 + 1] : 0u;
        uint32_t Z = wc ^ ((wc >> 1) | (nb.w[(1 * 4 + 1) * 3 + 2] << 31));
        const int valid = dim - 1 - 32 * zb;
        if (valid < 32) Z &= valid <= 0 ? 0u : ((1u << valid) - 1u);
        R.X[lane] = X;
        R.Y[lane] = Y;
        R.Z[lane] = Z;
        // the owner lines' crossing words, as nb_vertex_id forms them
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int i = q >> 1, j = q & 1;
#pragma unroll
          for (int b = 0; b < 2; ++b) {
            const uint32_t w0 = nb.w[((i + 1) * 4 + (j + 1)) * 3 + b + 1];
            R.ox_[lane][q * 2 + b] = (x + i + 1 < dim) ? w0 ^ nb.w[((i + 2) * 4 + (j + 1)) * 3 + b + 1] : 0u;
            R.oy_[lane][q * 2 + b] = (y + j + 1 < dim) ? w0 ^ nb.w[((i + 1) * 4 + (j + 2)) * 3 + b + 1] : 0u;
          }
          const uint32_t w0 = nb.w[((i + 1) * 4 + (j + 1)) * 3 + 1];
          uint32_t Zq = w0 ^ ((w0 >> 1) | (nb.w[((i + 1) * 4 + (j + 1)) * 3 + 2] << 31));
          if (valid < 32) Zq &= valid <= 0 ? 0u : ((1u << valid) - 1u);
          R.oz_[lane][q] = Zq;
        }
        const uint32_t nv = __popc(X) + __popc(Y) + __popc(Z);
        const uint32_t ntri = __popc(R.p0[lane]) + 2u * __popc(R.p1[lane]) + 4u * __popc(R.p2[lane]);
        packed = nv | (ntri << 16);  // at most 96 and 160 per word
      }
      uint32_t incl = packed;
#pragma unroll
      for (int o = 1; o < kTileWords; o <<= 1) {
        const uint32_t v = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += v;
      }
      if (lane < kTileWords) {
        R.voff[lane + 1] = (int)(incl & 0xFFFFu);
        R.toff[lane + 1] = (int)(incl >> 16);
      }
      if (lane == 0) R.voff[0] = R.toff[0] = 0;
    }
    __syncwarp();
    // 4. one lane per vertex: the k-th vertex of word t is at the cell l whose
    // preceding cells own k or fewer crossings, the (k - that)-th of its axes
    const int nvt = R.voff[nt];
    for (int j = lane; j < nvt; j += 32) {
      const int t = tile_word(R.voff, nt, j);
      const int k = j - R.voff[t];
      const uint32_t X = R.X[t], Y = R.Y[t], Z = R.Z[t];
      int l = 0;
#pragma unroll
      for (int s = 16; s > 0; s >>= 1) {
        const uint32_t m = lane_lt(l + s);
        if ((int)(__popc(X & m) + __popc(Y & m) + __popc(Z & m)) <= k) l += s;
      }
      const uint32_t lt = lane_lt(l);
      const int r = k - (int)(__popc(X & lt) + __popc(Y & lt) + __popc(Z & lt));
      uint32_t own = ((X >> l) & 1u) | (((Y >> l) & 1u) << 1) | (((Z >> l) & 1u) << 2);
      if (r >= 1) own &= own - 1u;
      if (r >= 2) own &= own - 1u;
      const int a = __ffs(own) - 1;
      const NbCache& nb = R.nb[t];
      const int64_t gv = R.vout[t] + (int64_t)nb.vb[0] + k;
      if (gv >= out.vcap) continue;
      const int dim = R.dim[t], x = R.x[t], y = R.y[t], z = 32 * R.zb[t] + l;
      const int x1 = x + (a == 0), y1 = y + (a == 1), z1 = z + (a == 2);
      const float* D = dens + R.dens[t];
      const int64_t cw = R.cw[t];
      const float oy = R.oy[t], sc = R.sc[t];
      const float s0 = end_density(ws, D, cw, oy, sc, dim, x, y, z);
      const float s1 = end_density(ws, D, cw, oy, sc, dim, x1, y1, z1);
      const float mu = (0.0f - s0) / (s1 - s0);
      const float q0[3] = {(float)x, (float)y, (float)z};
      const float dl[3] = {(float)(x1 - x), (float)(y1 - y), (float)(z1 - z)};
      float* P = out.pos + 3 * gv;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float dv = dl[c] * mu;
        P[c] = dv + q0[c];
      }
      if (out.boundary)
        out.boundary[gv] = (x == 0 || y == 0 || z == 0 || x == dim - 1 || y == dim - 1 || z == dim - 1 ||
                            x1 == dim - 1 || y1 == dim - 1 || z1 == dim - 1);
      if (out.nrm) { out.nrm[3 * gv] = 0.0f; out.nrm[3 * gv + 1] = 0.0f; out.nrm[3 * gv + 2] = 0.0f; }
      if (out.vkey) out.vkey[gv] = vertex_key(x, y, z, a);
      if (out.valence) {
        // inside bits of lines (x-1..x+1, y-1..y+1) at samples z-1..z+1
        uint32_t nbits = 0u;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int jj = 0; jj < 3; ++jj) {
            const int zr0 = l + 31, b = zr0 >> 5;  // z - 1 relative to block zb - 1
            const uint32_t* w = nb.w + (i * 4 + jj) * 3;
            const uint64_t q = ((uint64_t)w[b + 1] << 32) | w[b];
            nbits |= ((uint32_t)(q >> (zr0 & 31)) & 7u) << (3 * (3 * i + jj));
          }
        // init_valence: uses of this edge by the (up to) four interior cells
        // around it (polygonize skips far-face cells, DMCChunk.cpp:528)
        int val = 0;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          const int d1 = c >> 1, d2 = c & 1;
          const int ox = a == 0 ? 0 : -d1, oy = a == 0 ? -d1 : (a == 1 ? 0 : -d2), oz = a == 2 ? 0 : -d2;
          const int e = 4 * a + 2 * d1 + d2;
          const int cx = x + ox, cy = y + oy, cz = z + oz;
          if (cx < 0 || cy < 0 || cz < 0 || cx > dim - 2 || cy > dim - 2 || cz > dim - 2) continue;
          val += (int)((s_uses[packed_mask(nbits, ox, oy, oz)] >> (4 * e)) & 0xF);
        }
        out.valence[gv] = (uint8_t)val;
      }
    }
    // 5. one lane per triangle: the k-th triangle of word t is in the cell l
    // whose preceding cells hold k or fewer (count planes), its (k - that)-th
    const int ntt = R.toff[nt];
    for (int j = lane; j < ntt; j += 32) {
      const int t = tile_word(R.toff, nt, j);
      const int k = j - R.toff[t];
      const uint32_t c0 = R.p0[t], c1 = R.p1[t], c2 = R.p2[t];
      int l = 0;
#pragma unroll
      for (int s = 16; s > 0; s >>= 1) {
        const uint32_t m = lane_lt(l + s);
        if ((int)(__popc(c0 & m) + 2 * __popc(c1 & m) + 4 * __popc(c2 & m)) <= k) l += s;
      }
      const uint32_t lt = lane_lt(l);
      const int r = k - (int)(__popc(c0 & lt) + 2 * __popc(c1 & lt) + 4 * __popc(c2 & lt));
      const NbCache& nb = R.nb[t];
      // the cell's case: corner (dx, dy, dz) is bit 4 dx + 2 dy + dz
      int mask = 0;
#pragma unroll
      for (int d = 0; d < 4; ++d) {
        const uint32_t* w = nb.w + ((1 + (d >> 1)) * 4 + 1 + (d & 1)) * 3;
        const uint64_t q = ((uint64_t)w[2] << 32) | w[1];
        mask |= (int)((q >> l) & 3u) << (2 * d);
      }
      const uint64_t tw = s_tri[mask];
      if (3 * r + 3 > 3 * (int)(tw >> 60)) continue;  // the planes and the case table agree
      const int z = 32 * R.zb[t] + l;
      const int64_t gi = R.iout[t] + (int64_t)R.ib[t] + 3 * (int64_t)k;
      const int64_t vout = R.vout[t];
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const int e = tri_edge(tw, 3 * r + i);
        // EDGE_V owner of edge e: axis e >> 2, offsets from its two low bits
        const int ea = e >> 2, d1 = (e >> 1) & 1, d2 = e & 1;
        const int ox = ea == 0 ? 0 : d1, oy = ea == 0 ? d1 : (ea == 1 ? 0 : d2), oz = ea == 2 ? 0 : d2;
        const uint32_t vid = tile_vertex_id(R, t, ox, oy, z + oz, ea);
        if (gi + i < out.icap) {
          out.idx[gi + i] = vid;
          if (out.idx_global) out.idx_global[gi + i] = (uint32_t)(vout + vid);
        }
      }
    }
    __syncwarp();  // the next tile overwrites the stage
  }
}

// Mode Q emission over the work list, one thread per active cell: the cell's
// group vertices (ids from the word base and the group-count planes; mass
// point / centre placed here, QEF by k_place_qef when keys are kept) and the
// quads of the interior crossing edges its sample owns (slot from the word's
// index base and the popcounts of the owned crossings below it) -- exactly
// what k_emit<1,P> writes for the cell's lane.
template <int PLACE>
__global__ void __launch_bounds__(256, 3) k_emit_cells_q(const ChunkDev* __restrict__ chunks,
                                                         const uint32_t* __restrict__ words,
                                                         const float* __restrict__ dens, WordScratch ws, MeshOut out) {
  __shared__ SmemTabs T;
  load_tabs(T);
  const int64_t n = min((int64_t)*ws.ccount, ws.clist_cap);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const uint2 ent = ws.clist[i];
    const ChunkDev ch = chunks[ent.x];
    const int dim = ch.dim, zc = ch.zc;
    int x, y, z, k0;
    vertex_key_decode(ent.y, x, y, z, k0);
    const int zb = z >> 5, lane = z & 31;
    const uint32_t lt = lane_lt(lane);
    const uint32_t* W = words + ch.words;
    const uint32_t* vbase = ws.vcnt + ch.words;
    const float* D = dens + ch.dens;
    const int64_t wo = ((int64_t)x * dim + y) * zc + zb;
    const bool interior = x <= dim - 2 && y <= dim - 2 && z <= dim - 2;
    const int mask = interior ? cell_mask_at(W, dim, zc, x, y, z) : 0;
    const uint64_t gw = T.grp[mask];
    const int ng = (int)((gw >> 48) & 0xF);
    if (ng) {
      const uint32_t* pl = ws.gpl + 3 * (ch.words + wo);
      uint32_t vid = __ldg(vbase + wo) + __popc(__ldg(pl) & lt) + 2 * __popc(__ldg(pl + 1) & lt) +
                     4 * __popc(__ldg(pl + 2) & lt);
      const int nc = dim - 1;
      const uint8_t bnd = (x == 0 || y == 0 || z == 0 || x == nc - 1 || y == nc - 1 || z == nc - 1);
      for (int g = 0; g < ng; ++g, ++vid) {
        const int64_t gv = ch.vout + vid;
        if (gv >= out.vcap) continue;
        if (PLACE != 2 || !out.vkey) {
          float P[3];
          q_place<PLACE>(D, dim, x, y, z, mask, g, P);
          out.pos[3 * gv] = P[0];
          out.pos[3 * gv + 1] = P[1];
          out.pos[3 * gv + 2] = P[2];
        }
        if (out.nrm) { out.nrm[3 * gv] = 0.0f; out.nrm[3 * gv + 1] = 0.0f; out.nrm[3 * gv + 2] = 0.0f; }
        if (out.boundary) out.boundary[gv] = bnd;
        if (out.vkey) out.vkey[gv] = vertex_key(x, y, z, g);
        if (out.valence) {
          int val = 0;
          for (int e = 0; e < 12; ++e) {
            if ((int)((gw >> (4 * e)) & 0xF) != g) continue;
            const int c0 = edge_c0(e);
            val += q_edge_interior(dim, x + ((c0 >> 2) & 1), y + ((c0 >> 1) & 1), z + (c0 & 1), e >> 2);
          }
          out.valence[gv] = (uint8_t)val;
        }
      }
    }
    uint32_t Xi, Yi, Zi;
    q_quad_words(W, dim, zc, x, y, zb, Xi, Yi, Zi);
    const int own = (int)(((Xi >> lane) & 1u) | (((Yi >> lane) & 1u) << 1) | (((Zi >> lane) & 1u) << 2));
    if (!own) continue;
    int64_t gi = ch.iout + (int64_t)__ldg(ws.icnt + ch.words + wo) +
                 4 * (int64_t)(__popc(Xi & lt) + __popc(Yi & lt) + __popc(Zi & lt));
    const bool in0 = ((word_at(W, dim, zc, x, y, zb) >> lane) & 1u) != 0u;
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
        q[k] = q_vertex_base(vbase, ws.gpl + 3 * ch.words, dim, zc, cc[0], cc[1], cc[2]) +
               (uint32_t)((T.grp[cm] >> (4 * e)) & 0xF);
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

// Mode Q QEF placement, one thread per vertex (dense lanes, unlike the
// warp-per-word emit where only surface cells' lanes work): the same
// q_place<2> on the vertex's cell and group, decoded from its key.
__global__ void __launch_bounds__(128) k_place_qef(const ChunkDev* __restrict__ chunks, int n_chunks,
                                                   const uint32_t* __restrict__ words, const float* __restrict__ dens,
                                                   const uint32_t* __restrict__ vkey,
                                                   const int64_t* __restrict__ d_counts, int64_t vcap,
                                                   float* __restrict__ pos, uint8_t* __restrict__ qflag,
                                                   uint32_t* __restrict__ qlist, uint32_t* __restrict__ qcount,
                                                   float* __restrict__ qseed) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= min(vcap, d_counts[0])) return;
  const int c = find_chunk_by_vertex(chunks, n_chunks, v);
  const ChunkDev ch = chunks[c];
  const int dim = ch.dim;
  int x, y, z, g;
  vertex_key_decode(vkey[v], x, y, z, g);
  const int mask = cell_mask_at(words + ch.words, dim, ch.zc, x, y, z);
  float P[3];
  if (qflag) {
    // record the branch, and for a QEF-placed vertex its FP32 eigenvectors
    // (the seeds of the wide adjoint), in the list of QEF-placed vertices
    QefSolveInfo info;
    bool used = false;
    q_place<2>(dens + ch.dens, dim, x, y, z, mask, g, P, &info, &used);
    qflag[v] = used ? 1 : 0;
    if (used) {
      const uint32_t k = atomicAdd(qcount, 1u);
      qlist[k] = (uint32_t)v;
#pragma unroll
      for (int r = 0; r < 3; ++r) {
#pragma unroll
        for (int c3 = 0; c3 < 3; ++c3) qseed[9 * (int64_t)k + 3 * r + c3] = info.V[r][c3];
      }
    }
  } else {
    q_place<2>(dens + ch.dens, dim, x, y, z, mask, g, P);
  }
  pos[3 * v] = P[0];
  pos[3 * v + 1] = P[1];
  pos[3 * v + 2] = P[2];
}

int launch_emit(int mode, int placement, const ChunkDev* d_chunks, int n_chunks, const int* d_unit_start,
                int n_units, const uint32_t* words, const float* dens, const uint32_t* flags, WordScratch ws,
                MeshOut out, const int64_t* d_counts, cudaStream_t st) {
  if (mode == 0 && ws.clist) {
    // persistent: one wave of resident CTAs
    static std::atomic<int> grid[64] = {};
    const int g = per_device_once(grid, [](int dev) {
      int sms = 0, per_sm = 0;
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_emit_words_r, 32 * kEmitWarps, 0);
      return (sms > 0 ? sms : 1) * (per_sm > 0 ? per_sm : 1);
    });
    k_emit_words_r<<<g, 32 * kEmitWarps, 0, st>>>(d_chunks, words, dens, ws, out);
  } else if (mode == 0) {
    k_emit<0, 0><<<n_units, 256, 0, st>>>(d_chunks, n_chunks, d_unit_start, words, dens, flags, ws, out);
  } else if (ws.clist) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (placement == 2 && (!out.vkey || !d_counts)) out.vkey = nullptr;
    if (placement == 0) k_emit_cells_q<0><<<sms * 8, 256, 0, st>>>(d_chunks, words, dens, ws, out);
    else if (placement == 1) k_emit_cells_q<1><<<sms * 8, 256, 0, st>>>(d_chunks, words, dens, ws, out);
    else k_emit_cells_q<2><<<sms * 8, 256, 0, st>>>(d_chunks, words, dens, ws, out);
    if (placement == 2 && out.vkey && out.vcap > 0) {
      if (out.qflag) cudaMemsetAsync(out.qcount, 0, sizeof(uint32_t), st);
      k_place_qef<<<(int)((out.vcap + 127) / 128), 128, 0, st>>>(d_chunks, n_chunks, words, dens, out.vkey, d_counts,
                                                                out.vcap, out.pos, out.qflag, out.qlist, out.qcount,
                                                                out.qseed);
      return 2;
    }
  } else if (placement == 0) {
    k_emit<1, 0><<<n_units, 256, 0, st>>>(d_chunks, n_chunks, d_unit_start, words, dens, flags, ws, out);
  } else if (placement == 1) {
    k_emit<1, 1><<<n_units, 256, 0, st>>>(d_chunks, n_chunks, d_unit_start, words, dens, flags, ws, out);
  } else {
    if (!out.vkey || !d_counts) out.vkey = nullptr;  // no keys: the emit places in place
    k_emit<1, 2><<<n_units, 256, 0, st>>>(d_chunks, n_chunks, d_unit_start, words, dens, flags, ws, out);
    if (out.vkey && out.vcap > 0) {
      if (out.qflag) cudaMemsetAsync(out.qcount, 0, sizeof(uint32_t), st);
      k_place_qef<<<(int)((out.vcap + 127) / 128), 128, 0, st>>>(d_chunks, n_chunks, words, dens, out.vkey, d_counts,
                                                                out.vcap, out.pos, out.qflag, out.qlist, out.qcount,
                                                                out.qseed);
      return 2;
    }
  }
  return 1;
}

}  // namespace bmf
