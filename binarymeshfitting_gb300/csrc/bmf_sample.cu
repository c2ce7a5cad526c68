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

constexpr int kMaxColumn = 1024;  // samples per axis (kMaxDim)
constexpr int kColumnItem = 256;  // columns per k_columns2d CTA

// flags bits: 1 = a word that is neither empty nor full, 2 = a full word,
// 4 = an empty word.  contains_mesh = (f & 1) || ((f & 6) == 6), the
// reference's mesh / negative / positive logic (DMCChunk.cpp:141-162).
__global__ void __launch_bounds__(256) k_sample_label(const ChunkDev* __restrict__ chunks, int n_chunks,
                                                      const int* __restrict__ unit_start, FieldDev field,
                                                      const float* __restrict__ dens_in, float* __restrict__ dens_out,
                                                      uint32_t* __restrict__ words, uint32_t* __restrict__ flags,
                                                      const float* __restrict__ cols) {
  extern __shared__ uint32_t sw[];
  __shared__ int perm2[512];
  __shared__ float4 gtab[512];
  // BMF_FIELD_TERRAIN_2D: the height noise of the plane's (x, z) columns,
  // evaluated here or (cols non-null) read from k_columns2d's output
  __shared__ float s_col[kMaxColumn];
  const int u = blockIdx.x;
  const int c = find_chunk(unit_start, n_chunks, u);
  const ChunkDev ch = chunks[c];
  const int x = u - __ldg(unit_start + c);
  const int dim = ch.dim, zc = ch.zc;
  const int nw = dim * zc;
  if (field.kind == BMF_FIELD_TERRAIN_FBM || field.kind == BMF_FIELD_TERRAIN_2D) {  // the noise tables
    for (int i = threadIdx.x; i < 512; i += blockDim.x) {
      perm2[i] = field.perm[i & 255];
      gtab[i] = grad_coeffs(field.perm[i & 255]);
    }
  }
  for (int i = threadIdx.x; i < nw; i += blockDim.x) sw[i] = 0u;
  __syncthreads();
  const bool col2d = field.kind == BMF_FIELD_TERRAIN_2D && dim <= kMaxColumn;
  if (col2d) {  // one height evaluation per column, shared by the plane's dim samples of it
    const float pxc = ch.ox + (float)x * ch.scale;
    for (int z = threadIdx.x; z < dim; z += blockDim.x)
      s_col[z] = cols ? __ldg(cols + ch.words + (int64_t)x * dim + z)
                      : terrain2d_height(field, perm2, pxc, ch.oz + (float)z * ch.scale);
    __syncthreads();
  }

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
        terrain_run(field, perm2, gtab, px, py, pz, n, v);
      } else if (col2d) {
#pragma unroll
        for (int k = 0; k < kRun; ++k)
          if (k < n) v[k] = terrain2d_density(field, py, s_col[z0 + k]);
      } else {
#pragma unroll
        for (int k = 0; k < kRun; ++k)
          if (k < n) v[k] = eval_field(field, perm2, gtab, px, py, pz[k]);
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

// ---------------------------------------------------------------------------
// Terrain FBM fill over (x, y) lines: the work item is kFillLines consecutive
// lines of one chunk (line = x * dim + y); each thread owns one line and walks
// it in runs of kFillRun z-samples.  All threads of an item share the run's z
// coordinates, so everything that depends on z alone -- the lattice cell Z,
// the fraction zf, zf - 1 and fade(zf), per octave and sample -- is computed
// once per CTA into shared memory, and the z-lattice cell changes at the same
// sample for every lane (a warp-uniform branch).
//
// The noise is the line-separable form of bmf_device.cuh: per octave a
// sample costs l0 = alpha0 + beta0 * zf, l1 = alpha1 + beta1 * (zf - 1),
// l0 + w (l1 - l0) and the accumulation, nine FP32 operations.  alpha / beta
// change only when the lattice cell Z does; when Z advances by one, the old
// layer-1 pair becomes the new layer-0 pair and only layer 1 is set up.
//
// Items come from a device queue (persistent CTAs grab the next item with an
// atomic ticket; the queue is ordered largest chunks first) or, with no queue,
// one CTA per item.
// ---------------------------------------------------------------------------
// RUN (z-samples per step; 4, 8 or 16, dividing 16 so that a run's inside
// bits land in one word and its densities in one staged half block) is the
// tile height the batch autotuner picks.
constexpr int kFillLines = 256; // lines per item = threads per CTA
constexpr int kMaxOctaves = 32;
constexpr int kMaxFillRun = 16;
// z terms {zf, zf - 1, fade(zf), Z} per (octave, z): for every z of the
// item's lines at once when octaves * dim fit, else per run
constexpr int kZtEntries = 1024;
static_assert(kZtEntries >= kMaxOctaves * kMaxFillRun, "per-run z terms fit");

// Per (line, octave) state of the line walk: the x/y terms, the four hash
// bases, and the alpha / beta pairs of the current z-lattice cell Zp.
struct OctLine {
  float xf, yf, u, v, a0, b0, a1, b1;
  int pA, pA1, pB, pB1;
  int Zp;
};

__device__ __forceinline__ void oct_line_init(OctLine& s, float px, float py, float fr,
                                              const int* __restrict__ perm2) {
  const float xs = px * fr, ys = py * fr;
  const float fx = floorf(xs), fy = floorf(ys);
  const int X = ((int)fx) & 255, Y = ((int)fy) & 255;
  s.xf = xs - fx;
  s.yf = ys - fy;
  s.u = fade(s.xf);
  s.v = fade(s.yf);
  const int A = perm2[X] + Y, B = perm2[X + 1] + Y;
  s.pA = perm2[A];
  s.pA1 = perm2[A + 1];
  s.pB = perm2[B];
  s.pB1 = perm2[B + 1];
  s.Zp = -1;
}

// Enter z-lattice cell Z: when it is the next cell, the old layer-1 pair is
// the new layer-0 pair; otherwise both layers are set up.
__device__ __forceinline__ void oct_line_cell(OctLine& s, int Z, const float4* __restrict__ gtab) {
  const int pA = s.pA, pA1 = s.pA1, pB = s.pB, pB1 = s.pB1;
  const float x1 = s.xf - 1.0f, y1 = s.yf - 1.0f;
  if (s.Zp >= 0 && Z == ((s.Zp + 1) & 255)) {
    s.a0 = s.a1;
    s.b0 = s.b1;
  } else {
    layer_coeffs(gtab, pA + Z, pB + Z, pA1 + Z, pB1 + Z, s.xf, s.yf, x1, y1, s.u, s.v, s.a0, s.b0);
  }
  const int Z1 = Z + 1;
  layer_coeffs(gtab, pA + Z1, pB + Z1, pA1 + Z1, pB1 + Z1, s.xf, s.yf, x1, y1, s.u, s.v, s.a1, s.b1);
  s.Zp = Z;
}

// Band fill (BAND = true).  The terrain density is d = (py - h) - a * FBM with
// py constant along a line, and every octave's noise is bounded: at offsets
// (u, v, w) in the lattice cell the corner weights W_c (products of fade and
// 1 - fade) are non-negative and sum to one, and a corner's gradient has two
// components +/-1 and one 0, so its dot product is at most m_c, the sum of the
// two largest of |u - cx|, |v - cy|, |w - cz|; hence |noise| <= F(u, v, w) =
// sum_c W_c m_c.  Each partial derivative of F is at most fade' + 1 <= 2.875
// in magnitude, so F is at most its maximum over a grid of spacing h plus
// 4.3125 h: 1.0364 + 0.0216 on a 201^3 grid (recomputed by the test suite),
// below kNoiseBound = 1.0625.  Before each
// octave o a run therefore knows its FBM sums to within
// T_o = kNoiseBound * sum_{j >= o} |amp_j|: when every sample's partial sum S lies
// below (py - h) / a - T_o (all outside) or above (py - h) / a + T_o (all
// inside), the signs -- the occupancy words -- are final and the run stops.
// Its samples then hold the partial density (right sign, inexact value) and
// clear their bits in the `exact` mask (laid out like the words); the mesh
// only reads densities at the ends of sign-changing edges, and
// k_fill_fixup recomputes those that are inexact before the emit runs, with
// the same operations, so the output is bit-identical to a full fill.
// Lanes take the lines of an item y-major (x fastest), so a warp's lanes
// share py and mostly stop at the same octave.
#ifndef BMF_BAND_CTAS
#define BMF_BAND_CTAS 3
#endif
constexpr int kBandCtas = BMF_BAND_CTAS;  // resident CTAs per SM the band fill's registers are sized for
constexpr float kNoiseBound = 1.0625f;  // |improved noise| <= 1.058 (above)
constexpr float kBandMargin = 1e-3f;  // float rounding of the sums, far below this

// Dynamic shared memory: the density stage (16-sample half blocks of the
// CTA's lines, rows padded to 17 floats; not used by the band fill, which
// stores only its exact runs, straight from registers) and, for up to
// kCacheOctaves octaves, each line's lattice-cell state (alpha / beta pairs
// and Zp) carried from one run to the next, so a run re-enters a cell only
// when Z changes.
constexpr int kStageRow = 17;
constexpr int kCacheOctaves = 8;
constexpr size_t kStageFloats = (size_t)kFillLines * kStageRow;
__host__ __device__ constexpr size_t fill_smem_bytes(int octaves, bool band) {
  return (band ? 0 : sizeof(float) * kStageFloats) +
         (octaves <= kCacheOctaves ? (size_t)octaves * kFillLines * (sizeof(float4) + sizeof(int)) : 0);
}

template <int kFillRun, bool BAND>
__global__ void __launch_bounds__(kFillLines, BAND ? kBandCtas : 3) k_fill_terrain(const ChunkDev* __restrict__ chunks,
                                                             const int2* __restrict__ items, int n_items,
                                                             int* __restrict__ queue, FieldDev field,
                                                             float* __restrict__ dens_out,
                                                             uint32_t* __restrict__ words,
                                                             uint32_t* __restrict__ flags,
                                                             uint32_t* __restrict__ exact) {
  __shared__ int perm2[512];
  __shared__ float4 gtab[512];
  __shared__ float4 zt[kZtEntries];
  __shared__ float s_tail[kMaxOctaves + 1];  // band test: T_o + margin
  // density of the CTA's lines for one 16-sample half block, flushed with
  // coalesced 64-byte row stores (rows padded to 17: conflict-free columns)
  extern __shared__ float4 s_dyn[];
  float* s_stage = reinterpret_cast<float*>(s_dyn);
  __shared__ int s_item;
  for (int i = threadIdx.x; i < 512; i += blockDim.x) {
    perm2[i] = field.perm[i & 255];
    gtab[i] = grad_coeffs(field.perm[i & 255]);
  }
  const int oct = min((int)field.p[5], kMaxOctaves);
  const float h0 = field.p[0], ampl = field.p[1], freq = field.p[2], lac = field.p[3], gain = field.p[4];
  const bool cache = oct <= kCacheOctaves;
  float4* s_ab = s_dyn + (BAND ? 0 : kStageFloats / 4);          // [octave][line]: a0, b0, a1, b1
  int* s_zp = reinterpret_cast<int*>(s_ab + (size_t)oct * kFillLines);  // [octave][line]: Zp
  if (BAND && threadIdx.x == 0) {
    // T_o = kNoiseBound sum_{j >= o} |amp_j|: the total, then less one octave at a
    // time (rounding far below the margin)
    float tot = 0.0f, a = 1.0f;
    for (int o = 0; o < oct; ++o, a = a * gain) tot += fabsf(a) * kNoiseBound;
    a = 1.0f;
    for (int o = 0; o < oct; ++o, a = a * gain) {
      s_tail[o] = tot + kBandMargin;
      tot -= fabsf(a) * kNoiseBound;
    }
    s_tail[oct] = kBandMargin;
  }
  for (int pass = 0;; ++pass) {
    __syncthreads();
    if (threadIdx.x == 0) s_item = queue ? atomicAdd(queue, 1) : (pass == 0 ? (int)blockIdx.x : n_items);
    __syncthreads();
    const int it = s_item;
    if (it >= n_items) break;
    const int2 item = items ? items[it] : make_int2(0, it * kFillLines);
    const ChunkDev ch = chunks[item.x];
    const int dim = ch.dim, zc = ch.zc;
    // the thread's line: item.y + thread in x-major order (line = x * dim + y),
    // or, for the band fill, in y-major order (x fastest: a warp shares y)
    const int lidx = item.y + (int)threadIdx.x;
    const bool active = lidx < dim * dim;
    int x = 0, y = 0;
    if (active) {
      if (BAND) {
        y = lidx / dim;
        x = lidx - y * dim;
      } else {
        x = lidx / dim;
        y = lidx - x * dim;
      }
    }
    const int line = x * dim + y;  // in memory
    const float px = ch.ox + (float)x * ch.scale, py = ch.oy + (float)y * ch.scale;
    uint32_t* wline = words + ch.words + (int64_t)line * zc;
    uint32_t* eline = BAND ? exact + ch.words + (int64_t)line * zc : nullptr;
    // band test of this line: S below ca - tail (all outside) or above ca + tail (all inside)
    const float ca = BAND ? (py - h0) / ampl : 0.0f;
    const float caM = BAND ? 1e-6f * fabsf(ca) : 0.0f;
    if (BAND && cache) {  // no cell state carried in from the previous item
      for (int o = 0; o < oct; ++o) s_zp[o * kFillLines + (int)threadIdx.x] = -1;
    }
    // the z terms depend on the chunk only: all of them once per item when they fit
    const bool whole = oct * dim <= kZtEntries;
    // dim = RUN k + 1 (33, 65, 129, ...): the line's last sample is evaluated
    // in its last full run instead of a one-sample run that would set up every
    // octave's line state again (needs the z terms of every sample resident)
    const bool fold = whole && dim > kFillRun && (dim - 1) % kFillRun == 0;
    const int nruns = fold ? (dim - 1) / kFillRun : (dim + kFillRun - 1) / kFillRun;
    if (whole) {
      for (int e = threadIdx.x; e < oct * dim; e += blockDim.x) {
        const int o = e / dim, z = e - o * dim;
        float fr = freq;
        for (int i = 0; i < o; ++i) fr = fr * lac;
        const float pz = ch.oz + (float)z * ch.scale;
        const float zs = pz * fr;
        const float fz = floorf(zs);
        const float zf = zs - fz;
        zt[e] = make_float4(zf, zf - 1.0f, fade(zf), __int_as_float(((int)fz) & 255));
      }
    }
    uint32_t wacc = 0u, eacc = 0u, fl = 0u;
    for (int zr = 0; zr < nruns; ++zr) {
      const int z0 = zr * kFillRun, n = min(kFillRun, dim - z0);
      if (!whole || zr == 0) __syncthreads();
      if (!whole && (int)threadIdx.x < oct * kFillRun) {
        const int o = threadIdx.x / kFillRun, k = threadIdx.x % kFillRun;
        float fr = freq;
        for (int i = 0; i < o; ++i) fr = fr * lac;
        const float pz = ch.oz + (float)(z0 + k) * ch.scale;
        const float zs = pz * fr;
        const float fz = floorf(zs);
        const float zf = zs - fz;
        zt[threadIdx.x] = make_float4(zf, zf - 1.0f, fade(zf), __int_as_float(((int)fz) & 255));
      }
      if (!whole) __syncthreads();
      // z terms of (octave o, sample k of this run)
      const int zt_o = whole ? dim : kFillRun, zt_k = whole ? z0 : 0;
      if (active) {
      uint32_t bits = 0u;
      float* row = s_stage + threadIdx.x * kStageRow + (z0 & 15);
      float* grow = BAND ? dens_out + ch.dens + (int64_t)line * dim + z0 : nullptr;  // band: direct stores
      const bool tail = fold && zr == nruns - 1;  // sample z0 + RUN too
      uint32_t tail_bit = 0u;
      bool run_exact = true;
      if (n == kFillRun) {
        // a full run: RUN samples per octave, unrolled, no tail guards
        float sum[kFillRun], sum_t = 0.0f;
#pragma unroll
        for (int k = 0; k < kFillRun; ++k) sum[k] = 0.0f;
        float amp = 1.0f, fr = freq;
        // band: the whole line may be decided before any octave
        const int o_end = (BAND && (ca - s_tail[0] - caM > 0.0f || ca + s_tail[0] + caM < 0.0f)) ? 0 : oct;
        if (BAND && o_end == 0) run_exact = false;
#pragma unroll 1
        for (int o = 0; o < o_end; ++o) {
          OctLine L;
          oct_line_init(L, px, py, fr, perm2);
          const int si = o * kFillLines + (int)threadIdx.x;
          if (cache && zr > 0) {  // the cell this line was in at the end of its previous run
            const float4 ab = s_ab[si];
            L.a0 = ab.x;
            L.b0 = ab.y;
            L.a1 = ab.z;
            L.b1 = ab.w;
            L.Zp = s_zp[si];
          }
          const float4* zo = zt + o * zt_o + zt_k;
          float4 tn = zo[0];
#pragma unroll
          for (int k = 0; k < kFillRun; ++k) {
            // the next sample's z terms load before this sample's cell set-up
            const float4 t = tn;
            if (k + 1 < kFillRun) tn = zo[k + 1];
            const int Z = __float_as_int(t.w);
            if (Z != L.Zp) oct_line_cell(L, Z, gtab);  // same for every lane of the CTA
            const float l0 = __fmaf_rn(L.b0, t.x, L.a0);
            const float l1 = __fmaf_rn(L.b1, t.y, L.a1);
            sum[k] = __fmaf_rn(amp, __fmaf_rn(t.z, l1 - l0, l0), sum[k]);
          }
          if (tail) {  // the same operations as the sample's own run would do
            const float4 t = zo[kFillRun];
            const int Z = __float_as_int(t.w);
            if (Z != L.Zp) oct_line_cell(L, Z, gtab);
            const float l0 = __fmaf_rn(L.b0, t.x, L.a0);
            const float l1 = __fmaf_rn(L.b1, t.y, L.a1);
            sum_t = __fmaf_rn(amp, __fmaf_rn(t.z, l1 - l0, l0), sum_t);
          }
          if (cache) {
            s_ab[si] = make_float4(L.a0, L.b0, L.a1, L.b1);
            s_zp[si] = L.Zp;
          }
          if (BAND && o + 1 < oct) {
            // every sample decided by octaves 0..o: the rest cannot change a sign
            float mn = sum[0], mx = sum[0];
#pragma unroll
            for (int k = 1; k < kFillRun; ++k) {
              mn = fminf(mn, sum[k]);
              mx = fmaxf(mx, sum[k]);
            }
            if (tail) {
              mn = fminf(mn, sum_t);
              mx = fmaxf(mx, sum_t);
            }
            const float tb = s_tail[o + 1] + caM;
            if (mx < ca - tb || mn > ca + tb) {
              run_exact = false;
              break;
            }
          }
          fr = fr * lac;
          amp = amp * gain;
        }
#pragma unroll
        for (int k = 0; k < kFillRun; ++k) {
          const float d = __fmaf_rn(-ampl, sum[k], py - h0);
          if (!BAND)
            row[k] = d;
          else if (run_exact)  // a decided run's inexact densities are never read: not stored
            grow[k] = d;
          if (d < 0.0f) bits |= 1u << k;
        }
        if (tail) {  // outside the staged half block: stored directly
          const float d = __fmaf_rn(-ampl, sum_t, py - h0);
          if (dens_out && (!BAND || run_exact)) dens_out[ch.dens + (int64_t)line * dim + z0 + kFillRun] = d;
          tail_bit = d < 0.0f ? 1u : 0u;
        }
      } else {
        // the line's last, partial run: one sample at a time (same operations
        // in the same order per sample; its cell state is not needed after it)
#pragma unroll 1
        for (int k = 0; k < n; ++k) {
          float sum = 0.0f, amp = 1.0f, fr = freq;
#pragma unroll 1
          for (int o = 0; o < oct; ++o) {
            OctLine L;
            oct_line_init(L, px, py, fr, perm2);
            const int si = o * kFillLines + (int)threadIdx.x;
            if (cache && (zr > 0 || k > 0)) {
              const float4 ab = s_ab[si];
              L.a0 = ab.x;
              L.b0 = ab.y;
              L.a1 = ab.z;
              L.b1 = ab.w;
              L.Zp = s_zp[si];
            }
            const float4 t = zt[o * zt_o + zt_k + k];
            const int Z = __float_as_int(t.w);
            if (Z != L.Zp) oct_line_cell(L, Z, gtab);
            const float l0 = __fmaf_rn(L.b0, t.x, L.a0);
            const float l1 = __fmaf_rn(L.b1, t.y, L.a1);
            sum = __fmaf_rn(amp, __fmaf_rn(t.z, l1 - l0, l0), sum);
            if (cache && k + 1 < n) {
              s_ab[si] = make_float4(L.a0, L.b0, L.a1, L.b1);
              s_zp[si] = L.Zp;
            }
            fr = fr * lac;
            amp = amp * gain;
          }
          const float d = __fmaf_rn(-ampl, sum, py - h0);
          if (BAND)
            grow[k] = d;
          else
            row[k] = d;
          if (d < 0.0f) bits |= 1u << k;
        }
      }
      wacc |= bits << (z0 & 31);
      const uint32_t ebits = run_exact ? (n >= 32 ? kFull : ((1u << n) - 1u)) : 0u;
      if (BAND) eacc |= ebits << (z0 & 31);
      const int tz = z0 + kFillRun;  // the folded sample, in this word or the next
      if (tail && (tz & 31) != 0) {
        wacc |= tail_bit << (tz & 31);
        if (BAND && run_exact) eacc |= 1u << (tz & 31);
      }
      if (((z0 + kFillRun) & 31) == 0 || zr == nruns - 1) {
        wline[z0 >> 5] = wacc;
        if (BAND) eline[z0 >> 5] = eacc;
        fl |= (wacc != 0u && wacc != kFull) ? 1u : (wacc == kFull ? 2u : 4u);
        wacc = 0u;
        eacc = 0u;
      }
      if (tail && (tz & 31) == 0) {
        wline[tz >> 5] = tail_bit;
        if (BAND) eline[tz >> 5] = run_exact ? 1u : 0u;
        fl |= tail_bit ? 1u : 4u;  // a one-sample word: any value but all-ones
      }
      }  // active
      if (!BAND && dens_out && (((z0 + kFillRun) & 15) == 0 || zr == nruns - 1)) {
        // flush the half block: warp w writes rows [32w, 32w + 32), two
        // 16-sample row segments per instruction
        __syncthreads();
        const int zh0 = z0 & ~15, nz = min(16, dim - zh0);
        const int lane = threadIdx.x & 31, col = lane & 15;
        const int l0 = (int)(threadIdx.x & ~31) + (lane >> 4);  // this lane's first row
        // rows left for this lane (every second row from l0), 0 past the chunk's lines or columns
        const int nrow = col < nz ? min(16, (dim * dim - item.y - l0 + 1) >> 1) : 0;
        const float* sp = s_stage + l0 * kStageRow + col;
        float* gp = dens_out + ch.dens + (int64_t)(item.y + l0) * dim + zh0 + col;
#pragma unroll 4
        for (int j = 0; j < 16; ++j) {
          if (j < nrow) *gp = sp[2 * kStageRow * j];
          gp += 2 * dim;
        }
        __syncthreads();  // the next half block's rows overwrite the stage
      }
    }
    fl = __reduce_or_sync(kFull, fl);
    if ((threadIdx.x & 31) == 0 && fl) atomicOr(flags + item.x, fl);
    if (!queue) break;
  }
}


// The kernels' static + staging shared memory exceeds the 48 KB default: opt
// in once per device.
static void fill_terrain_smem_optin() {
  static std::atomic<int> done[64] = {};
  per_device_once(done, [](int) {
    const int mx = (int)fill_smem_bytes(kCacheOctaves, false);
    cudaFuncSetAttribute(k_fill_terrain<4, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_fill_terrain<8, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_fill_terrain<16, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_fill_terrain<4, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_fill_terrain<8, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    cudaFuncSetAttribute(k_fill_terrain<16, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    return 1;
  });
}

template <bool BAND>
static void fill_terrain_run(int run, int g, size_t sm, cudaStream_t st, const ChunkDev* d_chunks,
                             const int2* d_items, int n_items, int* d_queue, const FieldDev& field, float* dens_out,
                             uint32_t* words, uint32_t* flags, uint32_t* exact) {
  if (run == 4)
    k_fill_terrain<4, BAND><<<g, kFillLines, sm, st>>>(d_chunks, d_items, n_items, d_queue, field, dens_out, words,
                                                       flags, exact);
  else if (run == 16)
    k_fill_terrain<16, BAND><<<g, kFillLines, sm, st>>>(d_chunks, d_items, n_items, d_queue, field, dens_out, words,
                                                        flags, exact);
  else
    k_fill_terrain<8, BAND><<<g, kFillLines, sm, st>>>(d_chunks, d_items, n_items, d_queue, field, dens_out, words,
                                                       flags, exact);
}

void launch_fill_terrain(int run, const ChunkDev* d_chunks, const int2* d_items, int n_items, int* d_queue,
                         int grid, const FieldDev& field, float* dens_out, uint32_t* words, uint32_t* flags,
                         uint32_t* exact, cudaStream_t st) {
  if (n_items <= 0) return;
  if (d_queue) cudaMemsetAsync(d_queue, 0, sizeof(int), st);
  const int g = d_queue ? grid : n_items;
  fill_terrain_smem_optin();
  const bool band = exact && dens_out;
  const size_t sm = fill_smem_bytes(min((int)field.p[5], kMaxOctaves), band);
  if (band)
    fill_terrain_run<true>(run, g, sm, st, d_chunks, d_items, n_items, d_queue, field, dens_out, words, flags, exact);
  else
    fill_terrain_run<false>(run, g, sm, st, d_chunks, d_items, n_items, d_queue, field, dens_out, words, flags,
                            nullptr);
}

bool fill_band_supported(const FieldDev& field) {
  return (field.kind == BMF_FIELD_TERRAIN_FBM && field.p[1] > 0.0f) || field.kind == BMF_FIELD_TERRAIN_2D;
}

// ---------------------------------------------------------------------------
// Exact densities where the band fill left a decided sample inexact but the
// mesh reads it: the two ends of every sign-changing grid edge.  k_count
// lists those samples ({chunk, sample index}); one thread per listed sample.
// A sample at the end of several crossings may be listed more than once;
// every copy stores the same value.
// ---------------------------------------------------------------------------
// The exact terrain density of one sample: per octave the line's x/y terms,
// the z terms and both z-layers of its lattice cell, combined with the
// operations of k_fill_terrain's run loop, in the same order.
__device__ float terrain_exact(const FieldDev& f, const int* __restrict__ perm2, const float4* __restrict__ gtab,
                               const ChunkDev& ch, int x, int y, int z) {
  const int oct = min((int)f.p[5], kMaxOctaves);
  const float h0 = f.p[0], ampl = f.p[1], freq = f.p[2], lac = f.p[3], gain = f.p[4];
  const float px = ch.ox + (float)x * ch.scale, py = ch.oy + (float)y * ch.scale;
  const float pz = ch.oz + (float)z * ch.scale;
  float sum = 0.0f, amp = 1.0f, fr = freq;
  for (int o = 0; o < oct; ++o) {
    OctLine L;
    oct_line_init(L, px, py, fr, perm2);
    const float zs = pz * fr;
    const float fz = floorf(zs);
    const float zf = zs - fz;
    oct_line_cell(L, ((int)fz) & 255, gtab);
    const float l0 = __fmaf_rn(L.b0, zf, L.a0);
    const float l1 = __fmaf_rn(L.b1, zf - 1.0f, L.a1);
    sum = __fmaf_rn(amp, __fmaf_rn(fade(zf), l1 - l0, l0), sum);
    fr = fr * lac;
    amp = amp * gain;
  }
  return __fmaf_rn(-ampl, sum, py - h0);
}

__global__ void __launch_bounds__(256) k_fill_fixup(const ChunkDev* __restrict__ chunks, const uint2* __restrict__ list,
                                                    const uint32_t* __restrict__ count, int64_t cap, FieldDev field,
                                                    float* __restrict__ dens) {
  __shared__ int perm2[512];
  __shared__ float4 gtab[512];
  for (int i = threadIdx.x; i < 512; i += blockDim.x) {
    perm2[i] = field.perm[i & 255];
    gtab[i] = grad_coeffs(field.perm[i & 255]);
  }
  __syncthreads();
  const int64_t n = min((int64_t)*count, cap);
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const uint2 ent = list[e];
    const ChunkDev ch = chunks[ent.x];
    const uint32_t dim = (uint32_t)ch.dim, line = ent.y / dim;
    const int z = (int)(ent.y - line * dim), x = (int)(line / dim), y = (int)(line - (uint32_t)x * dim);
    dens[ch.dens + (int64_t)ent.y] = terrain_exact(field, perm2, gtab, ch, x, y, z);
  }
}

void launch_fill_fixup(const ChunkDev* d_chunks, const WordScratch& ws, const FieldDev& field, float* dens,
                       cudaStream_t st) {
  static std::atomic<int> grid[64] = {};
  const int g = per_device_once(grid, [](int dev) {
    int sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fill_fixup, 256, 0);
    return (sms > 0 ? sms : 1) * (per_sm > 0 ? per_sm : 1);
  });
  k_fill_fixup<<<g, 256, 0, st>>>(d_chunks, ws.fix, ws.fcount, ws.fix_cap, field, dens);
}

int fill_terrain_items(int dim) { return (dim * dim + kFillLines - 1) / kFillLines; }
int fill_terrain_lines() { return kFillLines; }
int fill_terrain_resident_ctas(int run, int octaves, bool band) {
  const size_t sm = fill_smem_bytes(min(octaves, kMaxOctaves), band);
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  fill_terrain_smem_optin();
  if (band) {
    if (run == 4)
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fill_terrain<4, true>, kFillLines, sm);
    else if (run == 16)
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fill_terrain<16, true>, kFillLines, sm);
    else
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fill_terrain<8, true>, kFillLines, sm);
  } else {
    if (run == 4)
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fill_terrain<4, false>, kFillLines, sm);
    else if (run == 16)
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fill_terrain<16, false>, kFillLines, sm);
    else
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fill_terrain<8, false>, kFillLines, sm);
  }
  return sms * (per_sm > 0 ? per_sm : 1);
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

// The 2D heightmap's (x, z) column heights of a batch, one thread per column
// over items of kColumnItem consecutive columns of one chunk ({chunk, first
// column}, column = x * dim + z), stored at chunk.words + column: every
// column is evaluated once, by a full CTA, instead of by the dim threads of
// an x-plane's CTA while the rest wait.
__global__ void __launch_bounds__(kColumnItem) k_columns2d(const ChunkDev* __restrict__ chunks,
                                                         const int2* __restrict__ items, FieldDev field,
                                                         float* __restrict__ cols) {
  __shared__ int perm2[512];
  for (int i = threadIdx.x; i < 512; i += blockDim.x) perm2[i] = field.perm[i & 255];
  __syncthreads();
  const int2 it = items[blockIdx.x];
  const ChunkDev& ch = chunks[it.x];
  const int dim = ch.dim, col = it.y + (int)threadIdx.x;
  if (col >= dim * dim) return;
  const int x = col / dim, z = col - x * dim;
  const float pxc = ch.ox + (float)x * ch.scale;
  cols[ch.words + (int64_t)col] = terrain2d_height(field, perm2, pxc, ch.oz + (float)z * ch.scale);
}

void launch_columns2d(const ChunkDev* d_chunks, const int2* d_items, int n_items, const FieldDev& field, float* cols,
                      cudaStream_t st) {
  if (n_items > 0) k_columns2d<<<n_items, kColumnItem, 0, st>>>(d_chunks, d_items, field, cols);
}
int columns2d_item() { return kColumnItem; }

// The 2D heightmap's occupancy words from its column heights, no densities
// (the column fill).  One warp per x-plane at a time (persistent; a warp's
// planes ascend, so it finds each plane's chunk by searching forward from
// the previous one, 32 candidates a step).  Per block zb a lane holds the
// height of column z = 32 zb + lane; per line y every lane evaluates its
// sample's density sign with the full fill's operations and a ballot forms
// the word, which lane y % 32 keeps, so each lane stores one word per 32 lines.
__global__ void __launch_bounds__(256) k_words2d(const ChunkDev* __restrict__ chunks, int n_chunks,
                                                 const int* __restrict__ unit_start, int n_units, FieldDev field,
                                                 const float* __restrict__ cols, uint32_t* __restrict__ words,
                                                 uint32_t* __restrict__ flags) {
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  int c = 0;
  for (int u = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; u < n_units; u += nwarps) {
    for (;;) {
      const int cand = c + 1 + lane;
      const uint32_t le = __ballot_sync(kFull, cand < n_chunks && __ldg(unit_start + cand) <= u);
      c += __popc(le);  // unit_start increases, so le is a prefix of the lanes
      if (le != kFull) break;
    }
    const ChunkDev& ch = chunks[c];
    const int x = u - __ldg(unit_start + c), dim = ch.dim, zc = ch.zc;
    const float oy = ch.oy, scale = ch.scale;
    const float* colx = cols + ch.words + (int64_t)x * dim;
    uint32_t* wx = words + ch.words + (int64_t)x * dim * zc;
    uint32_t f = 0u;
    for (int zb = 0; zb < zc; ++zb) {
      const int z = 32 * zb + lane;
      const bool zin = z < dim;
      const float n = zin ? __ldg(colx + z) : 0.0f;
      for (int yb = 0; yb < dim; yb += 32) {
        uint32_t mine = 0u;
        const int ny = min(32, dim - yb);
        for (int j = 0; j < ny; ++j) {
          const float py = oy + (float)(yb + j) * scale;
          const uint32_t w = __ballot_sync(kFull, zin && terrain2d_density(field, py, n) < 0.0f);
          if (lane == j) mine = w;
        }
        if (lane < ny) {
          wx[(int64_t)(yb + lane) * zc + zb] = mine;
          f |= (mine != 0u && mine != kFull) ? 1u : (mine == kFull ? 2u : 4u);
        }
      }
    }
    f |= __shfl_xor_sync(kFull, f, 16);
    f |= __shfl_xor_sync(kFull, f, 8);
    f |= __shfl_xor_sync(kFull, f, 4);
    f |= __shfl_xor_sync(kFull, f, 2);
    f |= __shfl_xor_sync(kFull, f, 1);
    if (lane == 0 && f) atomicOr(flags + c, f);
  }
}

void launch_words2d(const ChunkDev* d_chunks, int n_chunks, const int* d_unit_start, int n_units,
                    const FieldDev& field, const float* cols, uint32_t* words, uint32_t* flags, cudaStream_t st) {
  static std::atomic<int> grid[64] = {};
  const int g = per_device_once(grid, [](int dev) {
    int sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_words2d, 256, 0);
    return (sms > 0 ? sms : 1) * (per_sm > 0 ? per_sm : 1);
  });
  const int need = (n_units + 7) / 8;  // eight warps per CTA, one plane each at a time
  if (need > 0) k_words2d<<<min(g, need), 256, 0, st>>>(d_chunks, n_chunks, d_unit_start, n_units, field, cols, words,
                                                       flags);
}

void launch_sample_label(const ChunkDev* d_chunks, int n_chunks, const int* d_unit_start, int n_units, int max_dim,
                         const FieldDev& field, const float* dens_in, float* dens_out, uint32_t* words,
                         uint32_t* flags, cudaStream_t st, const float* cols) {
  if (field.kind == BMF_FIELD_TERRAIN_FBM && n_chunks == 1) {
    launch_fill_terrain(16, d_chunks, nullptr, fill_terrain_items(max_dim), nullptr, 0, field, dens_out, words, flags,
                        nullptr, st);
    return;
  }
  const int max_zc = (max_dim + 31) / 32;
  const size_t smem = (size_t)max_dim * max_zc * sizeof(uint32_t);
  k_sample_label<<<n_units, 256, smem, st>>>(d_chunks, n_chunks, d_unit_start, field, dens_in, dens_out, words,
                                             flags, field.kind == BMF_FIELD_TERRAIN_2D ? cols : nullptr);
}

void launch_cell_masks(int dim, const uint32_t* W, uint8_t* masks, cudaStream_t st) {
  const int zc = (dim + 31) / 32;
  const int64_t n = (int64_t)dim * dim * 32 * zc;
  const int blocks = (int)((n + 255) / 256 < 152 * 16 ? (n + 255) / 256 : 152 * 16);
  k_cell_masks<<<blocks, 256, 0, st>>>(dim, zc, W, masks);
}

}  // namespace bmf
