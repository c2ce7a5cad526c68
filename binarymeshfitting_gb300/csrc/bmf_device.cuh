// Device-side building blocks shared by the sm_103a kernels.
//
// Every translation unit is compiled with --fmad=false and IEEE division /
// square root, so each float expression below is rounded exactly as written:
// the kernels reproduce the reference's single-precision results bit for bit
// (DMCChunk.cpp:657-674 lerp, MeshProcessor.cpp:130-306 averages) and this
// project's own field definitions (bmf_fields.h).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/bmf_fields.h"
#include "bmf_case_tables.h"

namespace bmf {

constexpr unsigned kFull = 0xFFFFFFFFu;

// ---------------------------------------------------------------------------
// Case tables (generated from the reference's MCTable.h / Tables.hpp).
// ---------------------------------------------------------------------------
static __constant__ uint64_t c_tri_cases[256] = BMF_TRI_CASES_INIT;
static __constant__ uint64_t c_group_cases[256] = BMF_GROUP_CASES_INIT;
static __constant__ uint64_t c_edge_uses[256] = BMF_EDGE_USES_INIT;
// Global-memory copies for staging into shared memory with coalesced loads
// (thread-indexed constant loads would serialise).
static __device__ uint64_t g_tri_cases[256] = BMF_TRI_CASES_INIT;
static __device__ uint64_t g_group_cases[256] = BMF_GROUP_CASES_INIT;
static __device__ uint64_t g_edge_uses[256] = BMF_EDGE_USES_INIT;

__device__ __forceinline__ int tri_edge(uint64_t w, int i) { return (int)((w >> (4 * i)) & 0xF); }
__device__ __forceinline__ int group_count(int mask) { return (int)((c_group_cases[mask] >> 48) & 0xF); }
__device__ __forceinline__ int group_of(int mask, int e) { return (int)((c_group_cases[mask] >> (4 * e)) & 0xF); }
__device__ __forceinline__ int edge_uses(int mask, int e) { return (int)((c_edge_uses[mask] >> (4 * e)) & 0xF); }

// Corners of edge e (corner c = 4dx + 2dy + dz).
__device__ __forceinline__ int edge_c0(int e) {
  // x-edges 0-3: corners e, e+4; y-edges 4-7: 4dx+dz; z-edges 8-11: 4dx+2dy.
  return e < 4 ? e : (e < 8 ? (((e - 4) >> 1) << 2) | ((e - 4) & 1) : ((e - 8) << 1));
}
__device__ __forceinline__ int edge_c1(int e) { return e < 4 ? e + 4 : (e < 8 ? edge_c0(e) + 2 : edge_c0(e) + 1); }

// ---------------------------------------------------------------------------
// Chunk record used by every kernel (one per chunk in a batch).
// ---------------------------------------------------------------------------
struct ChunkDev {
  float ox, oy, oz, scale;
  int dim;        // samples per axis
  int zc;         // 32-bit occupancy words per (x, y) line = ceil(dim / 32)
  int64_t dens;   // offset of the chunk's density block (floats); -1 = not materialised
  int64_t words;  // offset of the chunk's occupancy words (u32)
  int64_t vout;   // offset of the chunk's vertices in the output arena
  int64_t iout;   // offset of the chunk's indices in the output arena
};

// Field parameters passed by value.  perm is the noise permutation.
struct FieldDev {
  int kind;
  float p[BMF_FIELD_MAX_PARAMS];
  uint8_t perm[256];
};

// ---------------------------------------------------------------------------
// Deterministic scalar math (same definitions as the CPU oracle, written for
// the device).
// ---------------------------------------------------------------------------

// sin: Cody-Waite reduction by pi/2 (two 12-bit pieces + float remainder) and
// the Taylor series of sin/cos on [-pi/4, pi/4], Horner form.
__device__ __forceinline__ float det_sin(float x) {
  const float k = rintf(x * 0x1.45f306p-1f);
  float r = x - k * 0x1.92p+0f;
  r = r - k * 0x1.fb4p-12f;
  r = r - k * 0x1.4442d2p-24f;
  const int q = ((int)k) & 3;
  const float r2 = r * r;
  float s = r2 * 2.7557319e-6f;
  s = s + -1.9841270e-4f;
  s = s * r2;
  s = s + 8.3333333e-3f;
  s = s * r2;
  s = s + -1.6666667e-1f;
  s = s * r2;
  s = s * r;
  s = s + r;
  float c = r2 * 2.4801587e-5f;
  c = c + -1.3888889e-3f;
  c = c * r2;
  c = c + 4.1666667e-2f;
  c = c * r2;
  c = c + -0.5f;
  c = c * r2;
  c = c + 1.0f;
  const float v = (q & 1) ? c : s;
  return (q & 2) ? -v : v;
}

// Noise arithmetic: fused multiply-adds (one rounding each) at fixed places --
// fade's two inner steps, every lerp a + t (b - a) = fma(t, b - a, a), a
// corner's s = fma(gy, y, gx * x), l = fma(beta, zk, alpha) and the FBM sums.
// The oracle calls fmaf at exactly these places (and rounds every other
// operation separately), so the two agree bit for bit.
__device__ __forceinline__ float fade(float t) {
  float a = __fmaf_rn(t, 6.0f, -15.0f);
  a = __fmaf_rn(t, a, 10.0f);
  float t3 = t * t;
  t3 = t3 * t;
  return t3 * a;
}
__device__ __forceinline__ float lerp_t(float t, float a, float b) { return __fmaf_rn(t, b - a, a); }

// ---------------------------------------------------------------------------
// Improved gradient noise (K. Perlin, SIGGRAPH 2002) in line-separable form.
//
// A corner gradient grad(h, x, y, z) = (+/-u) + (+/-v) with u in {x, y} and v in
// {x, y, z} (never the same axis as u) is written gx * x + gy * y + c * z with
// gx, gy, c in {0, +1, -1}: s = fma(gy, y, gx * x) is the textbook x/y part
// with one rounding.  lerp is linear, so a z-layer's x/y interpolant of the
// four corners is alpha + beta * zk exactly, with
//     alpha = lerp(v, lerp(u, s00, s10), lerp(u, s01, s11))   (beta: the c's),
// and the noise value is  l0 = alpha0 + beta0 * zf,  l1 = alpha1 + beta1 * (zf - 1),
// l0 + w (l1 - l0).  In exact arithmetic this is the textbook value; in float it
// differs from the textbook order by rounding only, and the CPU oracle evaluates
// exactly these operations, so samples agree bit for bit.  alpha and beta
// depend on x, y and the lattice cell Z, not on the sample's own z: a z-line
// sets them up once per lattice cell, and the layer-1 pair of cell Z is the
// layer-0 pair of cell Z + 1 (same hashes, same operations).
//
// Tables are 512 entries {gx, gy, c, 0}, entry i coding perm[i & 255], so hash
// chains index them without masks.
// ---------------------------------------------------------------------------
__host__ __device__ inline float4 grad_coeffs(int h) {
  h &= 15;
  const float su = (h & 1) ? -1.0f : 1.0f, sv = (h & 2) ? -1.0f : 1.0f;
  float4 t = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  if (h < 8) t.x = su; else t.y = su;
  if (h < 4) t.y = sv;
  else if (h == 12 || h == 14) t.x = sv;
  else t.z = sv;
  return t;
}

// s and c of one corner at lattice offsets (xc, yc).
__device__ __forceinline__ void seg_corner(float4 t, float xc, float yc, float& s, float& c) {
  s = __fmaf_rn(t.y, yc, t.x * xc);
  c = t.z;
}

// alpha / beta of one z-layer from the hashes of its four corners
// (h00 = AA + k, h10 = BA + k, h01 = AB + k, h11 = BB + k).
__device__ __forceinline__ void layer_coeffs(const float4* __restrict__ gtab, int h00, int h10, int h01, int h11,
                                             float xf, float yf, float x1, float y1, float u, float v, float& a,
                                             float& b) {
  float s00, c00, s10, c10, s01, c01, s11, c11;
  seg_corner(gtab[h00], xf, yf, s00, c00);
  seg_corner(gtab[h10], x1, yf, s10, c10);
  seg_corner(gtab[h01], xf, y1, s01, c01);
  seg_corner(gtab[h11], x1, y1, s11, c11);
  const float sa = lerp_t(u, s00, s10), sb = lerp_t(u, s01, s11);
  a = lerp_t(v, sa, sb);
  const float ca = lerp_t(u, c00, c10), cb = lerp_t(u, c01, c11);
  b = lerp_t(v, ca, cb);
}

// One noise value (perm2: the permutation duplicated to 512 entries).
__device__ __forceinline__ float perlin(const int* __restrict__ perm2, const float4* __restrict__ gtab, float x, float y,
                                        float z) {
  const float fx = floorf(x), fy = floorf(y), fz = floorf(z);
  const int X = ((int)fx) & 255, Y = ((int)fy) & 255, Z = ((int)fz) & 255;
  x = x - fx;
  y = y - fy;
  z = z - fz;
  const float u = fade(x), v = fade(y), w = fade(z);
  const int A = perm2[X] + Y, B = perm2[X + 1] + Y;
  const int AA = perm2[A] + Z, AB = perm2[A + 1] + Z, BA = perm2[B] + Z, BB = perm2[B + 1] + Z;
  const float x1 = x - 1.0f, y1 = y - 1.0f, z1 = z - 1.0f;
  float a0, b0, a1, b1;
  layer_coeffs(gtab, AA, BA, AB, BB, x, y, x1, y1, u, v, a0, b0);
  layer_coeffs(gtab, AA + 1, BA + 1, AB + 1, BB + 1, x, y, x1, y1, u, v, a1, b1);
  const float l0 = __fmaf_rn(b0, z, a0);
  const float l1 = __fmaf_rn(b1, z1, a1);
  return __fmaf_rn(w, l1 - l0, l0);
}

constexpr int kRun = 4;

// Terrain field (y - h) - a * FBM over a run of n <= kRun samples at
// z-coordinates pz[k]; px, py are the line's world x, y.  Every x/y-dependent
// term is computed once per octave, and alpha / beta once per lattice cell.
__device__ __forceinline__ void terrain_run(const FieldDev& f, const int* __restrict__ perm2,
                                            const float4* __restrict__ gtab, float px, float py, const float* pz,
                                            int n, float* out) {
  float sum[kRun];
#pragma unroll
  for (int k = 0; k < kRun; ++k) sum[k] = 0.0f;
  const int oct = (int)f.p[5];
  float amp = 1.0f, fr = f.p[2];
  for (int o = 0; o < oct; ++o) {
    const float xs = px * fr, ys = py * fr;
    const float fx = floorf(xs), fy = floorf(ys);
    const int X = ((int)fx) & 255, Y = ((int)fy) & 255;
    const float xf = xs - fx, yf = ys - fy;
    const float u = fade(xf), v = fade(yf);
    const float x1 = xf - 1.0f, y1 = yf - 1.0f;
    const int A = perm2[X] + Y, B = perm2[X + 1] + Y;
    const int pA = perm2[A], pA1 = perm2[A + 1], pB = perm2[B], pB1 = perm2[B + 1];
    float a0 = 0.0f, b0 = 0.0f, a1 = 0.0f, b1 = 0.0f;
    int Zp = -1;
#pragma unroll
    for (int k = 0; k < kRun; ++k) {
      if (k >= n) break;
      const float zs = pz[k] * fr;
      const float fz = floorf(zs);
      const int Z = ((int)fz) & 255;
      const float zf = zs - fz;
      const float w = fade(zf);
      const float z1 = zf - 1.0f;
      if (Z != Zp) {
        Zp = Z;
        layer_coeffs(gtab, pA + Z, pB + Z, pA1 + Z, pB1 + Z, xf, yf, x1, y1, u, v, a0, b0);
        layer_coeffs(gtab, pA + Z + 1, pB + Z + 1, pA1 + Z + 1, pB1 + Z + 1, xf, yf, x1, y1, u, v, a1, b1);
      }
      const float l0 = __fmaf_rn(b0, zf, a0);
      const float l1 = __fmaf_rn(b1, z1, a1);
      const float nv = __fmaf_rn(w, l1 - l0, l0);
      sum[k] = __fmaf_rn(amp, nv, sum[k]);
    }
    fr = fr * f.p[3];
    amp = amp * f.p[4];
  }
#pragma unroll
  for (int k = 0; k < kRun; ++k)
    if (k < n) out[k] = __fmaf_rn(-f.p[1], sum[k], py - f.p[0]);
}

__device__ __forceinline__ float len3(float x, float y, float z) {
  const float a = x * x, b = y * y, c = z * z;
  return sqrtf((a + b) + c);
}

// Evaluates a density field at world position (px, py, pz).
// ---------------------------------------------------------------------------
// BMF_FIELD_TERRAIN_2D (bmf_fields.h): 2D gradient noise (8 directions) and 2D
// value noise on the permutation, quintic fade, every lerp fma(t, b - a, a).
// ---------------------------------------------------------------------------
__device__ __forceinline__ float grad2_dot(int h, float x, float z) {
  h &= 7;
  const float gx = (h < 4) ? ((h & 1) ? -1.0f : 1.0f) : ((h & 2) ? 0.0f : ((h & 1) ? -1.0f : 1.0f));
  const float gz = (h < 4) ? ((h & 2) ? -1.0f : 1.0f) : ((h & 2) ? ((h & 1) ? -1.0f : 1.0f) : 0.0f);
  return __fmaf_rn(gz, z, gx * x);
}
// component c (0 or 1) hashes its lattice column with an offset of 73 c
__device__ __forceinline__ float noise2_grad(const int* __restrict__ perm2, int c, float x, float z) {
  const float fx = floorf(x), fz = floorf(z);
  const int X = ((int)fx) & 255, Z = ((int)fz) & 255;
  const float xf = x - fx, zf = z - fz, x1 = xf - 1.0f, z1 = zf - 1.0f;
  const float u = fade(xf), w = fade(zf);
  const int A = perm2[X + 73 * c] + Z, B = perm2[X + 1 + 73 * c] + Z;
  const float g00 = grad2_dot(perm2[A], xf, zf), g10 = grad2_dot(perm2[B], x1, zf);
  const float g01 = grad2_dot(perm2[A + 1], xf, z1), g11 = grad2_dot(perm2[B + 1], x1, z1);
  return lerp_t(w, lerp_t(u, g00, g10), lerp_t(u, g01, g11));
}
__device__ __forceinline__ float noise2_value(const int* __restrict__ perm2, float x, float z) {
  const float fx = floorf(x), fz = floorf(z);
  const int X = ((int)fx) & 255, Z = ((int)fz) & 255;
  const float xf = x - fx, zf = z - fz;
  const float u = fade(xf), w = fade(zf);
  const int A = perm2[X] + Z, B = perm2[X + 1] + Z;
  const float k = 2.0f / 255.0f;
  const float v00 = (float)perm2[A] * k - 1.0f, v10 = (float)perm2[B] * k - 1.0f;
  const float v01 = (float)perm2[A + 1] * k - 1.0f, v11 = (float)perm2[B + 1] * k - 1.0f;
  return lerp_t(w, lerp_t(u, v00, v10), lerp_t(u, v01, v11));
}
// the height noise n(x, z) in [-1, 1] of one (x, z) column
__device__ __forceinline__ float terrain2d_height(const FieldDev& f, const int* __restrict__ perm2, float px,
                                                  float pz) {
  const float g = f.p[0];
  float xn = (px * g) * 0.01f, zn = (pz * g) * 0.01f;
  const int poct = (int)f.p[2];
  float a = f.p[3], fr = f.p[4];
  for (int k = 0; k < poct; ++k) {
    const float sx = xn * fr, sz = zn * fr;
    const float dx = noise2_grad(perm2, 0, sx, sz), dz = noise2_grad(perm2, 1, sx, sz);
    xn = __fmaf_rn(a, dx, xn);
    zn = __fmaf_rn(a, dz, zn);
    fr = fr * 2.0f;
    a = a * f.p[5];
  }
  const int voct = (int)f.p[7];
  float sum = 0.0f, bound = 0.0f, amp = 1.0f, vf = 1.0f;
  for (int o = 0; o < voct; ++o) {
    sum = __fmaf_rn(amp, noise2_value(perm2, xn * vf, zn * vf), sum);
    bound = bound + amp;
    vf = vf * 2.0f;
    amp = amp * 0.5f;
  }
  return voct > 0 ? sum / bound : 0.0f;
}
// density of one sample given its column's height noise n
__device__ __forceinline__ float terrain2d_density(const FieldDev& f, float py, float n) {
  const float dy = py * f.p[0];
  return -dy - n * f.p[1];
}

__device__ __forceinline__ float eval_field(const FieldDev& f, const int* __restrict__ perm,
                                            const float4* __restrict__ gtab, float px, float py,
                                            float pz) {
  switch (f.kind) {
    case BMF_FIELD_SPHERE_WAVE: {
      const float l = len3(px - f.p[0], py - f.p[1], pz - f.p[2]);
      float s = det_sin(f.p[5] * px) * det_sin(f.p[5] * py);
      s = s * det_sin(f.p[5] * pz);
      return (l - f.p[3]) + f.p[4] * s;
    }
    case BMF_FIELD_TERRAIN_FBM: {
      const int oct = (int)f.p[5];
      float sum = 0.0f, amp = 1.0f, fr = f.p[2];
      for (int o = 0; o < oct; ++o) {
        const float n = perlin(perm, gtab, px * fr, py * fr, pz * fr);
        sum = __fmaf_rn(amp, n, sum);
        fr = fr * f.p[3];
        amp = amp * f.p[4];
      }
      return __fmaf_rn(-f.p[1], sum, py - f.p[0]);
    }
    case BMF_FIELD_TERRAIN_2D:
      return terrain2d_density(f, py, terrain2d_height(f, perm, px, pz));
    case BMF_FIELD_TORUS_Z: {  // ImplicitSampler.cpp:27-34
      const float r1 = f.p[0] / 4.0f, r2 = f.p[0] / 10.0f;
      const float q_x = fabsf(sqrtf(px * px + py * py)) - r1;
      const float len = sqrtf(q_x * q_x + pz * pz);
      return -(len - r2);
    }
    case BMF_FIELD_SPHERE: {  // ImplicitSampler.cpp:46-50
      const float r = f.p[0] * 0.25f;
      return -(len3(px, py, pz) - r);
    }
    case BMF_FIELD_CUBOID: {  // ImplicitSampler.cpp:52-60
      const float r = f.p[0] / 8.0f;
      const float dx = fabsf(px) - r, dy = fabsf(py) - r, dz = fabsf(pz) - r;
      const float m = fmaxf(dx, fmaxf(dy, dz));
      return -fminf(m, len3(dx, dy, dz));
    }
    default:  // BMF_FIELD_PLANE_Y, ImplicitSampler.cpp:62-65
      return -py;
  }
}

// ---------------------------------------------------------------------------
// Occupancy-word helpers.  W points at a chunk's words, [x][y][zb] row-major.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t word_at(const uint32_t* __restrict__ W, int dim, int zc, int x, int y, int zb) {
  if (x < 0 || y < 0 || x >= dim || y >= dim || zb < 0 || zb >= zc) return 0u;
  return __ldg(W + ((int64_t)x * dim + y) * zc + zb);
}
// Inside bits of samples z and z + 1 of one line L (bit 0: z); 0 for samples
// outside [0, dim).
__device__ __forceinline__ uint32_t line_bits2(const uint32_t* __restrict__ L, int dim, int z) {
  if (z >= dim) return 0u;
  uint32_t r;
  if (z >= 0 && (z & 31) != 31) {
    r = (__ldg(L + (z >> 5)) >> (z & 31)) & 3u;
  } else {  // z and z + 1 straddle two words (or z == -1)
    r = 0u;
    if (z >= 0 && z < dim) r = (__ldg(L + (z >> 5)) >> 31) & 1u;
    if (z + 1 >= 0 && z + 1 < dim) r |= (__ldg(L + ((z + 1) >> 5)) & 1u) << 1;
  }
  if (z + 1 >= dim) r &= 1u;
  return r;
}

// Reference cell mask (DMCChunk.cpp:202-438): bit 4dx + 2dy + dz is corner
// (x+dx, y+dy, z+dz); corners outside the chunk are 0.  Two bits per line.
__device__ __forceinline__ int cell_mask_at(const uint32_t* __restrict__ W, int dim, int zc, int x, int y, int z) {
  int m = 0;
#pragma unroll
  for (int i = 0; i < 2; ++i) {
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const int xx = x + i, yy = y + j;
      if (xx < 0 || yy < 0 || xx >= dim || yy >= dim) continue;
      m |= (int)line_bits2(W + (xx * dim + yy) * zc, dim, z) << (4 * i + 2 * j);
    }
  }
  return m;
}

// Bits of a z-line (x, y) block zb that have a crossing towards +z.
__device__ __forceinline__ uint32_t zcross_word(const uint32_t* __restrict__ W, int dim, int zc, int x, int y, int zb) {
  const uint32_t w = word_at(W, dim, zc, x, y, zb);
  const uint32_t wn = word_at(W, dim, zc, x, y, zb + 1);
  uint32_t Z = w ^ ((w >> 1) | (wn << 31));
  const int valid = dim - 1 - 32 * zb;  // cells z with z + 1 < dim
  if (valid < 32) Z &= valid <= 0 ? 0u : ((1u << valid) - 1u);
  return Z;
}
// Bits of line (x, y) block zb that have a crossing towards +x (0 on the far x face).
__device__ __forceinline__ uint32_t xcross_word(const uint32_t* __restrict__ W, int dim, int zc, int x, int y, int zb) {
  if (x + 1 >= dim) return 0u;
  return word_at(W, dim, zc, x, y, zb) ^ word_at(W, dim, zc, x + 1, y, zb);
}
__device__ __forceinline__ uint32_t ycross_word(const uint32_t* __restrict__ W, int dim, int zc, int x, int y, int zb) {
  if (y + 1 >= dim) return 0u;
  return word_at(W, dim, zc, x, y, zb) ^ word_at(W, dim, zc, x, y + 1, zb);
}

__device__ __forceinline__ uint32_t lane_lt(int lane) { return (1u << lane) - 1u; }

// Vertex key: where a vertex came from, as the sample (x, y, z) that owns it
// (9 bits each: chunks have at most 512 samples per axis) and k, the crossing
// axis (Mode R) or vertex group (Mode Q).
__device__ __forceinline__ uint32_t vertex_key(int x, int y, int z, int k) {
  return ((uint32_t)x << 20) | ((uint32_t)y << 11) | ((uint32_t)z << 2) | (uint32_t)k;
}
__device__ __forceinline__ void vertex_key_decode(uint32_t key, int& x, int& y, int& z, int& k) {
  x = (int)(key >> 20);
  y = (int)((key >> 11) & 511u);
  z = (int)((key >> 2) & 511u);
  k = (int)(key & 3u);
}

// Warp-inclusive scan of an int.
__device__ __forceinline__ int warp_incl_scan(int v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int n = __shfl_up_sync(kFull, v, o);
    if (lane >= o) v += n;
  }
  return v;
}

}  // namespace bmf
