/* CPU oracle for the chunk-extraction hot path (TEST INFRASTRUCTURE ONLY).
 * See bmf_oracle.h for what this file is and how it is pinned.  Every float
 * expression below is written in the exact evaluation order the reference
 * uses (or, for the parts the reference does not have, the order this project
 * specifies); the Makefile compiles it with -ffp-contract=off. */
#include "bmf_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/bmf_fields.h"
#include "../binarymeshfitting_gb300/csrc/bmf_case_tables.h"

/* ======================================================================== */
/* deterministic scalar math                                                 */
/* ======================================================================== */

/* sin(x): Cody-Waite reduction by pi/2 split into two 12-bit pieces and a
 * float remainder, then the Taylor series of sin / cos on [-pi/4, pi/4]
 * (degree 9 / 8) in Horner form. */
float bmfo_sin(float x) {
  const float two_over_pi = 0x1.45f306p-1f;
  const float p1 = 0x1.92p+0f, p2 = 0x1.fb4p-12f, p3 = 0x1.4442d2p-24f;
  float k = rintf(x * two_over_pi);
  float r = x - k * p1;
  r = r - k * p2;
  r = r - k * p3;
  int q = ((int)k) & 3;
  float r2 = r * r;
  float s = r2 * 2.7557319e-6f;       /* 1/9! */
  s = s + -1.9841270e-4f;             /* -1/7! */
  s = s * r2;
  s = s + 8.3333333e-3f;              /* 1/5! */
  s = s * r2;
  s = s + -1.6666667e-1f;             /* -1/3! */
  s = s * r2;
  s = s * r;
  s = s + r;
  float c = r2 * 2.4801587e-5f;       /* 1/8! */
  c = c + -1.3888889e-3f;             /* -1/6! */
  c = c * r2;
  c = c + 4.1666667e-2f;              /* 1/4! */
  c = c * r2;
  c = c + -0.5f;
  c = c * r2;
  c = c + 1.0f;
  switch (q) {
    case 0: return s;
    case 1: return c;
    case 2: return -s;
    default: return -c;
  }
}

static uint64_t splitmix64(uint64_t* state) {
  uint64_t z = (*state += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

/* Fisher-Yates shuffle of 0..255, index j = splitmix64 % (i + 1). */
void bmfo_perm_init(uint64_t seed, uint8_t perm[256]) {
  uint64_t st = seed;
  for (int i = 0; i < 256; ++i) perm[i] = (uint8_t)i;
  for (int i = 255; i > 0; --i) {
    int j = (int)(splitmix64(&st) % (uint64_t)(i + 1));
    uint8_t t = perm[i];
    perm[i] = perm[j];
    perm[j] = t;
  }
}

static float fade(float t) {
  float a = t * 6.0f;
  a = a - 15.0f;
  a = t * a;
  a = a + 10.0f;
  float t3 = t * t;
  t3 = t3 * t;
  return t3 * a;
}
static float lerpf(float t, float a, float b) { return a + t * (b - a); }
static float grad(int h, float x, float y, float z) {
  h &= 15;
  float u = h < 8 ? x : y;
  float v = h < 4 ? y : ((h == 12 || h == 14) ? x : z);
  return ((h & 1) ? -u : u) + ((h & 2) ? -v : v);
}

/* Improved gradient noise (K. Perlin, "Improving Noise", SIGGRAPH 2002),
 * textbook evaluation order: the eight corner gradients, then lerps along x,
 * y and z.  Kept as the precision yardstick of bmfo_perlin (tests). */
float bmfo_perlin_textbook(const uint8_t perm[256], float x, float y, float z) {
  float fx = floorf(x), fy = floorf(y), fz = floorf(z);
  int X = ((int)fx) & 255, Y = ((int)fy) & 255, Z = ((int)fz) & 255;
  x = x - fx;
  y = y - fy;
  z = z - fz;
  float u = fade(x), v = fade(y), w = fade(z);
#define P(i) ((int)perm[(i) & 255])
  int A = P(X) + Y, AA = P(A) + Z, AB = P(A + 1) + Z;
  int B = P(X + 1) + Y, BA = P(B) + Z, BB = P(B + 1) + Z;
  float x1 = x - 1.0f, y1 = y - 1.0f, z1 = z - 1.0f;
  float g000 = grad(P(AA), x, y, z), g100 = grad(P(BA), x1, y, z);
  float g010 = grad(P(AB), x, y1, z), g110 = grad(P(BB), x1, y1, z);
  float g001 = grad(P(AA + 1), x, y, z1), g101 = grad(P(BA + 1), x1, y, z1);
  float g011 = grad(P(AB + 1), x, y1, z1), g111 = grad(P(BB + 1), x1, y1, z1);
#undef P
  float l00 = lerpf(u, g000, g100), l10 = lerpf(u, g010, g110);
  float l01 = lerpf(u, g001, g101), l11 = lerpf(u, g011, g111);
  float l0 = lerpf(v, l00, l10), l1 = lerpf(v, l01, l11);
  return lerpf(w, l0, l1);
}

/* The line-separable noise evaluates with fused multiply-adds (fmaf, one
 * rounding each) at fixed places: fade's two inner steps, every lerp
 * a + t (b - a) = fmaf(t, b - a, a), a corner's s = fmaf(gy, y, gx * x), and
 * l = fmaf(beta, zk, alpha).  The GPU kernels use __fmaf_rn at exactly these
 * places, so the two agree bit for bit. */
static float fade_fma(float t) {
  float a = fmaf(t, 6.0f, -15.0f);
  a = fmaf(t, a, 10.0f);
  float t3 = t * t;
  t3 = t3 * t;
  return t3 * a;
}
static float lerp_fma(float t, float a, float b) { return fmaf(t, b - a, a); }

/* Gradient of hash h split into an x/y part and a z coefficient:
 * grad(h, x, y, z) = gx * x + gy * y + c * z with gx, gy, c in {0, +1, -1};
 * u (x for h < 8, else y) and v (y for h < 4, x for h = 12 or 14, else z) are
 * never the same axis, so s = gx * x + gy * y is the textbook (+/-u) + (+/-v)
 * (or +/-u when v is z) with one rounding, up to the sign of an exact zero. */
static void grad_split(int h, float* gx, float* gy, float* c) {
  h &= 15;
  const float su = (h & 1) ? -1.0f : 1.0f, sv = (h & 2) ? -1.0f : 1.0f;
  *gx = 0.0f;
  *gy = 0.0f;
  *c = 0.0f;
  if (h < 8) *gx = su; else *gy = su;
  if (h < 4) *gy = sv;
  else if (h == 12 || h == 14) *gx = sv;
  else *c = sv;
}

static void corner_sc(int h, float x, float y, float* s, float* c) {
  float gx, gy;
  grad_split(h, &gx, &gy, c);
  *s = fmaf(gy, y, gx * x);
}

/* One z-layer of the cell: the x/y lerps of the four corners' s and c parts.
 * The layer's interpolated value at depth zk is alpha + beta * zk. */
static void layer_coeffs(const uint8_t perm[256], int AAk, int ABk, int BAk, int BBk, float x, float y, float x1,
                         float y1, float u, float v, float* alpha, float* beta) {
#define P(i) ((int)perm[(i) & 255])
  float s00, c00, s10, c10, s01, c01, s11, c11;
  corner_sc(P(AAk), x, y, &s00, &c00);
  corner_sc(P(BAk), x1, y, &s10, &c10);
  corner_sc(P(ABk), x, y1, &s01, &c01);
  corner_sc(P(BBk), x1, y1, &s11, &c11);
#undef P
  *alpha = lerp_fma(v, lerp_fma(u, s00, s10), lerp_fma(u, s01, s11));
  *beta = lerp_fma(v, lerp_fma(u, c00, c10), lerp_fma(u, c01, c11));
}

/* Improved gradient noise in line-separable form.  Each corner gradient is
 * s + c * z (grad_split), and lerp is linear, so a z-layer's x/y interpolant is
 * alpha + beta * zk exactly; the noise is then
 *     l0 = alpha0 + beta0 * zf,  l1 = alpha1 + beta1 * (zf - 1),  l0 + w (l1 - l0).
 * In exact arithmetic this is the textbook value; in float it differs from it
 * by rounding only.  alpha and beta depend on x, y and the lattice cell Z, not
 * on the sample's own z, so a kernel walking a z-line sets them up once per
 * lattice cell and spends five operations per sample and octave (four fused).
 * The layer-1 coefficients of cell Z are the layer-0 coefficients of cell
 * Z + 1 (same hashes, same operations). */
float bmfo_perlin(const uint8_t perm[256], float x, float y, float z) {
  float fx = floorf(x), fy = floorf(y), fz = floorf(z);
  int X = ((int)fx) & 255, Y = ((int)fy) & 255, Z = ((int)fz) & 255;
  x = x - fx;
  y = y - fy;
  z = z - fz;
  float u = fade_fma(x), v = fade_fma(y), w = fade_fma(z);
#define P(i) ((int)perm[(i) & 255])
  int A = P(X) + Y, AA = P(A) + Z, AB = P(A + 1) + Z;
  int B = P(X + 1) + Y, BA = P(B) + Z, BB = P(B + 1) + Z;
#undef P
  float x1 = x - 1.0f, y1 = y - 1.0f, z1 = z - 1.0f;
  float a0, b0, a1, b1;
  layer_coeffs(perm, AA, AB, BA, BB, x, y, x1, y1, u, v, &a0, &b0);
  layer_coeffs(perm, AA + 1, AB + 1, BA + 1, BB + 1, x, y, x1, y1, u, v, &a1, &b1);
  float l0 = fmaf(b0, z, a0);
  float l1 = fmaf(b1, z1, a1);
  return fmaf(w, l1 - l0, l0);
}

float bmfo_fbm(const uint8_t perm[256], float x, float y, float z, int octaves, float freq, float lacunarity,
               float gain) {
  float sum = 0.0f, amp = 1.0f, f = freq;
  for (int o = 0; o < octaves; ++o) {
    float n = bmfo_perlin(perm, x * f, y * f, z * f);
    sum = fmaf(amp, n, sum);
    f = f * lacunarity;
    amp = amp * gain;
  }
  return sum;
}

/* ======================================================================== */
/* density fields                                                            */
/* ======================================================================== */

/* BMF_FIELD_TERRAIN_2D (include/bmf_fields.h): the project's restatement of
 * the reference's 2D perturbed heightmap sampler (NoiseSampler.cpp:148-194).
 * 2D gradient noise with 8 directions (component c hashes its lattice column
 * with an offset of 73 c) and 2D value noise, quintic fade, fmaf at the same
 * places as the kernels (grad2_dot, every lerp, the perturbation and the FBM
 * sum). */
static float grad2_dot(int h, float x, float z) {
  h &= 7;
  const float gx = (h < 4) ? ((h & 1) ? -1.0f : 1.0f) : ((h & 2) ? 0.0f : ((h & 1) ? -1.0f : 1.0f));
  const float gz = (h < 4) ? ((h & 2) ? -1.0f : 1.0f) : ((h & 2) ? ((h & 1) ? -1.0f : 1.0f) : 0.0f);
  return fmaf(gz, z, gx * x);
}
static int perm2_at(const uint8_t perm[256], int i) { return perm[i & 255]; }
static float noise2_grad(const uint8_t perm[256], int c, float x, float z) {
  const float fx = floorf(x), fz = floorf(z);
  const int X = ((int)fx) & 255, Z = ((int)fz) & 255;
  const float xf = x - fx, zf = z - fz, x1 = xf - 1.0f, z1 = zf - 1.0f;
  const float u = fade_fma(xf), w = fade_fma(zf);
  const int A = perm2_at(perm, X + 73 * c) + Z, B = perm2_at(perm, X + 1 + 73 * c) + Z;
  const float g00 = grad2_dot(perm2_at(perm, A), xf, zf), g10 = grad2_dot(perm2_at(perm, B), x1, zf);
  const float g01 = grad2_dot(perm2_at(perm, A + 1), xf, z1), g11 = grad2_dot(perm2_at(perm, B + 1), x1, z1);
  return lerp_fma(w, lerp_fma(u, g00, g10), lerp_fma(u, g01, g11));
}
static float noise2_value(const uint8_t perm[256], float x, float z) {
  const float fx = floorf(x), fz = floorf(z);
  const int X = ((int)fx) & 255, Z = ((int)fz) & 255;
  const float xf = x - fx, zf = z - fz;
  const float u = fade_fma(xf), w = fade_fma(zf);
  const int A = perm2_at(perm, X) + Z, B = perm2_at(perm, X + 1) + Z;
  const float k = 2.0f / 255.0f;
  const float v00 = (float)perm2_at(perm, A) * k - 1.0f, v10 = (float)perm2_at(perm, B) * k - 1.0f;
  const float v01 = (float)perm2_at(perm, A + 1) * k - 1.0f, v11 = (float)perm2_at(perm, B + 1) * k - 1.0f;
  return lerp_fma(w, lerp_fma(u, v00, v10), lerp_fma(u, v01, v11));
}
float bmfo_terrain2d_height(const uint8_t perm[256], const float* p, float px, float pz) {
  const float g = p[0];
  float xn = (px * g) * 0.01f, zn = (pz * g) * 0.01f;
  const int poct = (int)p[2];
  float a = p[3], fr = p[4];
  for (int k = 0; k < poct; ++k) {
    const float sx = xn * fr, sz = zn * fr;
    const float dx = noise2_grad(perm, 0, sx, sz), dz = noise2_grad(perm, 1, sx, sz);
    xn = fmaf(a, dx, xn);
    zn = fmaf(a, dz, zn);
    fr = fr * 2.0f;
    a = a * p[5];
  }
  const int voct = (int)p[7];
  float sum = 0.0f, bound = 0.0f, amp = 1.0f, vf = 1.0f;
  for (int o = 0; o < voct; ++o) {
    sum = fmaf(amp, noise2_value(perm, xn * vf, zn * vf), sum);
    bound = bound + amp;
    vf = vf * 2.0f;
    amp = amp * 0.5f;
  }
  return voct > 0 ? sum / bound : 0.0f;
}
float bmfo_noise2_grad(const uint8_t perm[256], int c, float x, float z) { return noise2_grad(perm, c, x, z); }
float bmfo_noise2_value(const uint8_t perm[256], float x, float z) { return noise2_value(perm, x, z); }

static float len3(float x, float y, float z) {
  float a = x * x, b = y * y, c = z * z;
  return sqrtf((a + b) + c);
}

/* The reference's own analytic fields, ImplicitSampler.cpp:27-65
 * (glm::length = sqrt of the component products summed left to right). */
static float ref_field(int kind, float res, float px, float py, float pz) {
  switch (kind) {
    case BMF_FIELD_TORUS_Z: {
      const float r1 = res / 4.0f, r2 = res / 10.0f;
      float q_x = fabsf(sqrtf(px * px + py * py)) - r1;
      float len = sqrtf(q_x * q_x + pz * pz);
      return -(len - r2);
    }
    case BMF_FIELD_SPHERE: {
      const float r = res * 0.25f;
      return -(len3(px, py, pz) - r);
    }
    case BMF_FIELD_CUBOID: {
      float r = res / 8.0f;
      float dx = fabsf(px) - r, dy = fabsf(py) - r, dz = fabsf(pz) - r;
      float m = fmaxf(dx, fmaxf(dy, dz));
      return -fminf(m, len3(dx, dy, dz));
    }
    default:
      return -py;
  }
}

void bmfo_fill_field(int kind, const float* params, int dim, const float origin[3], float scale, float* out) {
  uint8_t perm[256];
  if (kind == BMF_FIELD_TERRAIN_FBM || kind == BMF_FIELD_TERRAIN_2D) bmfo_perm_init((uint64_t)(int64_t)params[6], perm);
  for (int x = 0; x < dim; ++x) {
    float px = origin[0] + (float)x * scale;
    for (int y = 0; y < dim; ++y) {
      float py = origin[1] + (float)y * scale;
      for (int z = 0; z < dim; ++z) {
        float pz = origin[2] + (float)z * scale;
        float v;
        if (kind == BMF_FIELD_SPHERE_WAVE) {
          float l = len3(px - params[0], py - params[1], pz - params[2]);
          float s = bmfo_sin(params[5] * px) * bmfo_sin(params[5] * py);
          s = s * bmfo_sin(params[5] * pz);
          v = (l - params[3]) + params[4] * s;
        } else if (kind == BMF_FIELD_TERRAIN_FBM) {
          float n = bmfo_fbm(perm, px, py, pz, (int)params[5], params[2], params[3], params[4]);
          v = fmaf(-params[1], n, py - params[0]);
        } else if (kind == BMF_FIELD_TERRAIN_2D) {
          const float n = bmfo_terrain2d_height(perm, params, px, pz);
          const float dy = py * params[0];
          v = -dy - n * params[1];
        } else {
          v = ref_field(kind, params[0], px, py, pz);
        }
        out[((size_t)x * dim + y) * dim + z] = v;
      }
    }
  }
}

/* ======================================================================== */
/* DMCChunk::label_grid (DMCChunk.cpp:79-166)                                */
/* ======================================================================== */

int bmfo_label_grid(int dim, const float* density, uint32_t* words) {
  const int zc = (dim + 31) / 32;
  int mesh = 0, positive = 0, negative = 0;
  for (int x = 0; x < dim; ++x)
    for (int y = 0; y < dim; ++y)
      for (int zb = 0; zb < zc; ++zb) {
        const float* s = density + ((size_t)x * dim + y) * dim + zb * 32;
        int z_max = dim - zb * 32;
        if (z_max > 32) z_max = 32;
        uint32_t m = 0;
        for (int z = 0; z < z_max; ++z)
          if (s[z] < 0.0f) m |= 1u << z;
        words[((size_t)x * dim + y) * zc + zb] = m;
        if (m != 0) {
          if (m != 0xFFFFFFFFu) mesh = 1;
          else if (!mesh) negative = 1;
        } else if (!mesh) {
          positive = 1;
        }
      }
  return mesh ? 1 : (negative && positive);
}

/* ======================================================================== */
/* DMCChunk::label_edges mask passes (DMCChunk.cpp:168-438, EDGE_LINE :20-30) */
/* ======================================================================== */

/* One z-block of one pass: sample bit b (z = 8*l + j) sets corner bit m of
 * cell z and corner bit m+1 of cell z-1 (which may sit in the previous word,
 * or in the previous z-block's last word). */
static void edge_line(uint32_t line, int m, int zb, uint64_t* lm, uint64_t local[4]) {
  local[0] = local[1] = local[2] = local[3] = 0;
  for (int l = 0; l < 4; ++l)
    for (int j = 0; j < 8; ++j) {
      if (!((line >> (l * 8 + j)) & 1u)) continue;
      local[l] |= 1ull << (j * 8 + m);
      if (j > 0) local[l] |= 1ull << ((j - 1) * 8 + m + 1);
      else if (l > 0) local[l - 1] |= 1ull << (7 * 8 + m + 1);
      else if (zb > 0) lm[-1] |= 1ull << (7 * 8 + m + 1);
    }
}

void bmfo_cell_masks(int dim, const uint32_t* words, uint64_t* masks) {
  const int zc = (dim + 31) / 32;
  const int w8 = 4 * zc;
  uint64_t local[4];
  /* pass m = 0: corner (x, y) */
  for (int x = 0; x < dim; ++x)
    for (int y = 0; y < dim; ++y)
      for (int zb = 0; zb < zc; ++zb) {
        uint32_t line = words[((size_t)x * dim + y) * zc + zb];
        uint64_t* lm = masks + ((size_t)x * dim + y) * w8 + zb * 4;
        if (line == 0) {
          lm[0] = lm[1] = lm[2] = lm[3] = 0;
          continue;
        }
        edge_line(line, 0, zb, lm, local);
        lm[0] = local[0]; lm[1] = local[1]; lm[2] = local[2]; lm[3] = local[3];
      }
  /* passes m = 2 (x, y+1), 4 (x+1, y), 6 (x+1, y+1) */
  for (int pass = 1; pass < 4; ++pass) {
    const int m = 2 * pass, dx = pass >> 1, dy = pass & 1;
    for (int x = 0; x < dim - dx; ++x)
      for (int y = 0; y < dim - dy; ++y)
        for (int zb = 0; zb < zc; ++zb) {
          uint32_t line = words[((size_t)(x + dx) * dim + (y + dy)) * zc + zb];
          if (line == 0) continue;
          uint64_t* lm = masks + ((size_t)x * dim + y) * w8 + zb * 4;
          edge_line(line, m, zb, lm, local);
          for (int k = 0; k < 4; ++k)
            if (local[k]) lm[k] |= local[k];
        }
  }
}

/* ======================================================================== */
/* Mode R: enumeration + calculate_cell + polygonize                         */
/* ======================================================================== */

typedef struct {
  uint32_t lin;       /* edges[0].grid_v0 */
  uint8_t mask;
  uint32_t v[3];      /* iso-vertex index per own edge x/y/z, or UINT32_MAX */
} ocell;

/* _get_intersection + calculate_isovertex (DMCChunk.cpp:657-674). */
static void isovertex(const float* d, int dim, int x0, int y0, int z0, int x1, int y1, int z1, float* p) {
  float s0 = d[((size_t)x0 * dim + y0) * dim + z0];
  float s1 = d[((size_t)x1 * dim + y1) * dim + z1];
  float mu = (0.0f - s0) / (s1 - s0);
  float q0[3] = {(float)x0, (float)y0, (float)z0};
  float q1[3] = {(float)x1, (float)y1, (float)z1};
  for (int k = 0; k < 3; ++k) {
    float dv = (q1[k] - q0[k]) * mu;
    p[k] = dv + q0[k];
  }
}

int bmfo_extract_r(int dim, const float* density, const uint64_t* masks, int64_t vcap, int64_t icap, int64_t ccap,
                   float* vpos, uint8_t* vboundary, uint8_t* vvalence, uint32_t* idx, uint32_t* cell_lin,
                   uint16_t* cell_mask, bmfo_counts* counts) {
  const int zc = (dim + 31) / 32;
  const int w8 = 4 * zc;
  const size_t n = (size_t)dim * dim * dim;
  uint32_t* inds = (uint32_t*)malloc(n * sizeof(uint32_t));
  size_t cells_cap = 1024, ncells = 0;
  ocell* cells = (ocell*)malloc(cells_cap * sizeof(ocell));
  int64_t nv = 0, ni = 0;
  int overflow = 0;
  /* enumeration, DMCChunk.cpp:449-498 */
  for (int x = 0; x < dim; ++x)
    for (int y = 0; y < dim; ++y)
      for (int z = 0; z < dim; z += 8) {
        uint64_t mask = masks[((size_t)x * dim + y) * w8 + z / 8];
        size_t base = ((size_t)x * dim + y) * dim;
        if (mask != 0 && mask != ~0ull) {
          for (int sz = 0; sz < 8 && z + sz < dim; ++sz, mask >>= 8) {
            uint8_t sub = (uint8_t)(mask & 0xFF);
            int cz = z + sz;
            if (sub == 0 || sub == 255) {
              inds[base + cz] = 0xFFFFFFFFu;
              continue;
            }
            /* calculate_cell, DMCChunk.cpp:593-655 */
            ocell c;
            c.lin = (uint32_t)(base + cz);
            c.mask = sub;
            const int cross[3] = {((sub & 1) != ((sub >> 4) & 1)) && x + 1 < dim,
                                  ((sub & 1) != ((sub >> 2) & 1)) && y + 1 < dim,
                                  ((sub & 1) != ((sub >> 1) & 1)) && cz + 1 < dim};
            for (int a = 0; a < 3; ++a) {
              c.v[a] = 0xFFFFFFFFu;
              if (!cross[a]) continue;
              int x1 = x + (a == 0), y1 = y + (a == 1), z1 = cz + (a == 2);
              c.v[a] = (uint32_t)nv;
              if (nv < vcap) {
                if (vpos) isovertex(density, dim, x, y, cz, x1, y1, z1, vpos + 3 * nv);
                if (vboundary)
                  vboundary[nv] = (x == 0 || y == 0 || cz == 0 || x == dim - 1 || y == dim - 1 || cz == dim - 1 ||
                                   x1 == dim - 1 || y1 == dim - 1 || z1 == dim - 1);
                if (vvalence) vvalence[nv] = 0;
              } else {
                overflow = 1;
              }
              ++nv;
            }
            inds[base + cz] = (uint32_t)ncells;
            if (ncells == cells_cap) {
              cells_cap *= 2;
              cells = (ocell*)realloc(cells, cells_cap * sizeof(ocell));
            }
            cells[ncells++] = c;
          }
        } else {
          for (int sz = 0; sz < 8 && z + sz < dim; ++sz) inds[base + z + sz] = 0xFFFFFFFFu;
        }
      }
  /* polygonize + polygonize_cell, DMCChunk.cpp:514-576; neighbour edges via
   * EDGE_V (:32): edge e of the 12 lives in cell (x,y,z)+offset on axis a. */
  static const int eoff[12][4] = {{0, 0, 0, 0}, {0, 0, 1, 0}, {0, 1, 0, 0}, {0, 1, 1, 0},
                                  {0, 0, 0, 1}, {0, 0, 1, 1}, {1, 0, 0, 1}, {1, 0, 1, 1},
                                  {0, 0, 0, 2}, {0, 1, 0, 2}, {1, 0, 0, 2}, {1, 1, 0, 2}};
  for (size_t i = 0; i < ncells; ++i) {
    const ocell* c = &cells[i];
    int x = (int)(c->lin / (uint32_t)dim / (uint32_t)dim), y = (int)(c->lin / (uint32_t)dim % (uint32_t)dim),
        z = (int)(c->lin % (uint32_t)dim);
    if (x >= dim - 1 || y >= dim - 1 || z >= dim - 1) continue;
    uint64_t tri = kBmfTriCases[c->mask];
    int nt = (int)(tri >> 60);
    for (int k = 0; k < 3 * nt; ++k) {
      int e = (int)((tri >> (4 * k)) & 0xF);
      uint32_t vid;
      if (e == 0 || e == 4 || e == 8) {
        vid = c->v[e / 4];
      } else {
        size_t nlin = ((size_t)(x + eoff[e][0]) * dim + (y + eoff[e][1])) * dim + (z + eoff[e][2]);
        vid = cells[inds[nlin]].v[eoff[e][3]];
      }
      if (ni < icap) {
        if (idx) idx[ni] = vid;
      } else {
        overflow = 1;
      }
      if (vvalence && (int64_t)vid < vcap) vvalence[vid]++;
      ++ni;
    }
  }
  if (cell_lin || cell_mask) {
    for (size_t i = 0; i < ncells && (int64_t)i < ccap; ++i) {
      if (cell_lin) cell_lin[i] = cells[i].lin;
      if (cell_mask) cell_mask[i] = cells[i].mask;
    }
    if ((int64_t)ncells > ccap) overflow = 1;
  }
  if (counts) {
    counts->n_cells = (int64_t)ncells;
    counts->n_verts = nv;
    counts->n_idx = ni;
  }
  free(inds);
  free(cells);
  return overflow ? -1 : 0;
}

/* ======================================================================== */
/* QEF: restatement of qef_simd.h:150-579                                    */
/* ======================================================================== */
/* FP32, with the same lane arithmetic and evaluation order as the SSE code;
 * the one approximate step (_mm_rsqrt_ps, qef_simd.h:196) is the exact
 * 1/sqrt here. */

typedef float m4[4][4];

static float dot4f(const float a[4], const float b[4]) {
  float m0 = a[0] * b[0], m1 = a[1] * b[1], m2 = a[2] * b[2], m3 = a[3] * b[3];
  return (m0 + m1) + (m3 + m2);
}
static void vec_mul_m4f(const float a[4], m4 B, float out[4]) {
  for (int k = 0; k < 4; ++k) {
    float r = a[0] * B[0][k];
    r = r + a[1] * B[1][k];
    r = r + a[2] * B[2][k];
    r = r + a[3] * B[3][k];
    out[k] = r;
  }
}
static void givens_f(m4 vtav, int a, int b, float* c_out, float* s_out) {
  float pp = vtav[a][a], pq = vtav[a][b], qq = vtav[b][b];
  float pq2 = pq * 2.0f;
  float qq_sub_pp = qq - pp;
  float tau = qq_sub_pp / pq2;
  float tau_sq_1 = tau * tau + 1.0f;
  float stt = sqrtf(tau_sq_1);
  float tan_inv = (tau >= 0.0f) ? (tau + stt) : (tau - stt);
  float tn = 1.0f / tan_inv;
  float tan_sq_1 = 1.0f + tn * tn;
  float c = 1.0f / sqrtf(tan_sq_1);
  float s = tn * c;
  if (pq == 0.0f) {
    c = 1.0f;
    s = 0.0f;
  }
  *c_out = c;
  *s_out = s;
}
static void rotateq_f(m4 vtav, float c, float s, int a, int b) {
  float u = vtav[a][a], v = vtav[b][b], A = vtav[a][b];
  float cc = c * c, ss = s * s;
  float c2 = 2.0f * c;
  float c2s = c2 * s;
  float mx = c2s * A;
  float x = (cc * u - mx) + ss * v;
  float y = (ss * u + mx) + cc * v;
  vtav[a][a] = x;
  vtav[b][b] = y;
}
static void rotate_f(m4 vtav, m4 v, float c, float s, int a, int b) {
  float u[4] = {v[0][a], v[1][a], v[2][a], vtav[0][3 - b]};
  float w[4] = {v[0][b], v[1][b], v[2][b], vtav[1 - a][2]};
  float x[4], y[4];
  for (int k = 0; k < 4; ++k) {
    x[k] = c * u[k] - s * w[k];
    y[k] = s * u[k] + c * w[k];
  }
  v[0][a] = x[0]; v[1][a] = x[1]; v[2][a] = x[2]; vtav[0][3 - b] = x[3];
  v[0][b] = y[0]; v[1][b] = y[1]; v[2][b] = y[2]; vtav[1 - a][2] = y[3];
  vtav[a][b] = 0.0f;
}

float bmfo_qef_f32(const float* pos, const float* nrm, int count, float* out) {
  if (count < 2 || count > 12) {
    out[0] = out[1] = out[2] = 0.0f;
    return 0.0f;
  }
  m4 ata;
  memset(ata, 0, sizeof(ata));
  float atb[4] = {0, 0, 0, 0}, acc[4] = {0, 0, 0, 0};
  for (int i = 0; i < count; ++i) { /* qef_simd_add, qef_simd.h:411-430 */
    float p[4] = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], 1.0f};
    float n[4] = {nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2], 0.0f};
    for (int r = 0; r < 3; ++r)
      for (int k = 0; k < 4; ++k) ata[r][k] = ata[r][k] + n[r] * n[k];
    float d = dot4f(p, n);
    float dd[4] = {d, d, d, 0.0f};
    for (int k = 0; k < 4; ++k) atb[k] = atb[k] + dd[k] * n[k];
    for (int k = 0; k < 4; ++k) acc[k] = acc[k] + p[k];
  }
  /* qef_simd_solve, qef_simd.h:444-461 */
  float mp[4];
  for (int k = 0; k < 4; ++k) mp[k] = acc[k] / acc[3];
  float pr[4];
  vec_mul_m4f(mp, ata, pr);
  for (int k = 0; k < 4; ++k) pr[k] = atb[k] - pr[k];
  /* svd_solve_ATA_ATb + svd_solve_sym, qef_simd.h:304-406 */
  m4 V;
  memset(V, 0, sizeof(V));
  V[0][0] = V[1][1] = V[2][2] = 1.0f;
  m4 vtav;
  memcpy(vtav, ata, sizeof(vtav));
  for (int sweep = 0; sweep < 5; ++sweep) {
    static const int pairs[3][2] = {{0, 1}, {0, 2}, {1, 2}};
    for (int q = 0; q < 3; ++q) {
      int a = pairs[q][0], b = pairs[q][1];
      if (vtav[a][b] != 0.0f) {
        float c, s;
        givens_f(vtav, a, b, &c, &s);
        rotateq_f(vtav, c, s, a, b);
        rotate_f(vtav, V, c, s, a, b);
        vtav[a][b] = 0.0f;
      }
    }
  }
  float sigma[4] = {vtav[0][0], vtav[1][1], vtav[2][2], 0.0f};
  float invdet[4];
  for (int k = 0; k < 4; ++k) { /* svd_invdet, qef_simd.h:346-357 */
    float one_over = 1.0f / sigma[k];
    float a1 = fabsf(sigma[k]), a2 = fabsf(one_over);
    float mn = (a1 < a2) ? a1 : a2;
    invdet[k] = (mn >= 0.001f) ? one_over : 0.0f;
  }
  m4 mm, o;
  memset(o, 0, sizeof(o));
  for (int r = 0; r < 3; ++r)
    for (int k = 0; k < 4; ++k) mm[r][k] = V[r][k] * invdet[k];
  for (int r = 0; r < 3; ++r)
    for (int k = 0; k < 3; ++k) o[r][k] = dot4f(mm[k], V[r]);
  float x[4];
  vec_mul_m4f(pr, o, x);
  /* qef_simd_calc_error, qef_simd.h:434-440 */
  float t[4];
  vec_mul_m4f(x, ata, t);
  for (int k = 0; k < 4; ++k) t[k] = atb[k] - t[k];
  float err = dot4f(t, t);
  out[0] = x[0] + mp[0];
  out[1] = x[1] + mp[1];
  out[2] = x[2] + mp[2];
  return err;
}

/* FP64 twin of bmfo_qef_f32 (same algorithm, double throughout): the
 * accuracy reference the FP32 results are measured against. */
double bmfo_qef_f64(const double* pos, const double* nrm, int count, double* out) {
  if (count < 2 || count > 12) {
    out[0] = out[1] = out[2] = 0.0;
    return 0.0;
  }
  double ata[3][3] = {{0}}, atb[3] = {0}, acc[3] = {0};
  for (int i = 0; i < count; ++i) {
    const double* p = pos + 3 * i;
    const double* n = nrm + 3 * i;
    for (int r = 0; r < 3; ++r)
      for (int k = 0; k < 3; ++k) ata[r][k] += n[r] * n[k];
    double d = p[0] * n[0] + p[1] * n[1] + p[2] * n[2];
    for (int k = 0; k < 3; ++k) atb[k] += d * n[k];
    for (int k = 0; k < 3; ++k) acc[k] += p[k];
  }
  double mp[3] = {acc[0] / count, acc[1] / count, acc[2] / count};
  double pr[3];
  for (int k = 0; k < 3; ++k) pr[k] = atb[k] - (mp[0] * ata[0][k] + mp[1] * ata[1][k] + mp[2] * ata[2][k]);
  double A[3][3], V[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  memcpy(A, ata, sizeof(A));
  for (int sweep = 0; sweep < 5; ++sweep) {
    static const int pairs[3][2] = {{0, 1}, {0, 2}, {1, 2}};
    for (int q = 0; q < 3; ++q) {
      int a = pairs[q][0], b = pairs[q][1];
      if (A[a][b] == 0.0) continue;
      double tau = (A[b][b] - A[a][a]) / (2.0 * A[a][b]);
      double stt = sqrt(1.0 + tau * tau);
      double tn = 1.0 / (tau >= 0.0 ? tau + stt : tau - stt);
      double c = 1.0 / sqrt(1.0 + tn * tn), s = tn * c;
      /* full symmetric Jacobi rotation A <- J^T A J, V <- V J */
      for (int k = 0; k < 3; ++k) {
        double aka = A[k][a], akb = A[k][b];
        A[k][a] = c * aka - s * akb;
        A[k][b] = s * aka + c * akb;
      }
      for (int k = 0; k < 3; ++k) {
        double aak = A[a][k], abk = A[b][k];
        A[a][k] = c * aak - s * abk;
        A[b][k] = s * aak + c * abk;
      }
      A[a][b] = A[b][a] = 0.0;
      for (int k = 0; k < 3; ++k) {
        double vka = V[k][a], vkb = V[k][b];
        V[k][a] = c * vka - s * vkb;
        V[k][b] = s * vka + c * vkb;
      }
    }
  }
  double inv[3];
  for (int k = 0; k < 3; ++k) {
    double sg = A[k][k], oo = 1.0 / sg;
    double mn = fabs(sg) < fabs(oo) ? fabs(sg) : fabs(oo);
    inv[k] = mn >= 0.001 ? oo : 0.0;
  }
  double x[3] = {0, 0, 0};
  for (int r = 0; r < 3; ++r)
    for (int k = 0; k < 3; ++k) {
      double pinv = V[r][0] * inv[0] * V[k][0] + V[r][1] * inv[1] * V[k][1] + V[r][2] * inv[2] * V[k][2];
      x[k] += pr[r] * pinv;
    }
  double err = 0.0;
  for (int k = 0; k < 3; ++k) {
    double t = atb[k] - (x[0] * ata[0][k] + x[1] * ata[1][k] + x[2] * ata[2][k]);
    err += t * t;
  }
  for (int k = 0; k < 3; ++k) out[k] = x[k] + mp[k];
  return err;
}

/* ======================================================================== */
/* Mode Q: DMC / manifold dual contouring quads                              */
/* ======================================================================== */
/* Specification (this project's; the reference keeps only the tables,
 * Tables.hpp:76-354, and a commented-out quad pipeline):
 *  - cells are the interior cells (x,y,z) in [0, dim-2]^3 with their full
 *    8-corner mask; a cell with mask not 0/255 hosts one vertex per vertex
 *    group of its case, numbered in linear cell order (z fastest), groups in
 *    table order;
 *  - each sign-changing grid edge whose four surrounding cells all exist
 *    emits one quad, edges visited in linear order of their lower sample,
 *    axis x before y before z.  For an edge along axis a with the two other
 *    axes (b, c) = ((a+1)%3, (a+2)%3), the cells are taken at offsets
 *    (b, c) = (-1,-1), (0,-1), (0,0), (-1,0); that order is kept when the
 *    lower sample is inside (value < 0) and reversed (first cell fixed)
 *    when it is outside, which gives the quads the facing of the reference's
 *    Marching-Cubes triangles (normal = (v1-v0) x (v2-v0) points outward);
 *  - a vertex is a boundary vertex when its cell touches a chunk face. */

static const int q_corner[12][2] = {{0, 4}, {1, 5}, {2, 6}, {3, 7}, {0, 2}, {1, 3},
                                    {4, 6}, {5, 7}, {0, 1}, {2, 3}, {4, 5}, {6, 7}};

static int inside_bit(const uint32_t* words, int dim, int zc, int x, int y, int z) {
  return (int)((words[((size_t)x * dim + y) * zc + (z >> 5)] >> (z & 31)) & 1u);
}
static int full_mask(const uint32_t* words, int dim, int zc, int x, int y, int z) {
  int m = 0;
  for (int c = 0; c < 8; ++c)
    m |= inside_bit(words, dim, zc, x + ((c >> 2) & 1), y + ((c >> 1) & 1), z + (c & 1)) << c;
  return m;
}
static float dens(const float* d, int dim, int x, int y, int z) { return d[((size_t)x * dim + y) * dim + z]; }

/* Central-difference grid gradient, one-sided at the chunk faces, halved on
 * the central stencil: g = (s[+1] - s[-1]) * 0.5. */
static void grid_gradient(const float* d, int dim, int x, int y, int z, float g[3]) {
  int c[3] = {x, y, z};
  for (int a = 0; a < 3; ++a) {
    int lo[3] = {x, y, z}, hi[3] = {x, y, z};
    float h = 0.5f;
    if (c[a] > 0) lo[a]--; else h = 1.0f;
    if (c[a] < dim - 1) hi[a]++; else h = 1.0f;
    g[a] = (dens(d, dim, hi[0], hi[1], hi[2]) - dens(d, dim, lo[0], lo[1], lo[2])) * h;
  }
}

/* Crossing point and hermite normal of cell edge e (corners ca -> cb). */
static void hermite(const float* d, int dim, int x, int y, int z, int e, float p[3], float n[3]) {
  int ca = q_corner[e][0], cb = q_corner[e][1];
  int a0[3] = {x + ((ca >> 2) & 1), y + ((ca >> 1) & 1), z + (ca & 1)};
  int a1[3] = {x + ((cb >> 2) & 1), y + ((cb >> 1) & 1), z + (cb & 1)};
  float s0 = dens(d, dim, a0[0], a0[1], a0[2]), s1 = dens(d, dim, a1[0], a1[1], a1[2]);
  float mu = (0.0f - s0) / (s1 - s0);
  float g0[3], g1[3];
  if (n) {
    grid_gradient(d, dim, a0[0], a0[1], a0[2], g0);
    grid_gradient(d, dim, a1[0], a1[1], a1[2], g1);
  }
  for (int k = 0; k < 3; ++k) {
    float dv = ((float)a1[k] - (float)a0[k]) * mu;
    p[k] = dv + (float)a0[k];
  }
  if (n) {
    float g[3];
    for (int k = 0; k < 3; ++k) g[k] = g0[k] + (g1[k] - g0[k]) * mu;
    float l2 = (g[0] * g[0] + g[1] * g[1]) + g[2] * g[2];
    float inv = 1.0f / sqrtf(l2);
    for (int k = 0; k < 3; ++k) n[k] = g[k] * inv;
  }
}

static void place_group(const float* d, int dim, int x, int y, int z, int mask, int group, int placement,
                        float out[3], int* used_qef) {
  if (used_qef) *used_qef = 0;
  if (placement == 0) {
    out[0] = (float)x + 0.5f;
    out[1] = (float)y + 0.5f;
    out[2] = (float)z + 0.5f;
    return;
  }
  uint64_t gw = kBmfGroupCases[mask];
  float P[12 * 3], N[12 * 3];
  int cnt = 0;
  for (int e = 0; e < 12; ++e) {
    if ((int)((gw >> (4 * e)) & 0xF) != group) continue;
    hermite(d, dim, x, y, z, e, P + 3 * cnt, placement >= 2 ? N + 3 * cnt : NULL);
    ++cnt;
  }
  float mp[3] = {0, 0, 0};
  for (int i = 0; i < cnt; ++i)
    for (int k = 0; k < 3; ++k) mp[k] = mp[k] + P[3 * i + k];
  for (int k = 0; k < 3; ++k) mp[k] = mp[k] / (float)cnt;
  if (placement == 1) {
    memcpy(out, mp, sizeof(mp));
    return;
  }
  float q[3];
  if (placement == 2) {
    bmfo_qef_f32(P, N, cnt, q);
  } else {
    double Pd[36], Nd[36], qd[3];
    for (int i = 0; i < 3 * cnt; ++i) {
      Pd[i] = P[i];
      Nd[i] = N[i];
    }
    bmfo_qef_f64(Pd, Nd, cnt, qd);
    q[0] = (float)qd[0]; q[1] = (float)qd[1]; q[2] = (float)qd[2];
  }
  /* A solution outside the cell falls back to the mass point. */
  int ok = q[0] >= (float)x && q[0] <= (float)(x + 1) && q[1] >= (float)y && q[1] <= (float)(y + 1) &&
           q[2] >= (float)z && q[2] <= (float)(z + 1);
  memcpy(out, ok ? q : mp, sizeof(q));
  if (used_qef) *used_qef = ok;
}

int bmfo_place_q_f32(int dim, const float* density, int x, int y, int z, int mask, int group, float out[3]) {
  int used = 0;
  place_group(density, dim, x, y, z, mask, group, 2, out, &used);
  return used;
}

int bmfo_extract_q(int dim, const float* density, const uint32_t* words, int placement, int64_t vcap, int64_t icap,
                   float* vpos, uint8_t* vboundary, uint8_t* vvalence, uint32_t* idx, bmfo_counts* counts) {
  const int zc = (dim + 31) / 32;
  const int nc = dim - 1;
  const size_t ncell = (size_t)nc * nc * nc;
  uint32_t* vbase = (uint32_t*)malloc((ncell ? ncell : 1) * sizeof(uint32_t));
  uint8_t* cmask = (uint8_t*)malloc(ncell ? ncell : 1);
  int64_t nv = 0, ni = 0, ncells = 0;
  int overflow = 0;
  for (int x = 0; x < nc; ++x)
    for (int y = 0; y < nc; ++y)
      for (int z = 0; z < nc; ++z) {
        size_t c = ((size_t)x * nc + y) * nc + z;
        int m = full_mask(words, dim, zc, x, y, z);
        cmask[c] = (uint8_t)m;
        vbase[c] = (uint32_t)nv;
        if (m == 0 || m == 255) continue;
        ++ncells;
        int ng = (int)((kBmfGroupCases[m] >> 48) & 0xF);
        for (int g = 0; g < ng; ++g, ++nv) {
          if (nv >= vcap) {
            overflow = 1;
            continue;
          }
          if (vpos) place_group(density, dim, x, y, z, m, g, placement, vpos + 3 * nv, NULL);
          if (vboundary) vboundary[nv] = (x == 0 || y == 0 || z == 0 || x == nc - 1 || y == nc - 1 || z == nc - 1);
          if (vvalence) vvalence[nv] = 0;
        }
      }
  static const int ob[4] = {-1, 0, 0, -1}, oc[4] = {-1, -1, 0, 0};
  for (int x = 0; x < dim; ++x)
    for (int y = 0; y < dim; ++y)
      for (int z = 0; z < dim; ++z) {
        int s[3] = {x, y, z};
        int in0 = inside_bit(words, dim, zc, x, y, z);
        for (int a = 0; a < 3; ++a) {
          int b = (a + 1) % 3, cax = (a + 2) % 3;
          if (s[a] > dim - 2 || s[b] < 1 || s[b] > dim - 2 || s[cax] < 1 || s[cax] > dim - 2) continue;
          int t[3] = {x, y, z};
          t[a]++;
          if (inside_bit(words, dim, zc, t[0], t[1], t[2]) == in0) continue;
          uint32_t q[4];
          for (int k = 0; k < 4; ++k) {
            int cc[3] = {x, y, z};
            cc[b] += ob[k];
            cc[cax] += oc[k];
            int lo[3] = {0, 0, 0}; /* edge's offset inside this cell */
            lo[b] = -ob[k];
            lo[cax] = -oc[k];
            int e = a == 0 ? 2 * lo[1] + lo[2] : (a == 1 ? 4 + 2 * lo[0] + lo[2] : 8 + 2 * lo[0] + lo[1]);
            size_t ci = ((size_t)cc[0] * nc + cc[1]) * nc + cc[2];
            int g = (int)((kBmfGroupCases[cmask[ci]] >> (4 * e)) & 0xF);
            q[k] = vbase[ci] + (uint32_t)g;
          }
          uint32_t o[4] = {q[0], q[1], q[2], q[3]};
          if (!in0) {
            o[1] = q[3];
            o[3] = q[1];
          }
          for (int k = 0; k < 4; ++k) {
            if (ni < icap) {
              if (idx) idx[ni] = o[k];
            } else {
              overflow = 1;
            }
            if (vvalence && (int64_t)o[k] < vcap) vvalence[o[k]]++;
            ++ni;
          }
        }
      }
  if (counts) {
    counts->n_cells = ncells;
    counts->n_verts = nv;
    counts->n_idx = ni;
  }
  free(vbase);
  free(cmask);
  return overflow ? -1 : 0;
}

/* ======================================================================== */
/* MeshProcessor<N> (MeshProcessor.cpp:26-306)                               */
/* ======================================================================== */

static void v3norm(const float v[3], float out[3]) {
  float l2 = (v[0] * v[0] + v[1] * v[1]) + v[2] * v[2];
  float inv = 1.0f / sqrtf(l2);
  out[0] = v[0] * inv;
  out[1] = v[1] * inv;
  out[2] = v[2] * inv;
}
static void v3cross(const float a[3], const float b[3], float o[3]) {
  o[0] = a[1] * b[2] - b[1] * a[2];
  o[1] = a[2] * b[0] - b[2] * a[0];
  o[2] = a[0] * b[1] - b[0] * a[1];
}
static void v3sub(const float* a, const float* b, float o[3]) {
  o[0] = a[0] - b[0];
  o[1] = a[1] - b[1];
  o[2] = a[2] - b[2];
}

/* WorldOctree::split_leaves (WorldOctree.cpp:129-161): depth-first with an
 * explicit stack (children pushed 0..7 at the MCDX/MCDY/MCDZ offsets of
 * WorldOctree.cpp:177-199 / Tables.hpp:7-9, popped last-in first-out);
 * node_needs_split (WorldOctree.cpp:237-247) with middle = pos + size / 2
 * (WorldOctreeNode.cpp:27); each leaf framed like DMCChunk::label_grid
 * (DMCChunk.cpp:94-97) with ChunkGenerator.cpp:98's overlap.  prm: root
 * xyz, root size, focus xyz, split_multiplier, size_modifier, base_overlap;
 * out rows: origin xyz, scale, dim, level.  Returns the leaf count (at most
 * cap rows written) or -1 when the stack would exceed 64 * 8 entries. */
int64_t bmfo_lod_generate(const float* prm, int min_level, int max_level, int dim, int boundary_processing,
                          int iters, float* out, int64_t cap) {
  typedef struct { float p[3], size; int level; } node;
  node stack[64 * 8 + 8];
  int top = 0;
  int64_t n = 0;
  static const int mx[8] = {0, 1, 1, 0, 0, 1, 1, 0}, my[8] = {0, 0, 0, 0, 1, 1, 1, 1}, mz[8] = {0, 0, 1, 1, 0, 0, 1, 1};
  node r = {{prm[0], prm[1], prm[2]}, prm[3], 0};
  stack[top++] = r;
  while (top > 0) {
    node c = stack[--top];
    int split;
    if (c.level >= max_level) split = 0;
    else if (c.level < min_level) split = 1;
    else {
      float m[3], d[3];
      for (int k = 0; k < 3; ++k) m[k] = c.p[k] + c.size * 0.5f;
      for (int k = 0; k < 3; ++k) d[k] = prm[4 + k] - m[k];
      float dist = sqrtf((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]);
      split = dist < (c.size * prm[7] + prm[8]) + c.size * 0.5f;
    }
    if (!split) {
      if (n < cap) {
        float ov = (c.level == max_level && (!boundary_processing || iters == 0)) ? 0.0f
                                                                                : prm[9] + 0.005f * (float)iters;
        float delta = c.size * (1.0f + ov * 2.0f) / (float)(dim - 1);
        float shift = c.size * ov;
        float* o = out + 6 * n;
        o[0] = c.p[0] - shift;
        o[1] = c.p[1] - shift;
        o[2] = c.p[2] - shift;
        o[3] = delta;
        o[4] = (float)dim;
        o[5] = (float)c.level;
      }
      ++n;
      continue;
    }
    if (top + 8 > 64 * 8) return -1;
    float cs = c.size * 0.5f;
    for (int i = 0; i < 8; ++i) {
      node ch = {{c.p[0] + (float)mx[i] * cs, c.p[1] + (float)my[i] * cs, c.p[2] + (float)mz[i] * cs},
                 c.size * 0.5f, c.level + 1};
      stack[top++] = ch;
    }
  }
  return n;
}

/* GLChunk::format_data (GLChunk.cpp:278-335).  unwind == 0: p, n, c per
 * vertex (c is white: DMCChunk.cpp:681 sets (1, 1, 1) and the sweeps only
 * average colours).  unwind == 1: per quad (i += 4) its 4 corners, one normal
 * for all four: smooth ? (n0 + n1 + n2 + n3) * 0.25 : -normalize((m0 + m1) *
 * 0.5) with m0 = cross(normalize(p0 - p1), normalize(p0 - p2)),
 * m1 = cross(normalize(p2 - p3), normalize(p2 - p0)), a NaN x taking the
 * other.  Returns the vertices written. */
int64_t bmfo_format(int64_t nverts, const float* pos, const float* nrm, int64_t nidx, const uint32_t* idx, int unwind,
                    int smooth_normals, float* p, float* n, float* c) {
  if (!unwind) {
    for (int64_t i = 0; i < nverts; ++i)
      for (int k = 0; k < 3; ++k) {
        p[3 * i + k] = pos[3 * i + k];
        n[3 * i + k] = nrm ? nrm[3 * i + k] : 0.0f;
        c[3 * i + k] = 1.0f;
      }
    return nverts;
  }
  for (int64_t i = 0; i + 3 < nidx; i += 4) {
    const float* q[4];
    for (int k = 0; k < 4; ++k) q[k] = pos + 3 * (int64_t)idx[i + k];
    float m[3];
    if (smooth_normals) {
      for (int k = 0; k < 3; ++k) {
        float s = nrm[3 * (int64_t)idx[i] + k] + nrm[3 * (int64_t)idx[i + 1] + k];
        s = s + nrm[3 * (int64_t)idx[i + 2] + k];
        s = s + nrm[3 * (int64_t)idx[i + 3] + k];
        m[k] = s * 0.25f;
      }
    } else {
      float a[3], b[3], na[3], nb[3], m0[3], m1[3], h[3], o[3];
      v3sub(q[0], q[1], a);
      v3sub(q[0], q[2], b);
      v3norm(a, na);
      v3norm(b, nb);
      v3cross(na, nb, m0);
      v3sub(q[2], q[3], a);
      v3sub(q[2], q[0], b);
      v3norm(a, na);
      v3norm(b, nb);
      v3cross(na, nb, m1);
      if (isnan(m0[0])) memcpy(m0, m1, sizeof(m0));
      if (isnan(m1[0])) memcpy(m1, m0, sizeof(m1));
      for (int k = 0; k < 3; ++k) h[k] = (m0[k] + m1[k]) * 0.5f;
      v3norm(h, o);
      for (int k = 0; k < 3; ++k) m[k] = -o[k];
    }
    for (int j = 0; j < 4; ++j)
      for (int k = 0; k < 3; ++k) {
        p[3 * (i + j) + k] = q[j][k];
        n[3 * (i + j) + k] = m[k];
        c[3 * (i + j) + k] = 1.0f;
      }
  }
  return nidx / 4 * 4;
}

void bmfo_process(int N, int64_t nverts, float* pos, float* nrm, const uint8_t* vboundary, const uint8_t* vvalence,
                  int64_t nidx, const uint32_t* idx, int iters, int process_boundary, int smooth_normals) {
  if (nverts == 0 || nidx < N) return; /* MeshProcessor.cpp:28-29 */
  int64_t nprim = nidx / N;
  /* init: CSR offsets by exclusive scan of init_valence; init_primitives
   * fills each vertex's list with prim ids in ascending order (:26-128). */
  int64_t* off = (int64_t*)malloc((size_t)(nverts + 1) * sizeof(int64_t));
  int64_t a_count = 0;
  for (int64_t v = 0; v < nverts; ++v) {
    off[v] = a_count;
    a_count += vvalence[v];
  }
  off[nverts] = a_count;
  if (!a_count) {
    free(off);
    return;
  }
  uint32_t* adj = (uint32_t*)malloc((size_t)a_count * sizeof(uint32_t));
  int* nxt = (int*)calloc((size_t)nverts, sizeof(int));
  for (int64_t t = 0; t < nprim; ++t)
    for (int k = 0; k < N; ++k) {
      uint32_t v = idx[N * t + k];
      adj[off[v] + nxt[v]++] = (uint32_t)t;
    }
  float* dp = (float*)malloc((size_t)nprim * 3 * sizeof(float));
  float* dn = (float*)malloc((size_t)nprim * 3 * sizeof(float));
  const int hard_norm_max = 10;
  int max_norms = (iters / 2 - 3 < hard_norm_max ? iters / 2 - 3 : hard_norm_max);
  for (int pass = 0; pass <= iters; ++pass) {
    int m = pass;
    if (pass < iters) {
      /* optimize_dual_grid body, MeshProcessor.cpp:142-227 */
      for (int64_t t = 0; t < nprim; ++t) {
        const uint32_t* tv = idx + N * t;
        float p[3] = {0, 0, 0};
        for (int k = 0; k < N; ++k)
          for (int c = 0; c < 3; ++c) p[c] = p[c] + pos[3 * tv[k] + c];
        for (int c = 0; c < 3; ++c) dp[3 * t + c] = p[c] / (float)N;
        if (!smooth_normals) continue;
        if (m == 0 || m < max_norms || m < 3) {
          float a[3] = {0, 0, 0}, b[3] = {0, 0, 0}, na[3], nb[3], o[3];
          if (N == 3) {
            if (tv[0] != tv[1] && tv[1] != tv[2] && tv[0] != tv[2]) {
              v3sub(pos + 3 * tv[0], pos + 3 * tv[1], a);
              v3sub(pos + 3 * tv[0], pos + 3 * tv[2], b);
            }
            v3norm(a, na);
            v3norm(b, nb);
            v3cross(na, nb, o);
            for (int c = 0; c < 3; ++c) dn[3 * t + c] = -o[c];
          } else {
            float n1[3], n2[3];
            v3sub(pos + 3 * tv[0], pos + 3 * tv[1], a);
            v3sub(pos + 3 * tv[0], pos + 3 * tv[2], b);
            v3norm(a, na);
            v3norm(b, nb);
            v3cross(na, nb, n1);
            v3sub(pos + 3 * tv[2], pos + 3 * tv[3], a);
            v3sub(pos + 3 * tv[2], pos + 3 * tv[0], b);
            v3norm(a, na);
            v3norm(b, nb);
            v3cross(na, nb, n2);
            if (isnan(n1[0])) {
              memcpy(n1, n2, sizeof(n1));
              if (isnan(n1[0])) {
                n1[0] = 0.0f; n1[1] = 1.0f; n1[2] = 0.0f;
              }
            }
            if (isnan(n2[0])) memcpy(n2, n1, sizeof(n2));
            float h[3] = {(n1[0] + n2[0]) * 0.5f, (n1[1] + n2[1]) * 0.5f, (n1[2] + n2[2]) * 0.5f};
            v3norm(h, o);
            for (int c = 0; c < 3; ++c) dn[3 * t + c] = -o[c];
          }
        } else {
          float n[3] = {0, 0, 0};
          for (int k = 0; k < N; ++k)
            for (int c = 0; c < 3; ++c) n[c] = n[c] + nrm[3 * tv[k] + c];
          for (int c = 0; c < 3; ++c) dn[3 * t + c] = n[c];
        }
      }
    }
    /* optimize_primal_grid, MeshProcessor.cpp:238-306: after every dual step
     * but the last inside optimize_dual_grid (:229-232), then once more from
     * ChunkGenerator.cpp:120 with set_colors false. */
    if (pass == iters - 1) continue;
    if (pass == iters && iters == 0) break;
    int set_colors = pass < iters ? ((m == 3) || (m == 0 && iters <= 3)) : 0;
    float* newp = (float*)malloc((size_t)nverts * 3 * sizeof(float));
    float* newn = (float*)malloc((size_t)nverts * 3 * sizeof(float));
    memcpy(newp, pos, (size_t)nverts * 3 * sizeof(float));
    memcpy(newn, nrm, (size_t)nverts * 3 * sizeof(float));
    for (int64_t v = 0; v < nverts; ++v) {
      if (nxt[v] == 0 || (!process_boundary && vboundary[v])) continue;
      float p[3] = {0, 0, 0}, n[3] = {0, 0, 0};
      int count = 0;
      for (int k = 0; k < nxt[v]; ++k) {
        uint32_t t = adj[off[v] + k];
        ++count;
        for (int c = 0; c < 3; ++c) p[c] = p[c] + dp[3 * t + c];
        if (smooth_normals)
          for (int c = 0; c < 3; ++c) n[c] = n[c] + dn[3 * t + c];
      }
      for (int c = 0; c < 3; ++c) p[c] = p[c] / (float)count;
      if (smooth_normals)
        for (int c = 0; c < 3; ++c) n[c] = n[c] / (float)count;
      if (set_colors) {
        float o[3];
        v3norm(n, o);
        memcpy(n, o, sizeof(o));
      }
      memcpy(newp + 3 * v, p, sizeof(p));
      if (n[1] != 0.0f) memcpy(newn + 3 * v, n, sizeof(n));
    }
    memcpy(pos, newp, (size_t)nverts * 3 * sizeof(float));
    memcpy(nrm, newn, (size_t)nverts * 3 * sizeof(float));
    free(newp);
    free(newn);
  }
  free(off);
  free(adj);
  free(nxt);
  free(dp);
  free(dn);
}

/* ======================================================================== */
/* CPU baseline: whole path over a batch, OpenMP over chunks                 */
/* ======================================================================== */

/* FNV-1a (64-bit) of a byte range.  f32_canon != 0 reads the range as floats
 * and hashes every NaN as the canonical quiet NaN 0x7FC00000 (x86, Arm and the
 * GPU encode a NaN's sign and payload differently). */
uint64_t bmfo_digest64(const void* data, int64_t n_bytes, int f32_canon) {
  uint64_t h = 0xcbf29ce484222325ull;
  const uint8_t* b = (const uint8_t*)data;
  if (f32_canon) {
    for (int64_t i = 0; i + 4 <= n_bytes; i += 4) {
      uint32_t u;
      memcpy(&u, b + i, 4);
      if ((u & 0x7F800000u) == 0x7F800000u && (u & 0x007FFFFFu)) u = 0x7FC00000u;
      for (int k = 0; k < 4; ++k) {
        h ^= (u >> (8 * k)) & 0xFFu;
        h *= 0x100000001b3ull;
      }
    }
    return h;
  }
  for (int64_t i = 0; i < n_bytes; ++i) {
    h ^= b[i];
    h *= 0x100000001b3ull;
  }
  return h;
}

/* ChunkGenerator::extract_chunk (ChunkGenerator.cpp:80-147): per chunk, fill ->
 * label_grid -> label_edges + polygonize (Mode R) or the Mode Q emitter ->
 * MeshProcessor, OpenMP over chunks as the reference's batch loop. */
int64_t bmfo_extract_batch_digest(int n_chunks, const float* desc, int field, const float* params, int mode,
                                  int placement, int iters, int process_boundary, int smooth_normals,
                                  int64_t* out_counts, uint64_t* out_digest, int n_threads) {
  int64_t total = 0;
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#endif
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : total)
  for (int i = 0; i < n_chunks; ++i) {
    const float* d = desc + 5 * i;
    int dim = (int)d[4];
    int zc = (dim + 31) / 32;
    size_t n = (size_t)dim * dim * dim;
    float* dens_buf = (float*)malloc(n * sizeof(float));
    uint32_t* words = (uint32_t*)malloc((size_t)dim * dim * zc * sizeof(uint32_t));
    bmfo_fill_field(field, params, dim, d, d[3], dens_buf);
    int cm = bmfo_label_grid(dim, dens_buf, words);
    bmfo_counts c = {0, 0, 0};
    float* vp = NULL;
    float* vn = NULL;
    uint8_t* vb = NULL;
    uint8_t* vv = NULL;
    uint32_t* ix = NULL;
    if (cm) {
      bmfo_counts cnt;
      uint64_t* masks = NULL;
      if (mode == 0) {
        masks = (uint64_t*)malloc((size_t)dim * dim * 4 * zc * sizeof(uint64_t));
        bmfo_cell_masks(dim, words, masks);
        bmfo_extract_r(dim, dens_buf, masks, 0, 0, 0, NULL, NULL, NULL, NULL, NULL, NULL, &cnt);
      } else {
        bmfo_extract_q(dim, dens_buf, words, placement, 0, 0, NULL, NULL, NULL, NULL, &cnt);
      }
      int64_t vcap = cnt.n_verts, icap = cnt.n_idx;
      vp = (float*)malloc((size_t)(vcap ? vcap : 1) * 3 * sizeof(float));
      vn = (float*)calloc((size_t)(vcap ? vcap : 1) * 3, sizeof(float));
      vb = (uint8_t*)malloc((size_t)(vcap ? vcap : 1));
      vv = (uint8_t*)malloc((size_t)(vcap ? vcap : 1));
      ix = (uint32_t*)malloc((size_t)(icap ? icap : 1) * sizeof(uint32_t));
      if (mode == 0)
        bmfo_extract_r(dim, dens_buf, masks, vcap, icap, 0, vp, vb, vv, ix, NULL, NULL, &c);
      else
        bmfo_extract_q(dim, dens_buf, words, placement, vcap, icap, vp, vb, vv, ix, &c);
      if (iters > 0)
        bmfo_process(mode == 0 ? 3 : 4, c.n_verts, vp, vn, vb, vv, c.n_idx, ix, iters, process_boundary,
                     smooth_normals);
      free(masks);
    }
    if (out_counts) {
      out_counts[3 * i] = cm;
      out_counts[3 * i + 1] = c.n_verts;
      out_counts[3 * i + 2] = c.n_idx;
    }
    if (out_digest) {
      /* {indices, positions, boundary flags, normals} of the chunk's mesh */
      out_digest[4 * i + 0] = bmfo_digest64(ix, c.n_idx * 4, 0);
      out_digest[4 * i + 1] = bmfo_digest64(vp, c.n_verts * 12, 1);
      out_digest[4 * i + 2] = bmfo_digest64(vb, c.n_verts, 0);
      out_digest[4 * i + 3] = bmfo_digest64(vn, c.n_verts * 12, 1);
    }
    total += c.n_verts;
    free(vp); free(vn); free(vb); free(vv); free(ix);
    free(dens_buf);
    free(words);
  }
  return total;
}

int64_t bmfo_extract_batch(int n_chunks, const float* desc, int field, const float* params, int mode, int placement,
                           int iters, int smooth_normals, int64_t* out_counts, int n_threads) {
  return bmfo_extract_batch_digest(n_chunks, desc, field, params, mode, placement, iters, 0, smooth_normals,
                                   out_counts, NULL, n_threads);
}
