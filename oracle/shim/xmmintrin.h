// Portable stand-in for the SSE intrinsics used by the reference's qef_simd.h.
// Test infrastructure only.  It gives __m128 the MSVC-style m128_f32[] member
// the reference indexes, and implements each intrinsic lane by lane with the
// same IEEE single-precision semantics as the SSE instruction.  The one
// approximate instruction, rsqrtps, is issued through the compiler builtin on
// x86 so the compiled reference keeps the hardware approximation; elsewhere it
// falls back to the correctly rounded 1/sqrt.
#pragma once
#include <cmath>
#include <cstring>
#include <cstdint>

struct __m128 { float m128_f32[4]; };
struct __m256 { float m256_f32[8]; };

#define _MM_SHUFFLE(z, y, x, w) (((z) << 6) | ((y) << 4) | ((x) << 2) | (w))

static inline uint32_t bmf_shim_bits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
static inline float bmf_shim_float(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }

static inline __m128 _mm_set_ps(float e3, float e2, float e1, float e0) { __m128 r; r.m128_f32[0] = e0; r.m128_f32[1] = e1; r.m128_f32[2] = e2; r.m128_f32[3] = e3; return r; }
static inline __m128 _mm_set1_ps(float v) { return _mm_set_ps(v, v, v, v); }
static inline __m128 _mm_load1_ps(const float* p) { return _mm_set1_ps(*p); }
static inline __m128 _mm_load_ps(const float* p) { __m128 r; std::memcpy(r.m128_f32, p, 16); return r; }
static inline void _mm_store_ps(float* p, __m128 a) { std::memcpy(p, a.m128_f32, 16); }
static inline float _mm_cvtss_f32(__m128 a) { return a.m128_f32[0]; }

#define BMF_SHIM_LANEWISE(name, expr) \
  static inline __m128 name(__m128 a, __m128 b) { __m128 r; for (int i = 0; i < 4; ++i) { float x = a.m128_f32[i], y = b.m128_f32[i]; (void)y; r.m128_f32[i] = (expr); } return r; }
BMF_SHIM_LANEWISE(_mm_add_ps, x + y)
BMF_SHIM_LANEWISE(_mm_sub_ps, x - y)
BMF_SHIM_LANEWISE(_mm_mul_ps, x * y)
BMF_SHIM_LANEWISE(_mm_div_ps, x / y)
BMF_SHIM_LANEWISE(_mm_min_ps, (x < y) ? x : y)
BMF_SHIM_LANEWISE(_mm_max_ps, (x > y) ? x : y)
BMF_SHIM_LANEWISE(_mm_cmpge_ps, bmf_shim_float((x >= y) ? 0xFFFFFFFFu : 0u))
BMF_SHIM_LANEWISE(_mm_cmpeq_ps, bmf_shim_float((x == y) ? 0xFFFFFFFFu : 0u))
BMF_SHIM_LANEWISE(_mm_and_ps, bmf_shim_float(bmf_shim_bits(x) & bmf_shim_bits(y)))
BMF_SHIM_LANEWISE(_mm_andnot_ps, bmf_shim_float(~bmf_shim_bits(x) & bmf_shim_bits(y)))
BMF_SHIM_LANEWISE(_mm_or_ps, bmf_shim_float(bmf_shim_bits(x) | bmf_shim_bits(y)))
#undef BMF_SHIM_LANEWISE

static inline __m128 _mm_sqrt_ps(__m128 a) { __m128 r; for (int i = 0; i < 4; ++i) r.m128_f32[i] = std::sqrt(a.m128_f32[i]); return r; }
static inline __m128 _mm_rsqrt_ps(__m128 a) {
  __m128 r;
#if defined(__x86_64__) || defined(__i386__)
  typedef float bmf_v4sf __attribute__((__vector_size__(16)));
  bmf_v4sf v; std::memcpy(&v, a.m128_f32, 16);
  bmf_v4sf o = __builtin_ia32_rsqrtps(v);
  std::memcpy(r.m128_f32, &o, 16);
#else
  for (int i = 0; i < 4; ++i) r.m128_f32[i] = 1.0f / std::sqrt(a.m128_f32[i]);
#endif
  return r;
}
static inline __m128 bmf_shim_shuffle(__m128 a, __m128 b, int imm) {
  __m128 r;
  r.m128_f32[0] = a.m128_f32[imm & 3];
  r.m128_f32[1] = a.m128_f32[(imm >> 2) & 3];
  r.m128_f32[2] = b.m128_f32[(imm >> 4) & 3];
  r.m128_f32[3] = b.m128_f32[(imm >> 6) & 3];
  return r;
}
#define _mm_shuffle_ps(a, b, imm) bmf_shim_shuffle((a), (b), (imm))

static inline __m128 bmf_shim_lo(const __m256& a) { __m128 r; std::memcpy(r.m128_f32, a.m256_f32, 16); return r; }
static inline __m128 bmf_shim_hi(const __m256& a) { __m128 r; std::memcpy(r.m128_f32, a.m256_f32 + 4, 16); return r; }
static inline __m256 bmf_shim_join(__m128 lo, __m128 hi) { __m256 r; std::memcpy(r.m256_f32, lo.m128_f32, 16); std::memcpy(r.m256_f32 + 4, hi.m128_f32, 16); return r; }
static inline __m256 _mm256_mul_ps(__m256 a, __m256 b) { return bmf_shim_join(_mm_mul_ps(bmf_shim_lo(a), bmf_shim_lo(b)), _mm_mul_ps(bmf_shim_hi(a), bmf_shim_hi(b))); }
static inline __m256 _mm256_add_ps(__m256 a, __m256 b) { return bmf_shim_join(_mm_add_ps(bmf_shim_lo(a), bmf_shim_lo(b)), _mm_add_ps(bmf_shim_hi(a), bmf_shim_hi(b))); }
static inline __m256 _mm256_broadcast_ps(const __m128* p) { return bmf_shim_join(*p, *p); }
static inline __m256 bmf_shim_shuffle256(__m256 a, __m256 b, int imm) { return bmf_shim_join(bmf_shim_shuffle(bmf_shim_lo(a), bmf_shim_lo(b), imm), bmf_shim_shuffle(bmf_shim_hi(a), bmf_shim_hi(b), imm)); }
#define _mm256_shuffle_ps(a, b, imm) bmf_shim_shuffle256((a), (b), (imm))
