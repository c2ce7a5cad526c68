// The MeshProcessor sweep steps for one primitive (dual) and one vertex
// (primal), shared by the whole-mesh kernels (bmf_process.cu) and the
// chunk-by-chunk kernel (bmf_extract.cu).  MeshProcessor.cpp:130-306.
#pragma once

#include "bmf_device.cuh"

namespace bmf {

// Threads of the chunk-by-chunk sweep kernel's CTA and CTAs per SM: Mode R
// at full occupancy (1024 x 2, 32 registers); Mode Q, whose adjacency keeps a
// 12-entry list per vertex, at 512 threads without a register cap.
template <int MODE>
__host__ __device__ constexpr int chunk_sweep_threads() { return MODE == 0 ? 1024 : 512; }
template <int MODE>
__host__ __device__ constexpr int chunk_sweep_min_ctas() { return MODE == 0 ? 2 : 1; }

// COH selects the load for data that the same kernel also writes (positions,
// normals and dual values in the chunk-by-chunk kernel, which runs every
// sweep in one launch, and its adjacency): a plain L1-cached load, which
// block barriers order.  Otherwise the read-only path.
template <bool COH, typename T>
__device__ __forceinline__ T sweep_ld(const T* p) {
  if (COH) return __ldca(p);
  return __ldg(p);
}

__device__ __forceinline__ void nrm3(const float v[3], float o[3]) {
  const float l2 = (v[0] * v[0] + v[1] * v[1]) + v[2] * v[2];
  const float inv = 1.0f / sqrtf(l2);
  o[0] = v[0] * inv;
  o[1] = v[1] * inv;
  o[2] = v[2] * inv;
}
__device__ __forceinline__ void cross3(const float a[3], const float b[3], float o[3]) {
  o[0] = a[1] * b[2] - b[1] * a[2];
  o[1] = a[2] * b[0] - b[2] * a[0];
  o[2] = a[0] * b[1] - b[0] * a[1];
}

// optimize_dual_grid body (MeshProcessor.cpp:142-227).  normal_mode: 0 none,
// 1 face normal, 2 sum of vertex normals.  PACKED: primitive t's dual point
// and normal go to ((float4*)dual_p)[t] = (p, n.x) and ((float2*)dual_n)[t] =
// (n.y, n.z) -- one 16-byte and one 8-byte gather per primitive in the primal
// step instead of six 4-byte ones; the values are the same.  I: the index
// type of t and nvb -- int64_t over a whole mesh, or uint32_t within one
// chunk (idx and the dual arrays then start at the chunk's first primitive;
// vertex ids stay mesh-wide).
template <int N, bool COH = false, bool PACKED = false, typename I = int64_t>
__device__ __forceinline__ void dual_prim(I t, I nvb, const uint32_t* __restrict__ idx,
                                          const float* __restrict__ pos, const float* __restrict__ nrm,
                                          float* __restrict__ dual_p, float* __restrict__ dual_n, int normal_mode) {
  uint32_t v[N];
#pragma unroll
  for (int k = 0; k < N; ++k) {
    v[k] = __ldg(idx + N * t + k);
    if ((I)v[k] >= nvb) v[k] = 0;  // an index outside the mesh reads vertex 0 instead of faulting
  }
  // each corner position is loaded once; the centroid and the face normal
  // read the same registers
  float P[N][3];
#pragma unroll
  for (int k = 0; k < N; ++k)
#pragma unroll
    for (int c = 0; c < 3; ++c) P[k][c] = sweep_ld<COH>(pos + 3 * v[k] + c);
  float p[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
  for (int k = 0; k < N; ++k) {
#pragma unroll
    for (int c = 0; c < 3; ++c) p[c] = p[c] + P[k][c];
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) p[c] = p[c] / (float)N;
  if (normal_mode == 0) {
    if (PACKED) {
      reinterpret_cast<float4*>(dual_p)[t] = make_float4(p[0], p[1], p[2], 0.0f);
    } else {
#pragma unroll
      for (int c = 0; c < 3; ++c) dual_p[3 * t + c] = p[c];
    }
    return;
  }
  float o[3];
  if (normal_mode == 1) {
    if (N == 3) {
      float a[3] = {0.0f, 0.0f, 0.0f}, b[3] = {0.0f, 0.0f, 0.0f}, na[3], nb[3];
      if (v[0] != v[1] && v[1] != v[2] && v[0] != v[2]) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          a[c] = P[0][c] - P[1][c];
          b[c] = P[0][c] - P[2][c];
        }
      }
      nrm3(a, na);
      nrm3(b, nb);
      cross3(na, nb, o);
#pragma unroll
      for (int c = 0; c < 3; ++c) o[c] = -o[c];
    } else {
      float a[3], b[3], na[3], nb[3], n1[3], n2[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        a[c] = P[0][c] - P[1][c];
        b[c] = P[0][c] - P[2][c];
      }
      nrm3(a, na);
      nrm3(b, nb);
      cross3(na, nb, n1);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        a[c] = P[2][c] - P[N - 1][c];
        b[c] = P[2][c] - P[0][c];
      }
      nrm3(a, na);
      nrm3(b, nb);
      cross3(na, nb, n2);
      if (isnan(n1[0])) {
        n1[0] = n2[0]; n1[1] = n2[1]; n1[2] = n2[2];
        if (isnan(n1[0])) { n1[0] = 0.0f; n1[1] = 1.0f; n1[2] = 0.0f; }
      }
      if (isnan(n2[0])) { n2[0] = n1[0]; n2[1] = n1[1]; n2[2] = n1[2]; }
      const float h[3] = {(n1[0] + n2[0]) * 0.5f, (n1[1] + n2[1]) * 0.5f, (n1[2] + n2[2]) * 0.5f};
      nrm3(h, o);
#pragma unroll
      for (int c = 0; c < 3; ++c) o[c] = -o[c];
    }
  } else {
    o[0] = o[1] = o[2] = 0.0f;
#pragma unroll
    for (int k = 0; k < N; ++k) {
#pragma unroll
      for (int c = 0; c < 3; ++c) o[c] = o[c] + sweep_ld<COH>(nrm + 3 * v[k] + c);
    }
  }
  if (PACKED) {
    reinterpret_cast<float4*>(dual_p)[t] = make_float4(p[0], p[1], p[2], o[0]);
    reinterpret_cast<float2*>(dual_n)[t] = make_float2(o[1], o[2]);
  } else {
#pragma unroll
    for (int c = 0; c < 3; ++c) dual_p[3 * t + c] = p[c];
#pragma unroll
    for (int c = 0; c < 3; ++c) dual_n[3 * t + c] = o[c];
  }
}

// I: the index type of v and np_lim, as for dual_prim (within one chunk, off,
// cursor, valence, boundary, pos and nrm start at the chunk's first vertex;
// adjacency offsets and primitive ids stay mesh-wide).
// AT = uint16_t: the lists hold 16-bit ids relative to the chunk's first
// primitive (dual_p / dual_n then start there), stored from adj + abase on
// with the CSR offsets counted from abase.
template <bool COH = false, bool PACKED = false, typename I = int64_t, typename AT = uint32_t>
__device__ __forceinline__ void primal_vertex(I v, I np_lim, int64_t adj_cap,
                                              const uint32_t* __restrict__ off, const uint32_t* __restrict__ cursor,
                                              const uint8_t* __restrict__ valence, const uint32_t* __restrict__ adj,
                                              const uint8_t* __restrict__ boundary, const float* __restrict__ dual_p,
                                              const float* __restrict__ dual_n, float* __restrict__ pos,
                                              float* __restrict__ nrm, int process_boundary, int smooth_normals,
                                              int set_colors, int64_t abase = 0) {
  // list length: adj_next (MeshProcessor.cpp:247); with a prebuilt adjacency it equals init_valence
  const uint32_t ov = sweep_ld<COH>(off + v);
  const int64_t room = adj_cap - (int64_t)ov;
  const uint32_t n = (uint32_t)max((int64_t)0, min((int64_t)(cursor ? min(cursor[v], (uint32_t)valence[v])
                                                                    : (uint32_t)valence[v]), room));
  if (n == 0 || (!process_boundary && boundary[v])) return;
  const AT* a = reinterpret_cast<const AT*>(adj + abase) + ((int64_t)ov - abase);
  float p[3] = {0.0f, 0.0f, 0.0f}, nn[3] = {0.0f, 0.0f, 0.0f};
  uint32_t k0 = 0;
  if (PACKED) {
    // two primitives per step: both gathers are issued before the sums,
    // which keep the one-by-one order (the same rounding)
    for (; k0 + 2 <= n; k0 += 2) {
      const uint32_t t0 = sweep_ld<COH>(a + k0), t1 = sweep_ld<COH>(a + k0 + 1);
      const bool ok0 = (I)t0 < np_lim, ok1 = (I)t1 < np_lim;
      const float4 q0 = ok0 ? sweep_ld<COH>(reinterpret_cast<const float4*>(dual_p) + t0) : make_float4(0, 0, 0, 0);
      const float4 q1 = ok1 ? sweep_ld<COH>(reinterpret_cast<const float4*>(dual_p) + t1) : make_float4(0, 0, 0, 0);
      float2 r0 = make_float2(0.0f, 0.0f), r1 = make_float2(0.0f, 0.0f);
      if (smooth_normals) {
        if (ok0) r0 = sweep_ld<COH>(reinterpret_cast<const float2*>(dual_n) + t0);
        if (ok1) r1 = sweep_ld<COH>(reinterpret_cast<const float2*>(dual_n) + t1);
      }
      if (ok0) {
        p[0] = p[0] + q0.x; p[1] = p[1] + q0.y; p[2] = p[2] + q0.z;
        if (smooth_normals) { nn[0] = nn[0] + q0.w; nn[1] = nn[1] + r0.x; nn[2] = nn[2] + r0.y; }
      }
      if (ok1) {
        p[0] = p[0] + q1.x; p[1] = p[1] + q1.y; p[2] = p[2] + q1.z;
        if (smooth_normals) { nn[0] = nn[0] + q1.w; nn[1] = nn[1] + r1.x; nn[2] = nn[2] + r1.y; }
      }
    }
  }
  for (uint32_t k = k0; k < n; ++k) {
    const uint32_t t = sweep_ld<COH>(a + k);
    if ((I)t >= np_lim) continue;  // never read past the dual points
    if (PACKED) {
      const float4 q = sweep_ld<COH>(reinterpret_cast<const float4*>(dual_p) + t);
      p[0] = p[0] + q.x;
      p[1] = p[1] + q.y;
      p[2] = p[2] + q.z;
      if (smooth_normals) {
        const float2 r = sweep_ld<COH>(reinterpret_cast<const float2*>(dual_n) + t);
        nn[0] = nn[0] + q.w;
        nn[1] = nn[1] + r.x;
        nn[2] = nn[2] + r.y;
      }
    } else {
#pragma unroll
      for (int c = 0; c < 3; ++c) p[c] = p[c] + sweep_ld<COH>(dual_p + 3 * t + c);
      if (smooth_normals) {
#pragma unroll
        for (int c = 0; c < 3; ++c) nn[c] = nn[c] + sweep_ld<COH>(dual_n + 3 * t + c);
      }
    }
  }
  const float cnt = (float)n;
#pragma unroll
  for (int c = 0; c < 3; ++c) p[c] = p[c] / cnt;
  if (smooth_normals) {
#pragma unroll
    for (int c = 0; c < 3; ++c) nn[c] = nn[c] / cnt;
  }
  if (set_colors) {
    float o[3];
    nrm3(nn, o);
    nn[0] = o[0]; nn[1] = o[1]; nn[2] = o[2];
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) pos[3 * v + c] = p[c];
  if (nrm && nn[1] != 0.0f) {
#pragma unroll
    for (int c = 0; c < 3; ++c) nrm[3 * v + c] = nn[c];
  }
}

}  // namespace bmf
