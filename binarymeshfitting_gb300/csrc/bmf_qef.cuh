// Hermite data, the reference's FP32 QEF and its adjoint, shared by the
// extraction TU and the FP64 adjoint TU (compiled with FMA contraction).
#pragma once

#include <type_traits>

#include "bmf_device.cuh"
#include "bmf_df.cuh"
#include "bmf_internal.h"

namespace bmf {

// Chunk of vertex v: the last chunk whose vertex offset is <= v (empty
// chunks share the next one's offset).
__device__ __forceinline__ int find_chunk_by_vertex(const ChunkDev* __restrict__ chunks, int n, int64_t v) {
  int lo = 0, hi = n - 1;  // last chunk whose vout <= v (empty chunks share the next one's offset)
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (chunks[mid].vout <= v) lo = mid; else hi = mid - 1;
  }
  return lo;
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

// info / qef_used (optional, QEF placement): the solve's eigen data and
// whether the vertex took the QEF branch (a successful solve inside the cell)
// -- what the QEF adjoint needs from the forward.
template <int PLACE>
__device__ __forceinline__ void q_place(const float* D, int dim, int x, int y, int z, int mask, int g, float out[3],
                                        QefSolveInfo* info = nullptr, bool* qef_used = nullptr) {
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
    const bool solved = q.solve(s, info);
    const bool ok = s[0] >= (float)x && s[0] <= (float)(x + 1) && s[1] >= (float)y && s[1] <= (float)(y + 1) &&
                    s[2] >= (float)z && s[2] <= (float)(z + 1);
    if (qef_used) *qef_used = solved && ok;
    if (ok) {
      out[0] = s[0]; out[1] = s[1]; out[2] = s[2];
      return;
    }
  }
  out[0] = mp[0]; out[1] = mp[1]; out[2] = mp[2];
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
  T s0, s1, mu, p[3], g0[3], g1[3], n[3], glen, iglen;
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
  h.iglen = (T)1;
  if (want_n) {
    grid_gradient_t<T>(D, dim, h.a0[0], h.a0[1], h.a0[2], h.g0);
    grid_gradient_t<T>(D, dim, h.a1[0], h.a1[1], h.a1[2], h.g1);
    T G[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) G[k] = h.g0[k] + (h.g1[k] - h.g0[k]) * h.mu;
    h.glen = sqrt((G[0] * G[0] + G[1] * G[1]) + G[2] * G[2]);
    h.iglen = (T)1 / h.glen;
#pragma unroll
    for (int k = 0; k < 3; ++k) h.n[k] = G[k] * h.iglen;
  }
}

// Symmetric 3x3 eigen decomposition in a wide type R (FP64 or double-float),
// A = V diag(w) V^T, refined from the forward's FP32 eigenvectors: V0 is
// re-orthonormalised (Gram-Schmidt), A is rotated into that basis (nearly
// diagonal, off-diagonals ~1e-6 |A|) and cyclic Jacobi rotations finish it;
// convergence is quadratic, so one or two sweeps reach the stopping point
// (1e-17 |A| in FP64, 3e-14 |A| in double-float) instead of five or six from
// the identity.
// Stopping point of the refinement: 1e-17 |A| in FP64, 3e-14 |A| in
// double-float (about its resolution).
template <typename R>
struct EigTol {
  static constexpr double scale = 1e-17;
};
template <>
struct EigTol<DF> {
  static constexpr double scale = 3e-14;
};
template <typename R>
__device__ void eig3_refine(const R A[3][3], const float V0[3][3], R w[3], R V[3][3]) {
  // columns of V0, orthonormalised
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    R v[3] = {R(V0[0][c]), R(V0[1][c]), R(V0[2][c])};
#pragma unroll
    for (int k = 0; k < c; ++k) {
      const R d = v[0] * V[0][k] + v[1] * V[1][k] + v[2] * V[2][k];
#pragma unroll
      for (int r = 0; r < 3; ++r) v[r] -= d * V[r][k];
    }
    const R il = R(1.0f) / sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
#pragma unroll
    for (int r = 0; r < 3; ++r) V[r][c] = v[r] * il;
  }
  // B = V^T A V
  R AV[3][3], B[3][3];
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
    for (int c = 0; c < r; ++c) B[r][c] = B[c][r] = R(0.5f) * (B[r][c] + B[c][r]);
  }
  const R tol = R(EigTol<R>::scale) * (fabs(B[0][0]) + fabs(B[1][1]) + fabs(B[2][2]));
#pragma unroll 1
  for (int sweep = 0; sweep < 16; ++sweep) {
    if (fabs(B[0][1]) + fabs(B[0][2]) + fabs(B[1][2]) <= tol) break;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const int p = q == 2 ? 1 : 0, r = q == 0 ? 1 : 2;
      if (fabs(B[p][r]) <= tol) continue;
      const R tau = (B[r][r] - B[p][p]) / (R(2.0f) * B[p][r]);
      const R t = (tau >= R(0.0f) ? R(1.0f) : R(-1.0f)) / (fabs(tau) + sqrt(R(1.0f) + tau * tau));
      const R c = R(1.0f) / sqrt(R(1.0f) + t * t), s = t * c;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const R bkp = B[k][p], bkr = B[k][r];
        B[k][p] = c * bkp - s * bkr;
        B[k][r] = s * bkp + c * bkr;
      }
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const R bpk = B[p][k], brk = B[r][k];
        B[p][k] = c * bpk - s * brk;
        B[r][k] = s * bpk + c * brk;
      }
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const R vkp = V[k][p], vkr = V[k][r];
        V[k][p] = c * vkp - s * vkr;
        V[k][r] = s * vkp + c * vkr;
      }
    }
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) w[i] = B[i][i];
}

// The edges of cell-mask group g as a 12-bit set.  The adjoint loops walk
// it in ascending edge order (the order of the forward's accumulation): each
// lane runs only its own vertex's edges, not the union of the warp's.
__device__ __forceinline__ uint32_t group_edges(int mask, int g) {
  uint32_t m = 0u;
#pragma unroll
  for (int e = 0; e < 12; ++e) m |= (group_of(mask, e) == g ? 1u : 0u) << e;
  return m;
}

// LIST = 0: every vertex; 1: every vertex, but QEF-placed ones are only
// appended to qlist (for a dense second pass); 2: the vertices of qlist;
// 3: the vertices the forward did not flag in qflag (mass-point placed; the
// forward built qlist / qseed).
// CTAs per SM the double-float pass asks for: its code is larger than the
// instruction cache, and more resident warps hide the fetch misses better
// than the registers saved by spilling cost (measured: 3.71 ms backward at 4
// CTAs, 3.46 at 8, the same at 10 and 12).
template <typename T>
__host__ __device__ constexpr int place_bwd_min_ctas() { return std::is_same<T, DF>::value ? 8 : 1; }

template <int PLACE, typename T, int LIST>
__global__ void __launch_bounds__(128, place_bwd_min_ctas<T>()) k_place_bwd(const ChunkDev* __restrict__ chunks, int n_chunks,
                                                   const uint32_t* __restrict__ words, const float* __restrict__ dens,
                                                   const uint32_t* __restrict__ vkey,
                                                   const int64_t* __restrict__ d_counts, int64_t vcap,
                                                   const float* __restrict__ grad_pos, float* __restrict__ grad_dens,
                                                   uint32_t* __restrict__ qlist, uint32_t* __restrict__ qcount,
                                                   float* __restrict__ qseed, const uint8_t* __restrict__ qflag) {
  int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t slot = v;  // LIST == 2: the list entry
  if (LIST == 2) {
    if (v >= (int64_t)*qcount) return;
    v = qlist[v];
  }
  if (v >= (d_counts ? min(vcap, d_counts[0]) : vcap)) return;
  if (LIST == 3 && qflag[v]) return;  // QEF-placed: the list pass
  const int c = find_chunk_by_vertex(chunks, n_chunks, v);
  const ChunkDev ch = chunks[c];
  const int dim = ch.dim, zc = ch.zc;
  const uint32_t* W = words + ch.words;
  const float* D = dens + ch.dens;
  float* GD = grad_dens + ch.dens;
  int x, y, z, g;
  vertex_key_decode(vkey[v], x, y, z, g);
  const int mask = cell_mask_at(W, dim, zc, x, y, z);
  const uint32_t edges = group_edges(mask, g);
  const T gx[3] = {(T)grad_pos[3 * v], (T)grad_pos[3 * v + 1], (T)grad_pos[3 * v + 2]};
  int cnt = 0;
  bool use_qef = false;
  QefAdj<T> Q;
  QefAccum q;
  QefSolveInfo info;
  if constexpr (LIST == 2) {
    // a listed vertex is QEF-placed (the first pass's exact FP32 replay
    // decided it) and its FP32 eigenvectors, which seed the wide re-solve, were
    // kept by that pass
    cnt = __popc(edges);
    if (cnt == 0) return;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
#pragma unroll
      for (int k = 0; k < 3; ++k) info.V[r][k] = qseed[9 * slot + 3 * r + k];
    }
    use_qef = true;
  } else if constexpr (LIST == 3) {
    // the forward recorded the branch: a vertex left to this pass took the mass point
    cnt = __popc(edges);
    if (cnt == 0) return;
  } else {
    // the forward's branch: replay of q_place in FP32
    if (PLACE == 2) q.init();
    for (uint32_t em = edges; em; em &= em - 1u) {
      const int e = __ffs(em) - 1;
      float p[3], n[3];
      hermite(D, dim, x, y, z, e, PLACE == 2, p, n);
      ++cnt;
      if (PLACE == 2) q.add(p, n);
    }
    if (cnt == 0) return;
    if (PLACE == 2) {
      float s[3];
      if (q.solve(s, &info))
        use_qef = s[0] >= (float)x && s[0] <= (float)(x + 1) && s[1] >= (float)y && s[1] <= (float)(y + 1) &&
                  s[2] >= (float)z && s[2] <= (float)(z + 1);
      if (LIST == 1 && use_qef) {
        const uint32_t k = atomicAdd(qcount, 1u);
        qlist[k] = (uint32_t)v;
#pragma unroll
        for (int r = 0; r < 3; ++r) {
#pragma unroll
          for (int c3 = 0; c3 < 3; ++c3) qseed[9 * (int64_t)k + 3 * r + c3] = info.V[r][c3];
        }
        return;
      }
    }
  }
  if (PLACE == 2) {
    if (use_qef) {
      if constexpr (sizeof(T) == sizeof(float)) {
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
        // the same QEF in the wide type (FP64 or double-float): ATA, ATb, mass
        // point, converged eigen pairs
        T A[3][3] = {{T(0.0f), T(0.0f), T(0.0f)}, {T(0.0f), T(0.0f), T(0.0f)}, {T(0.0f), T(0.0f), T(0.0f)}};
        T b[3] = {T(0.0f), T(0.0f), T(0.0f)}, m[3] = {T(0.0f), T(0.0f), T(0.0f)};
        for (uint32_t em = edges; em; em &= em - 1u) {
          const int e = __ffs(em) - 1;
          HermiteT<T> h;
          hermite_t<T>(D, dim, x, y, z, e, true, h);
          const T d = h.n[0] * h.p[0] + h.n[1] * h.p[1] + h.n[2] * h.p[2];
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
          m[r] /= T(cnt);
#pragma unroll
          for (int k = 0; k < 3; ++k) Q.A[r][k] = A[r][k];
        }
#pragma unroll
        for (int r = 0; r < 3; ++r) {
          Q.mp[r] = m[r];
          Q.r[r] = b[r] - (A[r][0] * m[0] + A[r][1] * m[1] + A[r][2] * m[2]);
        }
        T w[3], V[3][3];
        eig3_refine<T>(A, info.V, w, V);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          const T oo = T(1.0f) / w[i];
          const T mn = fabs(w[i]) < fabs(oo) ? fabs(w[i]) : fabs(oo);
          Q.sigma[i] = w[i];
          Q.inv[i] = mn >= T(0.001f) ? oo : T(0.0f);
#pragma unroll
          for (int k = 0; k < 3; ++k) Q.V[k][i] = V[k][i];
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
    T Gs[3][3], M[3][3], F[3][3], W[3][3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
#pragma unroll
      for (int k = 0; k < 3; ++k) Gs[r][k] = (T)0.5 * (gx[r] * Q.r[k] + gx[k] * Q.r[r]);
    }
    // M = V^T Gs V as two 3x3 products (W = Gs V, then V^T W)
#pragma unroll
    for (int r = 0; r < 3; ++r) {
#pragma unroll
      for (int b = 0; b < 3; ++b) W[r][b] = Gs[r][0] * Q.V[0][b] + Gs[r][1] * Q.V[1][b] + Gs[r][2] * Q.V[2][b];
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        M[a][b] = Q.V[0][a] * W[0][b] + Q.V[1][a] * W[1][b] + Q.V[2][a] * W[2][b];
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
        F[a][b] = F[a][b] * M[a][b];
      }
    }
    // gA = V (F o M) V^T - sym(gr mp^T), again as two products
#pragma unroll
    for (int r = 0; r < 3; ++r) {
#pragma unroll
      for (int b = 0; b < 3; ++b) W[r][b] = Q.V[r][0] * F[0][b] + Q.V[r][1] * F[1][b] + Q.V[r][2] * F[2][b];
    }
#pragma unroll
    for (int r = 0; r < 3; ++r) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const T s = W[r][0] * Q.V[k][0] + W[r][1] * Q.V[k][1] + W[r][2] * Q.V[k][2];
        gA[r][k] = s - (T)0.5 * (gr[r] * Q.mp[k] + gr[k] * Q.mp[r]);
      }
    }
#pragma unroll
    for (int r = 0; r < 3; ++r) gm[r] -= Q.A[r][0] * gr[0] + Q.A[r][1] * gr[1] + Q.A[r][2] * gr[2];
  }
  // The chain rule into the density runs in FP32 on the forward's own hermite
  // data, whatever T is: the ill-conditioned part -- the eigen pairs of A, the
  // residual r and gm = gx - A gr -- is done in T; what remains is a product of
  // well-conditioned factors.
  float fA[3][3], fr[3], fm[3], fx[3];
#pragma unroll
  for (int r = 0; r < 3; ++r) {
#pragma unroll
    for (int k = 0; k < 3; ++k) fA[r][k] = (float)gA[r][k];
    fr[r] = (float)gr[r];
    fm[r] = (float)gm[r];
    fx[r] = (float)gx[r];
  }
  const float inv_cnt = 1.0f / (float)cnt;
  // per hermite pair: g_p, g_n, then into the density
  for (uint32_t em = edges; em; em &= em - 1u) {
    const int e = __ffs(em) - 1;
    HermiteT<float> h;
    hermite_t<float>(D, dim, x, y, z, e, PLACE == 2 && use_qef, h);  // the mass point needs no normals
    const int ax = e >> 2;
    float gp[3], gn[3] = {0.0f, 0.0f, 0.0f};
    if (!use_qef) {
#pragma unroll
      for (int k = 0; k < 3; ++k) gp[k] = fx[k] * inv_cnt;
    } else {
      const float d = h.n[0] * h.p[0] + h.n[1] * h.p[1] + h.n[2] * h.p[2];
      const float gd = fr[0] * h.n[0] + fr[1] * h.n[1] + fr[2] * h.n[2];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        gn[k] = 2.0f * (fA[k][0] * h.n[0] + fA[k][1] * h.n[1] + fA[k][2] * h.n[2]) + d * fr[k] + gd * h.p[k];
        gp[k] = gd * h.n[k] + fm[k] * inv_cnt;
      }
    }
    float gmu = gp[ax];
    if (use_qef) {
      const float nd = h.n[0] * gn[0] + h.n[1] * gn[1] + h.n[2] * gn[2];
      float gG[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        gG[k] = (gn[k] - h.n[k] * nd) * h.iglen;
        gmu += gG[k] * (h.g1[k] - h.g0[k]);
      }
      // central differences at both endpoints: g[a] = (s[hi] - s[lo]) * h
#pragma unroll
      for (int a = 0; a < 3; ++a) {
#pragma unroll
        for (int end = 0; end < 2; ++end) {
          const int* q0 = end ? h.a1 : h.a0;
          const float w = gG[a] * (end ? h.mu : 1.0f - h.mu);
          int lo[3] = {q0[0], q0[1], q0[2]}, hi[3] = {q0[0], q0[1], q0[2]};
          float hh = 0.5f;
          if (q0[a] > 0) lo[a]--; else hh = 1.0f;
          if (q0[a] < dim - 1) hi[a]++; else hh = 1.0f;
          atomicAdd(GD + ((int64_t)hi[0] * dim + hi[1]) * dim + hi[2], w * hh);
          atomicAdd(GD + ((int64_t)lo[0] * dim + lo[1]) * dim + lo[2], -w * hh);
        }
      }
    }
    const float iden = 1.0f / ((h.s1 - h.s0) * (h.s1 - h.s0));
    atomicAdd(GD + ((int64_t)h.a0[0] * dim + h.a0[1]) * dim + h.a0[2], gmu * (-h.s1 * iden));
    atomicAdd(GD + ((int64_t)h.a1[0] * dim + h.a1[1]) * dim + h.a1[2], gmu * (h.s0 * iden));
  }
}

}  // namespace bmf
