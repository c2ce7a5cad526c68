// Stage 5: MeshProcessor<N> dual / primal smoothing and normals
// (MeshProcessor.cpp:26-306), in the order ChunkGenerator::extract_chunk runs
// it (ChunkGenerator.cpp:112-124): iters dual steps, a primal step after each
// but the last inside optimize_dual_grid, then one more primal step.
//
// The reference's sweeps are Jacobi-style (a dual step reads only vertex
// positions, a primal step reads only dual points), so every primitive and
// every vertex is independent: one thread each.  The one order that matters
// for bit-exact sums is the adjacency order: init_primitives appends prims to
// each vertex in ascending prim id (MeshProcessor.cpp:114-127).  The CSR
// fill uses atomic cursors and then sorts each (short) list.
#include "bmf_device.cuh"
#include "bmf_internal.h"
#include "bmf_sweep.cuh"

namespace bmf {

constexpr int kScanBlock = 1024;
constexpr int kScanPer = 4;

// Block-level exclusive scan of u8 counts -> u32 offsets; writes block totals.
__global__ void __launch_bounds__(kScanBlock) k_scan_u8_local(const uint8_t* __restrict__ in, uint32_t* __restrict__ out,
                                                             int64_t n, const int64_t* __restrict__ d_n,
                                                             uint32_t* __restrict__ block_tot) {
  __shared__ uint32_t warp_tot[kScanBlock / 32];
  const int64_t n_valid = d_n ? min(n, *d_n) : n;
  const int64_t i0 = ((int64_t)blockIdx.x * kScanBlock + threadIdx.x) * kScanPer;
  uint32_t v[kScanPer], s = 0;
#pragma unroll
  for (int k = 0; k < kScanPer; ++k) {
    v[k] = (i0 + k < n_valid) ? in[i0 + k] : 0u;
    s += v[k];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t inc = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(kFull, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) warp_tot[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = warp_tot[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(kFull, w, o);
      if (lane >= o) w += t;
    }
    warp_tot[lane] = w;
  }
  __syncthreads();
  uint32_t e = (warp ? warp_tot[warp - 1] : 0u) + inc - s;
#pragma unroll
  for (int k = 0; k < kScanPer; ++k) {
    if (i0 + k < n) out[i0 + k] = e;
    e += v[k];
  }
  if (threadIdx.x == kScanBlock - 1) block_tot[blockIdx.x] = warp_tot[31];
}

// Scans the block totals in place (single CTA) and stores the grand total at [nb].
__global__ void __launch_bounds__(1024) k_scan_totals(uint32_t* __restrict__ t, int nb) {
  __shared__ uint32_t s[1024];
  uint32_t carry = 0;
  for (int base = 0; base < nb; base += 1024) {
    const int i = base + threadIdx.x;
    const uint32_t v = i < nb ? t[i] : 0u;
    s[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
      const uint32_t a = threadIdx.x >= o ? s[threadIdx.x - o] : 0u;
      __syncthreads();
      s[threadIdx.x] += a;
      __syncthreads();
    }
    if (i < nb) t[i] = carry + s[threadIdx.x] - v;
    carry += s[1023];
    __syncthreads();
  }
  if (threadIdx.x == 0) t[nb] = carry;
}

__global__ void k_scan_add(uint32_t* __restrict__ out, int64_t n, const uint32_t* __restrict__ block_off) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += block_off[i / ((int64_t)kScanBlock * kScanPer)];
}

void launch_exclusive_scan_u8_to_u32(const uint8_t* in, uint32_t* out, int64_t n, const int64_t* d_n,
                                     uint32_t* block_tmp, cudaStream_t st) {
  const int64_t per = (int64_t)kScanBlock * kScanPer;
  const int nb = (int)((n + per - 1) / per);
  if (nb == 0) return;
  k_scan_u8_local<<<nb, kScanBlock, 0, st>>>(in, out, n, d_n, block_tmp);
  k_scan_totals<<<1, 1024, 0, st>>>(block_tmp, nb);
  k_scan_add<<<(int)((n + 255) / 256), 256, 0, st>>>(out, n, block_tmp);
  // off[n] = total
  cudaMemcpyAsync(out + n, block_tmp + nb, sizeof(uint32_t), cudaMemcpyDeviceToDevice, st);
}

// set_adj (MeshRecursion.hpp:173-190): adj[off[v] + k] = prim.
__global__ void k_fill_adj(int N, int64_t n_slots, int64_t nv, const int64_t* __restrict__ d_counts,
                           const uint32_t* __restrict__ idx, const uint32_t* __restrict__ off,
                           const uint8_t* __restrict__ valence, uint32_t* __restrict__ cursor,
                           uint32_t* __restrict__ adj) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= (d_counts ? min(n_slots, d_counts[1] / N * N) : n_slots)) return;
  const uint32_t v = idx[j];
  if ((int64_t)v >= (d_counts ? min(nv, d_counts[0]) : nv)) return;  // an index outside the mesh is ignored
  const uint32_t k = atomicAdd(cursor + v, 1u);
  // a caller's valence may not sum to more than the index slots: stay inside adj
  if (k < valence[v] && (int64_t)off[v] + k < n_slots) adj[off[v] + k] = (uint32_t)(j / N);
}

// Restores ascending prim order in each vertex's list (insertion sort; the
// lists hold at most a few dozen entries).
__global__ void k_sort_adj(int64_t nv, int64_t adj_cap, const int64_t* __restrict__ d_counts,
                           const uint32_t* __restrict__ off, const uint32_t* __restrict__ cursor,
                           const uint8_t* __restrict__ valence, uint32_t* __restrict__ adj) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= (d_counts ? min(nv, d_counts[0]) : nv)) return;
  const int64_t room = adj_cap - (int64_t)off[v];
  const uint32_t n = (uint32_t)max((int64_t)0, min((int64_t)min(cursor[v], (uint32_t)valence[v]), room));
  uint32_t* a = adj + off[v];
  for (uint32_t i = 1; i < n; ++i) {
    const uint32_t key = a[i];
    int j = (int)i - 1;
    while (j >= 0 && a[j] > key) {
      a[j + 1] = a[j];
      --j;
    }
    a[j + 1] = key;
  }
}

template <int N>
__global__ void k_dual(int64_t n_prims, int64_t nv, const int64_t* __restrict__ d_counts,
                       const uint32_t* __restrict__ idx, const float* __restrict__ pos, const float* __restrict__ nrm,
                       float* __restrict__ dual_p, float* __restrict__ dual_n, int normal_mode) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (d_counts ? min(n_prims, d_counts[1] / N) : n_prims)) return;
  dual_prim<N>(t, d_counts ? min(nv, d_counts[0]) : nv, idx, pos, nrm, dual_p, dual_n, normal_mode);
}

// optimize_primal_grid (MeshProcessor.cpp:238-306).
__global__ void k_primal(int64_t nv, int64_t np_lim, int64_t adj_cap, const int64_t* __restrict__ d_counts,
                         const uint32_t* __restrict__ off, const uint32_t* __restrict__ cursor,
                         const uint8_t* __restrict__ valence, const uint32_t* __restrict__ adj,
                         const uint8_t* __restrict__ boundary, const float* __restrict__ dual_p,
                         const float* __restrict__ dual_n, float* __restrict__ pos, float* __restrict__ nrm,
                         int process_boundary, int smooth_normals, int set_colors) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= (d_counts ? min(nv, d_counts[0]) : nv)) return;
  primal_vertex(v, np_lim, adj_cap, off, cursor, valence, adj, boundary, dual_p, dual_n, pos, nrm, process_boundary,
                smooth_normals, set_colors);
}

// ---------------------------------------------------------------------------
// Draw layout (GLChunk::format_data, GLChunk.cpp:278-335): per-vertex p/n/c,
// or quads unwound to 4 vertices sharing one normal.  Colours are white: the
// vertex colour is (1, 1, 1) at creation (DMCChunk.cpp:681) and the sweeps
// only average it.  Counts come from d_counts (vertices, indices) when given.
// ---------------------------------------------------------------------------
__global__ void k_format_verts(int64_t nv, const int64_t* __restrict__ d_counts, int64_t cap,
                               const float* __restrict__ pos, const float* __restrict__ nrm, float* __restrict__ p,
                               float* __restrict__ n, float* __restrict__ c) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= min(cap, d_counts ? min(nv, d_counts[0]) : nv)) return;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    p[3 * v + k] = __ldg(pos + 3 * v + k);
    n[3 * v + k] = nrm ? __ldg(nrm + 3 * v + k) : 0.0f;
    c[3 * v + k] = 1.0f;
  }
}

// chunks (nullable): quad slots are arena positions and indices chunk-local;
// a quad's chunk is the last one whose index offset is <= its first slot.
__global__ void k_format_quads(const ChunkDev* __restrict__ chunks, int n_chunks, int64_t ni,
                               const int64_t* __restrict__ d_counts, int64_t cap, const float* __restrict__ pos,
                               const float* __restrict__ nrm, const uint32_t* __restrict__ idx, int smooth,
                               float* __restrict__ p, float* __restrict__ n, float* __restrict__ c) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nidx = d_counts ? min(ni, d_counts[1]) : ni;
  const int64_t i = 4 * q;
  if (i + 3 >= nidx || i + 3 >= cap) return;
  int64_t vo = 0, nvb = d_counts ? d_counts[0] : INT64_MAX;
  if (chunks) {
    int lo = 0, hi = n_chunks - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (chunks[mid].iout <= i) lo = mid; else hi = mid - 1;
    }
    vo = chunks[lo].vout;
  }
  int64_t v[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    v[k] = vo + (int64_t)__ldg(idx + i + k);
    if (v[k] >= nvb) v[k] = 0;  // an index outside the mesh reads vertex 0 instead of faulting
  }
  float P[4][3];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
#pragma unroll
    for (int d = 0; d < 3; ++d) P[k][d] = __ldg(pos + 3 * v[k] + d);
  }
  float m[3];
  if (smooth) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      float s = __ldg(nrm + 3 * v[0] + d) + __ldg(nrm + 3 * v[1] + d);
      s = s + __ldg(nrm + 3 * v[2] + d);
      s = s + __ldg(nrm + 3 * v[3] + d);
      m[d] = s * 0.25f;
    }
  } else {
    float a[3], b[3], na[3], nb[3], m0[3], m1[3], h[3], o[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      a[d] = P[0][d] - P[1][d];
      b[d] = P[0][d] - P[2][d];
    }
    nrm3(a, na);
    nrm3(b, nb);
    cross3(na, nb, m0);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      a[d] = P[2][d] - P[3][d];
      b[d] = P[2][d] - P[0][d];
    }
    nrm3(a, na);
    nrm3(b, nb);
    cross3(na, nb, m1);
    if (isnan(m0[0])) { m0[0] = m1[0]; m0[1] = m1[1]; m0[2] = m1[2]; }
    if (isnan(m1[0])) { m1[0] = m0[0]; m1[1] = m0[1]; m1[2] = m0[2]; }
#pragma unroll
    for (int d = 0; d < 3; ++d) h[d] = (m0[d] + m1[d]) * 0.5f;
    nrm3(h, o);
#pragma unroll
    for (int d = 0; d < 3; ++d) m[d] = -o[d];
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      p[3 * (i + k) + d] = P[k][d];
      n[3 * (i + k) + d] = m[d];
      c[3 * (i + k) + d] = 1.0f;
    }
  }
}

int launch_format(const ChunkDev* d_chunks, int n_chunks, int64_t nv, int64_t ni, const int64_t* d_counts,
                  const float* pos, const float* nrm, const uint32_t* idx, int unwind, int smooth, float* p, float* n,
                  float* c, int64_t cap, cudaStream_t st) {
  if (!unwind) {
    if (nv <= 0) return 0;
    k_format_verts<<<(int)((nv + 255) / 256), 256, 0, st>>>(nv, d_counts, cap, pos, nrm, p, n, c);
  } else {
    const int64_t nq = ni / 4;
    if (nq <= 0) return 0;
    k_format_quads<<<(int)((nq + 255) / 256), 256, 0, st>>>(d_chunks, n_chunks, ni, d_counts, cap, pos, nrm, idx,
                                                            smooth, p, n, c);
  }
  return 1;
}

// ---------------------------------------------------------------------------
// Adjoint of the position sweeps.  A dual step averages each primitive's N
// vertices; a primal step replaces every updated vertex (adjacency non-empty,
// not a frozen boundary vertex) by the mean of its primitives' dual points and
// leaves the others unchanged.  Both are linear in the positions and do not
// depend on them, so the backward needs no stored iterates: it applies the
// transposes, last sweep first.  Both transposes are gathers (per primitive /
// per vertex through the CSR), so they need no atomics.
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool primal_updates(const uint8_t* valence, const uint8_t* boundary, int64_t v,
                                               int process_boundary) {
  return valence[v] != 0 && (process_boundary || !boundary[v]);
}

// g_dual[t] = sum over the primitive's slots of g[v] / count(v), updated v only.
template <int N>
__global__ void k_primal_bwd(int64_t n_prims, int64_t nv, const int64_t* __restrict__ d_counts,
                             const uint32_t* __restrict__ idx, const uint8_t* __restrict__ valence,
                             const uint8_t* __restrict__ boundary, int process_boundary, const float* __restrict__ g,
                             float* __restrict__ g_dual) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (d_counts ? min(n_prims, d_counts[1] / N) : n_prims)) return;
  const int64_t nvb = d_counts ? min(nv, d_counts[0]) : nv;
  float s[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
  for (int k = 0; k < N; ++k) {
    const uint32_t v = __ldg(idx + N * t + k);
    if ((int64_t)v >= nvb || !primal_updates(valence, boundary, v, process_boundary)) continue;
    const float inv = 1.0f / (float)valence[v];
#pragma unroll
    for (int c = 0; c < 3; ++c) s[c] += __ldg(g + 3 * v + c) * inv;
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) g_dual[3 * t + c] = s[c];
}

// g[v] <- (updated(v) ? 0 : g[v]) + sum over t in adj(v) of g_dual[t] / N (in place).
__global__ void k_dual_bwd(int N, int64_t nv, int64_t n_prims, int64_t adj_cap, const int64_t* __restrict__ d_counts,
                           const uint32_t* __restrict__ off, const uint8_t* __restrict__ valence,
                           const uint32_t* __restrict__ adj, const uint8_t* __restrict__ boundary, int process_boundary,
                           const float* __restrict__ g_dual, float* __restrict__ g) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= (d_counts ? min(nv, d_counts[0]) : nv)) return;
  const int64_t room = adj_cap - (int64_t)off[v];
  const uint32_t n = (uint32_t)max((int64_t)0, min((int64_t)valence[v], room));
  float s[3] = {0.0f, 0.0f, 0.0f};
  if (!primal_updates(valence, boundary, v, process_boundary)) {
#pragma unroll
    for (int c = 0; c < 3; ++c) s[c] = g[3 * v + c];
  }
  const float invN = 1.0f / (float)N;
  for (uint32_t k = 0; k < n; ++k) {
    const uint32_t t = __ldg(adj + off[v] + k);
    if ((int64_t)t >= n_prims) continue;
#pragma unroll
    for (int c = 0; c < 3; ++c) s[c] += __ldg(g_dual + 3 * t + c) * invN;
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) g[3 * v + c] = s[c];
}

// Both transposes chunk by chunk: one CTA per chunk (from the queue) runs
// every backward step of its chunk with block barriers in between -- a
// chunk's primitives only read its own vertices and the reverse.  Per item the
// operations are those of k_primal_bwd / k_dual_bwd, so the results are the
// same; g and g_dual, which the kernel itself writes, are read with coherent
// L1 loads.
constexpr int kBwdChunkThreads = 512;

template <int N>
__global__ void __launch_bounds__(kBwdChunkThreads, 4) k_sweep_bwd_chunks(
    const ChunkDev* __restrict__ chunks, const uint32_t* __restrict__ tot, const int* __restrict__ order,
    int n_chunks, int* __restrict__ queue, int64_t nv, int64_t n_prims, int64_t adj_cap,
    const int64_t* __restrict__ d_counts, const uint32_t* __restrict__ off, const uint8_t* __restrict__ valence,
    const uint32_t* __restrict__ adj, const uint8_t* __restrict__ boundary, int process_boundary,
    const uint32_t* __restrict__ idx, float* __restrict__ g, float* __restrict__ g_dual, int iters) {
  __shared__ int s_item;
  const int64_t nvb = d_counts ? min(nv, d_counts[0]) : nv;
  const int64_t npb = d_counts ? min(n_prims, d_counts[1] / N) : n_prims;
  const float invN = 1.0f / (float)N;
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(queue, 1);
    __syncthreads();
    const int it = s_item;
    __syncthreads();  // everyone has read s_item before thread 0 takes the next
    if (it >= n_chunks) break;
    const int c = order[it];
    const int64_t v0 = chunks[c].vout, v1 = min(v0 + (int64_t)tot[2 * c], nvb);
    const int64_t p0 = chunks[c].iout / N, p1 = min((chunks[c].iout + (int64_t)tot[2 * c + 1]) / N, npb);
    for (int m = iters - 1; m >= 0; --m) {
      for (int64_t t = p0 + threadIdx.x; t < p1; t += kBwdChunkThreads) {
        float sd[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int k = 0; k < N; ++k) {
          const uint32_t v = __ldg(idx + N * t + k);
          if ((int64_t)v >= nvb || !primal_updates(valence, boundary, v, process_boundary)) continue;
          const float inv = 1.0f / (float)valence[v];
#pragma unroll
          for (int cc = 0; cc < 3; ++cc) sd[cc] += __ldca(g + 3 * v + cc) * inv;
        }
#pragma unroll
        for (int cc = 0; cc < 3; ++cc) g_dual[3 * t + cc] = sd[cc];
      }
      __syncthreads();
      for (int64_t v = v0 + threadIdx.x; v < v1; v += kBwdChunkThreads) {
        const int64_t room = adj_cap - (int64_t)off[v];
        const uint32_t n = (uint32_t)max((int64_t)0, min((int64_t)valence[v], room));
        float sv[3] = {0.0f, 0.0f, 0.0f};
        if (!primal_updates(valence, boundary, v, process_boundary)) {
#pragma unroll
          for (int cc = 0; cc < 3; ++cc) sv[cc] = g[3 * v + cc];
        }
        for (uint32_t k = 0; k < n; ++k) {
          const uint32_t t = __ldg(adj + off[v] + k);
          if ((int64_t)t >= n_prims) continue;
#pragma unroll
          for (int cc = 0; cc < 3; ++cc) sv[cc] += __ldca(g_dual + 3 * t + cc) * invN;
        }
#pragma unroll
        for (int cc = 0; cc < 3; ++cc) g[3 * v + cc] = sv[cc];
      }
      __syncthreads();
    }
  }
}

int launch_process_bwd(int N, int64_t nv, int64_t n_prims, const int64_t* d_counts, const uint8_t* boundary,
                       const uint8_t* valence, const uint32_t* idx, int iters, int process_boundary,
                       const ProcessScratch& s, float* g, const StructuredAdj* sa, cudaStream_t st) {
  if (nv == 0 || n_prims == 0 || iters <= 0) return 0;
  if (sa && sa->tot && sa->order && sa->queue) {
    // one slot array per primitive size: the two kernels' occupancies may differ
    static std::atomic<int> grid3[64] = {}, grid4[64] = {};
    const int grid = per_device_once(N == 3 ? grid3 : grid4, [N](int dev) {
      int sms = 0, per_sm = 0;
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      if (N == 3)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sweep_bwd_chunks<3>, kBwdChunkThreads, 0);
      else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sweep_bwd_chunks<4>, kBwdChunkThreads, 0);
      return (sms > 0 ? sms : 1) * (per_sm > 0 ? per_sm : 1);
    });
    cudaMemsetAsync(sa->queue, 0, sizeof(int), st);
    if (N == 3)
      k_sweep_bwd_chunks<3><<<grid, kBwdChunkThreads, 0, st>>>(
          sa->chunks, sa->tot, sa->order, sa->n_chunks, sa->queue, nv, n_prims, n_prims * N, d_counts, s.off,
          valence, s.adj, boundary, process_boundary, idx, g, s.dual_p, iters);
    else
      k_sweep_bwd_chunks<4><<<grid, kBwdChunkThreads, 0, st>>>(
          sa->chunks, sa->tot, sa->order, sa->n_chunks, sa->queue, nv, n_prims, n_prims * N, d_counts, s.off,
          valence, s.adj, boundary, process_boundary, idx, g, s.dual_p, iters);
    return 1;
  }
  const int vb = (int)((nv + 255) / 256), pb = (int)((n_prims + 255) / 256);
  for (int m = iters - 1; m >= 0; --m) {
    if (N == 3)
      k_primal_bwd<3><<<pb, 256, 0, st>>>(n_prims, nv, d_counts, idx, valence, boundary, process_boundary, g, s.dual_p);
    else
      k_primal_bwd<4><<<pb, 256, 0, st>>>(n_prims, nv, d_counts, idx, valence, boundary, process_boundary, g, s.dual_p);
    k_dual_bwd<<<vb, 256, 0, st>>>(N, nv, n_prims, n_prims * N, d_counts, s.off, valence, s.adj, boundary,
                                   process_boundary, s.dual_p, g);
  }
  return 2 * iters;
}

int launch_process(int N, int64_t nv, int64_t n_prims, const int64_t* d_counts, float* pos, float* nrm,
                   const uint8_t* boundary, const uint8_t* valence, const uint32_t* idx, int iters,
                   int process_boundary, int smooth_normals, ProcessScratch s, const StructuredAdj* sa,
                   cudaStream_t st) {
  if (nv == 0 || n_prims == 0 || iters <= 0) return 0;
  const int64_t n_slots = n_prims * N;
  const bool sn = smooth_normals != 0 && nrm != nullptr;
  if (sa && sa->tot && sa->order && sa->queue) {
    launch_sweep_chunks(*sa, N, nv, n_prims, d_counts, pos, nrm, boundary, valence, idx, iters, process_boundary,
                        sn ? 1 : 0, s, st);
    return 1;
  }
  int launched = 3;
  // CSR offsets: exclusive scan of init_valence (MeshProcessor.cpp:32-40)
  launch_exclusive_scan_u8_to_u32(valence, s.off, nv, d_counts, s.tmp, st);
  const int tb = s.block > 0 ? s.block : 256;
  const int vb = (int)((nv + 255) / 256);
  const int vbt = (int)((nv + tb - 1) / tb), pbt = (int)((n_prims + tb - 1) / tb);
  const uint32_t* cursor = nullptr;
  if (sa) {
    launch_adj_build(sa->mode, sa->chunks, sa->n_chunks, sa->words, sa->ws, sa->vkey, s.off, d_counts, nv, s.adj, st);
    launched += 1;
  } else {
    cudaMemsetAsync(s.cursor, 0, (size_t)nv * sizeof(uint32_t), st);
    k_fill_adj<<<(int)((n_slots + 255) / 256), 256, 0, st>>>(N, n_slots, nv, d_counts, idx, s.off, valence,
                                                             s.cursor, s.adj);
    k_sort_adj<<<vb, 256, 0, st>>>(nv, n_slots, d_counts, s.off, s.cursor, valence, s.adj);
    cursor = s.cursor;
    launched += 2;
  }
  const int hard_norm_max = 10;
  const int max_norms = (iters / 2 - 3 < hard_norm_max ? iters / 2 - 3 : hard_norm_max);
  for (int m = 0; m < iters; ++m) {
    const int normal_mode = !sn ? 0 : ((m == 0 || m < max_norms || m < 3) ? 1 : 2);
    if (N == 3)
      k_dual<3><<<pbt, tb, 0, st>>>(n_prims, nv, d_counts, idx, pos, nrm, s.dual_p, s.dual_n, normal_mode);
    else
      k_dual<4><<<pbt, tb, 0, st>>>(n_prims, nv, d_counts, idx, pos, nrm, s.dual_p, s.dual_n, normal_mode);
    // primal after every dual step but the last (MeshProcessor.cpp:229-232),
    // and once more after the loop with set_colors false (ChunkGenerator.cpp:120)
    const int set_colors = (m < iters - 1) ? ((m == 3) || (m == 0 && iters <= 3)) : 0;
    k_primal<<<vbt, tb, 0, st>>>(nv, n_prims, n_slots, d_counts, s.off, cursor, valence, s.adj, boundary, s.dual_p,
                                 s.dual_n, pos, nrm, process_boundary, sn ? 1 : 0, set_colors);
    launched += 2;
  }
  return launched;
}

}  // namespace bmf
