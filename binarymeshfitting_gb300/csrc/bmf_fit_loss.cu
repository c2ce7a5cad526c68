// The loss of the batched-fitting workload on the device: for each chunk the
// mean, over its output vertices, of the squared distance to a union of
// spheres (signed: |p - c| - r, the nearest sphere), summed over the chunks;
// and its gradient with respect to the vertex positions.  Everything is read
// on the device (vertex totals and chunk offsets of the last forward), so a
// fitting step -- forward, loss, backward, optimizer -- needs no host sync and
// can be captured in one CUDA graph.  The sum is reduced in a fixed order
// (per-block partial sums, then one block over them), so it is reproducible.
#include "../../include/bmf.h"
#include "bmf_device.cuh"
#include "bmf_internal.h"

namespace bmf {

constexpr int kLossThreads = 256;

__global__ void __launch_bounds__(kLossThreads) k_loss_spheres(const ChunkDev* __restrict__ chunks, int n_chunks,
                                                               const uint32_t* __restrict__ tot,
                                                               const int64_t* __restrict__ d_totals, int64_t vcap,
                                                               const float* __restrict__ pos,
                                                               const float* __restrict__ spheres, int k,
                                                               float* __restrict__ grad, float* __restrict__ partial) {
  __shared__ float s_warp[kLossThreads / 32];
  const int64_t nv = min(vcap, d_totals[0]);
  float acc = 0.0f;
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < vcap; v += (int64_t)gridDim.x * blockDim.x) {
    if (v >= nv) {
      grad[3 * v] = grad[3 * v + 1] = grad[3 * v + 2] = 0.0f;
      continue;
    }
    // the vertex's chunk: the last with vout <= v (an empty chunk shares its
    // offset with the next one)
    int lo = 0, hi = n_chunks - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (chunks[mid].vout <= v) lo = mid; else hi = mid - 1;
    }
    const float w = 1.0f / (float)max(1u, tot[2 * lo]);
    const float px = pos[3 * v], py = pos[3 * v + 1], pz = pos[3 * v + 2];
    const float* s = spheres + (int64_t)lo * k * 4;
    float best = INFINITY, bx = 0.0f, by = 0.0f, bz = 0.0f, bl = 0.0f;
    for (int j = 0; j < k; ++j) {
      const float dx = px - s[4 * j], dy = py - s[4 * j + 1], dz = pz - s[4 * j + 2];
      const float l = sqrtf((dx * dx + dy * dy) + dz * dz);
      const float d = l - s[4 * j + 3];
      if (d < best) {
        best = d;
        bx = dx, by = dy, bz = dz, bl = l;
      }
    }
    acc = acc + best * best * w;
    const float g = 2.0f * best * w, inv = bl > 0.0f ? g / bl : 0.0f;
    grad[3 * v] = bx * inv;
    grad[3 * v + 1] = by * inv;
    grad[3 * v + 2] = bz * inv;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(kFull, acc, o);
  if ((threadIdx.x & 31) == 0) s_warp[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    float t = threadIdx.x < kLossThreads / 32 ? s_warp[threadIdx.x] : 0.0f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(kFull, t, o);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
  }
}

// The partial sums in a fixed order: each thread a strided slice, then a tree.
__global__ void __launch_bounds__(kLossThreads) k_loss_sum(const float* __restrict__ partial, int n,
                                                           float* __restrict__ loss) {
  __shared__ float s[kLossThreads];
  float t = 0.0f;
  for (int i = threadIdx.x; i < n; i += kLossThreads) t += partial[i];
  s[threadIdx.x] = t;
  __syncthreads();
  for (int h = kLossThreads / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) s[threadIdx.x] += s[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) *loss = s[0];
}

int launch_fit_loss_spheres(const ChunkDev* d_chunks, int n_chunks, const uint32_t* d_tot, const int64_t* d_totals,
                            int64_t vcap, const float* pos, const float* spheres, int k, float* grad, float* partial,
                            int n_partial, float* loss, cudaStream_t st) {
  k_loss_spheres<<<n_partial, kLossThreads, 0, st>>>(d_chunks, n_chunks, d_tot, d_totals, vcap, pos, spheres, k, grad,
                                                     partial);
  k_loss_sum<<<1, kLossThreads, 0, st>>>(partial, n_partial, loss);
  return 2;
}

// Adam (Kingma & Ba) over the learnable grids, the optimizer of the batched
// fitting workload, with torch.optim.Adam's arithmetic (no weight decay, no
// amsgrad): m = b1 m + (1 - b1) g, v = b2 v + (1 - b2) g^2,
// p -= (lr / (1 - b1^t)) m / (sqrt(v) / sqrt(1 - b2^t) + eps).  The step
// count t lives on the device (read here, advanced by k_adam_tick after), so a
// replayed CUDA graph advances it.  One pass over p, g, m and v: HBM-bound,
// float4 accesses.
__device__ __forceinline__ void adam_one(float& p, float g, float& m, float& v, float b1, float b2, float step_size,
                                         float bc2s, float eps) {
  m = b1 * m + (1.0f - b1) * g;
  v = b2 * v + (1.0f - b2) * g * g;
  p = p - step_size * (m / (sqrtf(v) / bc2s + eps));
}

__global__ void __launch_bounds__(256) k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                                              float* __restrict__ v, int64_t n, const int* __restrict__ step, float lr,
                                              float b1, float b2, float eps, int vec) {
  const int t = *step + 1;
  const float bc1 = 1.0f - powf(b1, (float)t), bc2 = 1.0f - powf(b2, (float)t);
  const float step_size = lr / bc1, bc2s = sqrtf(bc2);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t i0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int64_t done = 0;
  if (vec) {  // float4 body (all four arrays 16-byte aligned)
    const int64_t n4 = n / 4;
    for (int64_t i = i0; i < n4; i += stride) {
      float4 P = reinterpret_cast<float4*>(p)[i], M = reinterpret_cast<float4*>(m)[i];
      float4 V = reinterpret_cast<float4*>(v)[i];
      const float4 G = __ldg(reinterpret_cast<const float4*>(g) + i);
      adam_one(P.x, G.x, M.x, V.x, b1, b2, step_size, bc2s, eps);
      adam_one(P.y, G.y, M.y, V.y, b1, b2, step_size, bc2s, eps);
      adam_one(P.z, G.z, M.z, V.z, b1, b2, step_size, bc2s, eps);
      adam_one(P.w, G.w, M.w, V.w, b1, b2, step_size, bc2s, eps);
      reinterpret_cast<float4*>(p)[i] = P;
      reinterpret_cast<float4*>(m)[i] = M;
      reinterpret_cast<float4*>(v)[i] = V;
    }
    done = n4 * 4;
  }
  for (int64_t i = done + i0; i < n; i += stride) {
    float P = p[i], M = m[i], V = v[i];
    adam_one(P, __ldg(g + i), M, V, b1, b2, step_size, bc2s, eps);
    p[i] = P;
    m[i] = M;
    v[i] = V;
  }
}

__global__ void k_adam_tick(int* step) { *step = *step + 1; }

int launch_adam(float* p, const float* g, float* m, float* v, int64_t n, int* step, float lr, float b1, float b2,
                float eps, cudaStream_t st) {
  static std::atomic<int> grid[64] = {};
  const int gsz = per_device_once(grid, [](int dev) {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return (sms > 0 ? sms : 1) * 8;
  });
  const int vec = (((uintptr_t)p | (uintptr_t)g | (uintptr_t)m | (uintptr_t)v) & 15) == 0;
  k_adam<<<gsz, 256, 0, st>>>(p, g, m, v, n, step, lr, b1, b2, eps, vec);
  k_adam_tick<<<1, 1, 0, st>>>(step);
  return 2;
}

}  // namespace bmf
