// bmf_polygonize_noalloc: the Mode R / Mode Q extraction of bmf_polygonize
// for callers that must not allocate device memory.
//
// Some hosts of this library cannot call cudaMalloc at the point where they
// extract a chunk: a renderer or engine that owns all device memory through
// its own pool and forbids other allocations, a real-time thread that may not
// block on the driver's allocator, or a caller that is already inside a
// region where allocating is not allowed.  This entry point takes no context
// (creating one allocates) and keeps its per-call scratch -- the chunk
// record, the contains_mesh flags, the per-word vertex / index counts and the
// per-word bit-planes -- in one file-scope device array of fixed size, so a
// call allocates nothing.  The caller still passes the density, the
// occupancy words and the output buffers.
//
// Limits and rules:
//  - chunks of at most BMF_NOALLOC_MAX_DIM (129) samples per axis; larger dims
//    are rejected with BMF_ERR_NOT_SUPPORTED before anything is launched;
//  - every GPU that loads the library holds the array (about 1.7 MB) until the
//    process exits;
//  - all calls share the one array: two calls whose work overlaps on the GPU
//    (different streams, or different host threads on the same device) race
//    and corrupt each other's counts.  Serialise them (one stream, or events);
//  - the array keeps the previous call's contents; everything the kernels read
//    before writing (the contains_mesh flags) is cleared by each call;
//  - the first call on a device looks up the array's device address for that
//    device (cudaGetSymbolAddress, with that device current) and caches it;
//    under CUDA's lazy module loading (the default) that lookup is also when
//    the driver loads this library's device code on the device and places the
//    array, so the first call per device can allocate device memory once.
//    Hosts that forbid any allocation later make that first call at start-up,
//    and before any stream capture.
#include <mutex>

#include "../../include/bmf.h"
#include "bmf_device.cuh"
#include "bmf_internal.h"

namespace bmf {
namespace {

constexpr int kNoAllocMaxDim = BMF_NOALLOC_MAX_DIM;
constexpr int64_t kMaxWords = (int64_t)kNoAllocMaxDim * kNoAllocMaxDim * ((kNoAllocMaxDim + 31) / 32);
// Layout (u32 units): [0, 64) chunk record + unit range + flags + chunk totals
// + device totals; then vcnt, icnt and the 3 bit-planes, one entry per word.
constexpr int64_t kHeader = 64;
constexpr int64_t kScratchWords = kHeader + 5 * kMaxWords;

static __device__ __align__(256) uint32_t g_noalloc_scratch[kScratchWords];

constexpr int kMaxDevices = 64;
std::mutex g_lookup_mutex;
uint32_t* g_scratch_ptr[kMaxDevices] = {};

// Writes the single chunk record and its unit range into the scratch header.
__global__ void k_noalloc_header(ChunkDev c, ChunkDev* dst, int* units) {
  *dst = c;
  units[0] = 0;
  units[1] = c.dim;
}

// Device address of the scratch array for the current device (looked up once).
bmf_status scratch_for_current_device(uint32_t** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return BMF_ERR_CUDA;
  std::lock_guard<std::mutex> lock(g_lookup_mutex);
  if (!g_scratch_ptr[dev]) {
    uint32_t* p = nullptr;
    if (cudaGetSymbolAddress((void**)&p, g_noalloc_scratch) != cudaSuccess || !p) return BMF_ERR_CUDA;
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return BMF_OK;
}

}  // namespace
}  // namespace bmf

using namespace bmf;

extern "C" bmf_status bmf_polygonize_noalloc(int32_t dim, const float* d_density, const uint32_t* d_words,
                                             int32_t mode, int32_t placement, bmf_mesh* out, void* stream) {
  if (dim > kNoAllocMaxDim) return BMF_ERR_NOT_SUPPORTED;
  if (dim < 2 || !d_words || !out || !out->d_pos || !out->d_idx || out->vcap < 0 || out->icap < 0 ||
      (mode != BMF_MODE_R && mode != BMF_MODE_Q) || placement < 0 || placement > 2)
    return BMF_ERR_INVALID_ARGUMENT;
  if (!d_density && (mode == BMF_MODE_R || placement != BMF_PLACE_CENTER)) return BMF_ERR_INVALID_ARGUMENT;
  cudaStream_t st = (cudaStream_t)stream;
  uint32_t* base = nullptr;
  bmf_status s = scratch_for_current_device(&base);
  if (s != BMF_OK) return s;
  static_assert(sizeof(ChunkDev) <= 32 * sizeof(uint32_t), "chunk record must fit the scratch header");
  ChunkDev* d_c = (ChunkDev*)base;                      // u32 [0, 32)
  int* d_u = (int*)(base + 32);                         // [32, 34)
  uint32_t* d_flags = base + 34;                        // [34, 35)
  uint32_t* d_tot = base + 36;                          // [36, 38)
  int64_t* d_totals = (int64_t*)(base + 40);            // [40, 44), 8-byte aligned
  const int zc = (dim + 31) / 32;
  const int64_t nw = (int64_t)dim * dim * zc;
  WordScratch ws{base + kHeader, base + kHeader + nw, base + kHeader + 2 * nw};

  ChunkDev c{};
  c.scale = 1.0f;
  c.dim = dim;
  c.zc = zc;
  k_noalloc_header<<<1, 1, 0, st>>>(c, d_c, d_u);
  launch_word_flags(d_c, 1, d_words, d_flags, st);  // clears and sets the flags
  launch_count(mode, d_c, 1, d_u, dim, d_words, d_flags, ws, st);
  launch_scan_chunks(d_c, 1, ws, d_tot, st);
  launch_chunk_offsets(d_c, 1, d_tot, d_flags, out->vcap, out->icap, nullptr, d_totals, st);
  MeshOut mo{out->d_pos, out->d_nrm, out->d_boundary, out->d_valence, out->d_idx, nullptr, out->vcap, out->icap};
  launch_emit(mode, placement, d_c, 1, d_u, dim, d_words, d_density, d_flags, ws, mo, nullptr, st);
  if (cudaPeekAtLastError() != cudaSuccess) return BMF_ERR_CUDA;
  int64_t totals[2] = {0, 0};
  uint32_t flags = 0;
  if (cudaMemcpyAsync(totals, d_totals, sizeof(totals), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaMemcpyAsync(&flags, d_flags, sizeof(flags), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return BMF_ERR_CUDA;
  out->n_verts = totals[0];
  out->n_idx = totals[1];
  out->contains_mesh = ((flags & 1u) || ((flags & 6u) == 6u)) ? 1 : 0;
  out->prim_size = mode == BMF_MODE_R ? 3 : 4;
  if (out->n_verts > out->vcap || out->n_idx > out->icap) return BMF_ERR_CAPACITY;
  return BMF_OK;
}
