// bmf_dropin -- a compiled C++ caller of libbmf_gb300.so, written the way a
// BinaryMeshFitting maintainer would call it (include/bmf.h directly, and the
// reference-named classes of include/bmf_adapter.hpp).
//
//   bmf_dropin check
//       1. the per-chunk replacement of ChunkGenerator::extract_chunk's body
//          (ChunkGenerator.cpp:98-124) through bmf_extract_chunk, on the
//          65^3-sample sphere-wave chunk, Mode R, without and with 4 sweeps;
//       2. the same chunk through DMCChunk::label_grid / label_edges /
//          polygonize and MeshProcessor<3>::init / optimize_dual_grid /
//          optimize_primal_grid / flush, which must give the same bytes;
//       3. ChunkGenerator::process_queue on two queues of the same shape (the
//          second reuses the plan: new descriptors, graph replay).
//       Prints one JSON object with the counts and chunk frames, so a test can
//       check them against the oracle.
//
//   bmf_dropin time <descs.bin> <field kind> <p0..p7> <mode> <placement> <iters> <normals> <warmup>
//       Times the plain drop-in loop: one bmf_extract_chunk per chunk over the
//       bmf_chunk_desc records of descs.bin, on device buffers allocated once
//       before the loop (one context, one stream, no allocation per call).
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "include/bmf.h"
#include "include/bmf_adapter.hpp"

namespace {

uint32_t bits(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
}

// FNV-1a of a byte range (a cheap equality fingerprint for the JSON report).
uint64_t fnv(const void* p, size_t n) {
  uint64_t h = 0xcbf29ce484222325ull;
  const uint8_t* b = (const uint8_t*)p;
  for (size_t i = 0; i < n; ++i) h = (h ^ b[i]) * 0x100000001b3ull;
  return h;
}

bmf_field sphere_wave() {
  bmf_field f = {};
  f.kind = BMF_FIELD_SPHERE_WAVE;
  const float p[6] = {32.0f, 32.0f, 32.0f, 20.0f, 1.5f, 0.3f};
  for (int i = 0; i < 6; ++i) f.params[i] = p[i];
  return f;
}

bmf_field terrain() {
  bmf_field f = {};
  f.kind = BMF_FIELD_TERRAIN_FBM;
  const float p[7] = {64.0f, 40.0f, 0.01f, 2.0f, 0.5f, 5.0f, 1337.0f};
  for (int i = 0; i < 7; ++i) f.params[i] = p[i];
  return f;
}

// One chunk through bmf_extract_chunk, growing the caller-owned buffers once
// when the first guess is too small (BMF_ERR_CAPACITY reports the needed
// counts).  Returns host copies of positions, normals and indices.
struct HostMesh {
  std::vector<float> pos, nrm;
  std::vector<uint32_t> idx;
  int64_t n_verts = 0, n_idx = 0;
  int contains_mesh = 0;
};

HostMesh extract_one(bmf::Context& ctx, const bmf_chunk_desc& desc, const bmf_field& field,
                     const bmf_extract_opts& opts) {
  bmf::VerticesIndicesBlock vi;
  int64_t vcap = 1024, icap = 4096;
  bmf_mesh m = {};
  for (int attempt = 0; attempt < 2; ++attempt) {
    vi.reserve(vcap, icap);
    m = vi.view();
    bmf_status s = bmf_extract_chunk(ctx.get(), &desc, &field, &opts, &m, ctx.stream());
    if (s == BMF_ERR_CAPACITY) {
      vcap = m.n_verts, icap = m.n_idx;
      continue;
    }
    bmf::check(s, ctx.get());
    break;
  }
  HostMesh h;
  h.n_verts = m.n_verts, h.n_idx = m.n_idx, h.contains_mesh = m.contains_mesh;
  h.pos = vi.pos.to_host((size_t)m.n_verts * 3, ctx.stream());
  h.nrm = vi.nrm.to_host((size_t)m.n_verts * 3, ctx.stream());
  h.idx = vi.idx.to_host((size_t)m.n_idx, ctx.stream());
  return h;
}

int check() {
  bmf::Context ctx(0);
  const bmf_field sw = sphere_wave();
  // 1. the per-chunk drop-in (configs' 64^3-cell sphere-wave chunk)
  bmf_chunk_desc desc = {{0.0f, 0.0f, 0.0f}, 1.0f, 65, 0};
  bmf_extract_opts plain = {BMF_MODE_R, BMF_PLACE_CENTER, 0, 0, 0, 0};
  HostMesh a = extract_one(ctx, desc, sw, plain);
  bmf_extract_opts smooth = {BMF_MODE_R, BMF_PLACE_CENTER, 4, 0, 1, 0};
  HostMesh b = extract_one(ctx, desc, sw, smooth);

  // 2. the reference-named classes: the same chunk, same 4 sweeps
  bmf::Sampler sampler = {sw, 64.0f};
  bmf::DMCChunk chunk(ctx, {0.0f, 0.0f, 0.0f}, 64.0f, 0, sampler, 65);
  chunk.label_grid(0.0f);
  chunk.label_edges();
  chunk.polygonize();
  bmf::MeshProcessor<3> mp(ctx, true, true);
  bool has_adj = mp.init(chunk.vi);
  mp.optimize_dual_grid(4, false);
  mp.optimize_primal_grid(false, false, false);
  mp.flush();
  std::vector<float> cpos = chunk.vi.pos.to_host((size_t)chunk.vi.n_verts * 3, ctx.stream());
  std::vector<float> cnrm = chunk.vi.nrm.to_host((size_t)chunk.vi.n_verts * 3, ctx.stream());
  std::vector<uint32_t> cidx = chunk.vi.idx.to_host((size_t)chunk.vi.n_idx, ctx.stream());
  bool classes_match = chunk.vi.n_verts == b.n_verts && chunk.vi.n_idx == b.n_idx &&
                       std::memcmp(cpos.data(), b.pos.data(), cpos.size() * 4) == 0 &&
                       std::memcmp(cnrm.data(), b.nrm.data(), cnrm.size() * 4) == 0 &&
                       std::memcmp(cidx.data(), b.idx.data(), cidx.size() * 4) == 0;

  // 3. process_queue twice with one queue shape
  bmf::WorldProperties props;
  props.max_level = 3;
  props.process_iters = 2;
  props.boundary_processing = false;
  props.smooth_normals = true;
  bmf::ChunkGenerator gen(ctx, props, {terrain(), 4096.0f}, 33);
  std::vector<bmf::WorldOctreeNode> nodes(8);
  std::vector<bmf::WorldOctreeNode*> queue;
  std::printf("{\"per_chunk\": {\"n_verts\": %lld, \"n_idx\": %lld, \"contains_mesh\": %d, \"pos_fnv\": \"%016llx\"},\n",
              (long long)a.n_verts, (long long)a.n_idx, a.contains_mesh,
              (unsigned long long)fnv(a.pos.data(), a.pos.size() * 4));
  std::printf(" \"per_chunk_smoothed\": {\"n_verts\": %lld, \"n_idx\": %lld, \"pos_fnv\": \"%016llx\", "
              "\"nrm_fnv\": \"%016llx\"},\n",
              (long long)b.n_verts, (long long)b.n_idx, (unsigned long long)fnv(b.pos.data(), b.pos.size() * 4),
              (unsigned long long)fnv(b.nrm.data(), b.nrm.size() * 4));
  std::printf(" \"classes\": {\"n_verts\": %lld, \"n_idx\": %lld, \"has_adjacency\": %d, \"match_extract_chunk\": %d},\n",
              (long long)chunk.vi.n_verts, (long long)chunk.vi.n_idx, (int)has_adj, (int)classes_match);
  std::printf(" \"queues\": [");
  for (int q = 0; q < 2; ++q) {
    queue.clear();
    for (int i = 0; i < 8; ++i) {
      // nodes of sizes 32..256 world units around the terrain band; the
      // second queue moves every node (same count and resolution)
      int level = i % 4;
      float size = 32.0f * (float)(1 << (3 - level));
      nodes[i] = {{1000.0f + 300.0f * i + 37.0f * q, 32.0f - 0.5f * size + 8.0f * q, 2000.0f - 150.0f * i}, size,
                  level};
      queue.push_back(&nodes[i]);
    }
    gen.process_queue(queue);
    std::printf("%s{\"plans_reused\": %d, \"n_verts\": %lld, \"chunks\": [", q ? ", " : "", gen.plans_reused,
                (long long)gen.n_verts);
    for (int i = 0; i < 8; ++i) {
      float delta;
      bmf::vec3 op;
      bmf::chunk_frame(nodes[i].pos, nodes[i].size, gen.overlap_for(nodes[i]), 33, &delta, &op);
      std::printf("%s{\"origin_bits\": [%u, %u, %u], \"scale_bits\": %u, \"contains_mesh\": %d, "
                  "\"n_verts\": %lld, \"n_idx\": %lld}",
                  i ? ", " : "", bits(op.x), bits(op.y), bits(op.z), bits(delta), (int)nodes[i].contains_mesh,
                  (long long)nodes[i].vertex_count, (long long)nodes[i].index_count);
    }
    std::printf("]}");
  }
  std::printf("]}\n");
  return classes_match ? 0 : 1;
}

int time_loop(int argc, char** argv) {
  if (argc < 17) {
    std::fprintf(stderr, "usage: bmf_dropin time <descs.bin> <kind> <p0..p7> <mode> <placement> <iters> <normals> "
                         "<warmup>\n");
    return 2;
  }
  FILE* f = std::fopen(argv[2], "rb");
  if (!f) {
    std::perror(argv[2]);
    return 2;
  }
  std::vector<bmf_chunk_desc> descs;
  bmf_chunk_desc d;
  while (std::fread(&d, sizeof(d), 1, f) == 1) descs.push_back(d);
  std::fclose(f);
  bmf_field field = {};
  field.kind = std::atoi(argv[3]);
  for (int i = 0; i < 8; ++i) field.params[i] = (float)std::atof(argv[4 + i]);
  bmf_extract_opts opts = {std::atoi(argv[12]), std::atoi(argv[13]), std::atoi(argv[14]), 0, std::atoi(argv[15]), 0};
  int warmup = std::atoi(argv[16]);

  bmf::Context ctx(0);
  // size the caller-owned buffers once: the largest chunk's counts
  bmf::VerticesIndicesBlock vi;
  int64_t vcap = 1024, icap = 4096;
  vi.reserve(vcap, icap);
  for (const bmf_chunk_desc& c : descs) {
    bmf_mesh m = vi.view();
    bmf_status s = bmf_extract_chunk(ctx.get(), &c, &field, &opts, &m, ctx.stream());
    if (s == BMF_ERR_CAPACITY) {
      vcap = std::max(vcap, m.n_verts), icap = std::max(icap, m.n_idx);
      vi.reserve(vcap, icap);
      continue;
    }
    bmf::check(s, ctx.get());
  }
  for (int w = 0; w < warmup && w < (int)descs.size(); ++w) {
    bmf_mesh m = vi.view();
    bmf::check(bmf_extract_chunk(ctx.get(), &descs[w], &field, &opts, &m, ctx.stream()), ctx.get());
  }
  bmf::check_cuda(cudaStreamSynchronize(ctx.stream()));
  int64_t verts = 0, launches0 = bmf_launch_count(ctx.get());
  auto t0 = std::chrono::steady_clock::now();
  for (const bmf_chunk_desc& c : descs) {
    bmf_mesh m = vi.view();
    bmf::check(bmf_extract_chunk(ctx.get(), &c, &field, &opts, &m, ctx.stream()), ctx.get());
    verts += m.n_verts;
  }
  bmf::check_cuda(cudaStreamSynchronize(ctx.stream()));
  double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  std::printf("{\"chunks\": %zu, \"seconds\": %.6f, \"chunks_per_s\": %.3f, \"vertices\": %lld, \"launches\": %lld}\n",
              descs.size(), s, descs.size() / s, (long long)verts,
              (long long)(bmf_launch_count(ctx.get()) - launches0));
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  try {
    if (argc >= 2 && std::strcmp(argv[1], "check") == 0) return check();
    if (argc >= 2 && std::strcmp(argv[1], "time") == 0) return time_loop(argc, argv);
  } catch (const bmf::Error& e) {
    std::fprintf(stderr, "bmf_dropin: %s (status %d)\n", e.what(), (int)e.status);
    return 3;
  }
  std::fprintf(stderr, "usage: bmf_dropin check | time ...\n");
  return 2;
}
