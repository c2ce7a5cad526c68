/* The oracle's entry points on seeded inputs, for a build with
 * AddressSanitizer and UndefinedBehaviorSanitizer (make -C oracle sanitize).
 * Test infrastructure only: it checks that the CPU restatement -- the checker
 * of every parity test -- reads and writes only its own buffers and has no
 * undefined behaviour on the shapes the tests use (1-cell grids to 33^3,
 * every field kind, both topologies and all placements, the sweeps, the draw
 * layout, the LOD generator, the batch driver and the FP64 fitting path).
 * Prints "oracle sanity ok" and exits 0; a sanitizer report aborts. */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "bmf_oracle.h"

static void* xcalloc(size_t n, size_t size) {
  void* p = calloc(n ? n : 1, size ? size : 1);
  if (!p) {
    fprintf(stderr, "out of memory\n");
    exit(2);
  }
  return p;
}

static int64_t one_chunk(int kind, const float* prm, int dim, const float org[3], float scale) {
  const int64_t n = (int64_t)dim * dim * dim;
  const int zc = (dim + 31) / 32;
  float* d = xcalloc((size_t)n, sizeof(float));
  uint32_t* w = xcalloc((size_t)dim * dim * zc, sizeof(uint32_t));
  uint64_t* m = xcalloc((size_t)dim * dim * 4 * zc, sizeof(uint64_t));
  if (kind == 0)
    memcpy(d, prm, sizeof(float) * (size_t)n);  /* a grid input: prm holds the samples */
  else
    bmfo_fill_field(kind, prm, dim, org, scale, d);
  const int cm = bmfo_label_grid(dim, d, w);
  bmfo_cell_masks(dim, w, m);
  int64_t total = 0;
  if (cm) {
    bmfo_counts c;
    memset(&c, 0, sizeof(c));
    bmfo_extract_r(dim, d, m, 0, 0, 0, NULL, NULL, NULL, NULL, NULL, NULL, &c);
    float* pos = xcalloc((size_t)c.n_verts * 3, sizeof(float));
    float* nrm = xcalloc((size_t)c.n_verts * 3, sizeof(float));
    uint8_t* bnd = xcalloc((size_t)c.n_verts, 1);
    uint8_t* val = xcalloc((size_t)c.n_verts, 1);
    uint32_t* idx = xcalloc((size_t)c.n_idx, sizeof(uint32_t));
    uint32_t* lin = xcalloc((size_t)c.n_cells, sizeof(uint32_t));
    uint16_t* cmask = xcalloc((size_t)c.n_cells, sizeof(uint16_t));
    if (bmfo_extract_r(dim, d, m, c.n_verts, c.n_idx, c.n_cells, pos, bnd, val, idx, lin, cmask, &c) != 0) exit(3);
    bmfo_process(3, c.n_verts, pos, nrm, bnd, val, c.n_idx, idx, 4, 0, 1);
    {
      float* p = xcalloc((size_t)c.n_verts * 3, sizeof(float));
      float* nn = xcalloc((size_t)c.n_verts * 3, sizeof(float));
      float* cc = xcalloc((size_t)c.n_verts * 3, sizeof(float));
      bmfo_format(c.n_verts, pos, nrm, c.n_idx, idx, 0, 1, p, nn, cc);
      free(p), free(nn), free(cc);
    }
    total += c.n_verts;
    free(pos), free(nrm), free(bnd), free(val), free(idx), free(lin), free(cmask);
    for (int placement = 0; placement < 4; ++placement) {
      bmfo_counts q;
      memset(&q, 0, sizeof(q));
      bmfo_extract_q(dim, d, w, placement, 0, 0, NULL, NULL, NULL, NULL, &q);
      float* qp = xcalloc((size_t)q.n_verts * 3, sizeof(float));
      float* qn = xcalloc((size_t)q.n_verts * 3, sizeof(float));
      uint8_t* qb = xcalloc((size_t)q.n_verts, 1);
      uint8_t* qv = xcalloc((size_t)q.n_verts, 1);
      uint32_t* qi = xcalloc((size_t)q.n_idx, sizeof(uint32_t));
      if (bmfo_extract_q(dim, d, w, placement, q.n_verts, q.n_idx, qp, qb, qv, qi, &q) != 0) exit(4);
      bmfo_process(4, q.n_verts, qp, qn, qb, qv, q.n_idx, qi, 2, 1, 1);
      {
        const int64_t cap = q.n_idx / 4 * 4;
        float* p = xcalloc((size_t)cap * 3, sizeof(float));
        float* nn = xcalloc((size_t)cap * 3, sizeof(float));
        float* cc = xcalloc((size_t)cap * 3, sizeof(float));
        bmfo_format(q.n_verts, qp, qn, q.n_idx, qi, 1, 0, p, nn, cc);
        free(p), free(nn), free(cc);
      }
      total += q.n_verts;
      free(qp), free(qn), free(qb), free(qv), free(qi);
    }
  }
  free(d), free(w), free(m);
  return total;
}

int main(void) {
  const float sphere_wave[8] = {32.0f, 32.0f, 32.0f, 20.0f, 1.5f, 0.3f, 0.0f, 0.0f};
  const float terrain[8] = {64.0f, 40.0f, 0.01f, 2.0f, 0.5f, 5.0f, 1337.0f, 0.0f};
  const float terrain2d[8] = {0.25f, 75.0f, 13.0f, 0.87f, 0.585f, 0.488f, 1337.0f, 3.0f};
  const float torus[8] = {16.0f, 16.0f, 16.0f, 9.0f, 3.0f, 0.0f, 0.0f, 0.0f};
  const float sphere[8] = {8.0f, 8.0f, 8.0f, 6.5f, 0.0f, 0.0f, 0.0f, 0.0f};
  const float cuboid[8] = {8.0f, 8.0f, 8.0f, 5.0f, 4.0f, 3.0f, 0.0f, 0.0f};
  const float plane[8] = {7.3f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
  const float org0[3] = {0.0f, 0.0f, 0.0f};
  const float org1[3] = {1000.0f, 32.0f, 2000.0f};
  const float org2[3] = {500.0f, -160.0f, 300.0f};
  const int dims[] = {2, 3, 5, 17, 33};
  int64_t total = 0;
  for (int i = 0; i < 5; ++i) {
    const int dim = dims[i];
    total += one_chunk(1, sphere_wave, dim, org0, 64.0f / (float)dim);
    total += one_chunk(2, terrain, dim, org1, 2.0f);
    total += one_chunk(7, terrain2d, dim, org2, 4.0f);
    total += one_chunk(3, torus, dim, org0, 32.0f / (float)dim);
    total += one_chunk(4, sphere, dim, org0, 16.0f / (float)dim);
    total += one_chunk(5, cuboid, dim, org0, 16.0f / (float)dim);
    total += one_chunk(6, plane, dim, org0, 16.0f / (float)dim);
  }
  /* a grid input of random signs */
  {
    const int dim = 9;
    float* g = xcalloc(dim * dim * dim, sizeof(float));
    uint32_t s = 12345u;
    for (int k = 0; k < dim * dim * dim; ++k) {
      s = s * 1664525u + 1013904223u;
      g[k] = (float)((int)(s >> 8) % 2001 - 1000) / 997.0f;
    }
    total += one_chunk(0, g, dim, org0, 1.0f);
    free(g);
  }
  /* QEF */
  {
    float p[36], nm[36], out[3];
    double pd[36], nd[36], od[3];
    for (int k = 0; k < 36; ++k) {
      p[k] = (float)((k * 37) % 11) * 0.1f;
      nm[k] = (float)((k * 17) % 7) * 0.2f - 0.6f;
      pd[k] = p[k];
      nd[k] = nm[k];
    }
    for (int cnt = 1; cnt <= 12; ++cnt) {
      bmfo_qef_f32(p, nm, cnt, out);
      bmfo_qef_f64(pd, nd, cnt, od);
    }
  }
  /* LOD generator */
  {
    const float prm[10] = {0.0f, 0.0f, 0.0f, 4096.0f, 2048.0f, 64.0f, 2048.0f, 1.0f, 2.0f, 0.035f};
    const int64_t cap = 1 << 16;
    float* rows = xcalloc((size_t)cap * 6, sizeof(float));
    const int64_t n = bmfo_lod_generate(prm, 1, 7, 33, 1, 4, rows, cap);
    if (n <= 0 || n > cap) exit(5);
    free(rows);
  }
  /* batch driver with digests, two threads */
  {
    const int nc = 6;
    float desc[5 * 6];
    for (int c = 0; c < nc; ++c) {
      desc[5 * c + 0] = 1000.0f + 64.0f * c;
      desc[5 * c + 1] = 32.0f;
      desc[5 * c + 2] = 2000.0f;
      desc[5 * c + 3] = 2.0f;
      desc[5 * c + 4] = (float)(c % 2 ? 17 : 9);
    }
    int64_t counts[3 * 6];
    uint64_t dig[4 * 6];
    bmfo_extract_batch_digest(nc, desc, 2, terrain, 0, 0, 4, 0, 1, counts, dig, 2);
    bmfo_extract_batch_digest(nc, desc, 2, terrain, 1, 2, 4, 1, 1, counts, dig, 2);
  }
  /* FP64 fitting path with gradients */
  {
    const int dim = 9;
    const int64_t n = dim * dim * dim;
    double* d = xcalloc((size_t)n, sizeof(double));
    double* g = xcalloc((size_t)n, sizeof(double));
    unsigned char* nb = xcalloc((size_t)n, 1);
    for (int x = 0; x < dim; ++x)
      for (int y = 0; y < dim; ++y)
        for (int z = 0; z < dim; ++z) {
          const double dx = x - 4.0, dy = y - 4.0, dz = z - 4.1;
          d[(x * dim + y) * dim + z] = dx * dx + dy * dy + dz * dz - 9.0;
        }
    const double box[7] = {4.0, 4.0, 4.0, 2.0, 2.5, 1.5, 0.5};
    const double sph[8] = {4.0, 4.0, 4.0, 2.5, 5.0, 4.0, 4.0, 1.5};
    int64_t oc[3];
    uint64_t h = 0;
    bmfo_fit_loss_f64(dim, d, 4, box, g, oc, &h, nb);
    bmfo_fit_loss_spheres_f64(dim, d, 4, sph, 2, g, oc, &h, nb);
    free(d), free(g), free(nb);
  }
  printf("oracle sanity ok (%lld vertices)\n", (long long)total);
  return 0;
}
