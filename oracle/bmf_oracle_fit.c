/* FP64 oracle of the differentiable extraction path (TEST INFRASTRUCTURE ONLY).
 *
 * Forward, all in double:
 *   topology   Mode Q of bmf_oracle.c (DMC quads from the signs of the density,
 *              groups from Tables.hpp:96-354 via the packed case table);
 *   placement  per vertex the QEF of qef_simd.h:411-461 on the group's hermite
 *              data -- crossing points by the reference's lerp
 *              (DMCChunk.cpp:657-662), normals = normalised lerp of the
 *              central-difference grid gradients -- solved with an eigen
 *              decomposition (cyclic Jacobi to convergence) and the same
 *              truncated pseudo-inverse (min(|s|, |1/s|) < 1e-3 -> 0); a
 *              solution outside its cell falls back to the mass point;
 *   smoothing  `iters` MeshProcessor<4> position sweeps in the order
 *              ChunkGenerator::extract_chunk runs them (MeshProcessor.cpp:
 *              130-306): dual = quad centroid, primal = mean of the incident
 *              dual points, boundary vertices frozen;
 *   loss       mean over vertices of sdf(p)^2 for a rounded box.
 * Backward: the exact adjoint of that function with the discrete choices
 * (topology, QEF truncation pattern, mass-point fallback) held fixed.  The
 * pseudo-inverse A+ = V f(S) V^T is differentiated with the Daleckii-Krein
 * formula, dA+ = V (F o (V^T dA V)) V^T, F_ij = (f_i - f_j)/(s_i - s_j),
 * F_ii = f'(s_i).
 *
 * This is the reference gradient the GPU adjoint (float) is measured against,
 * itself validated by central finite differences of this forward.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "bmf_oracle.h"
#include "../binarymeshfitting_gb300/csrc/bmf_case_tables.h"

static const int fc_corner[12][2] = {{0, 4}, {1, 5}, {2, 6}, {3, 7}, {0, 2}, {1, 3},
                                     {4, 6}, {5, 7}, {0, 1}, {2, 3}, {4, 5}, {6, 7}};

typedef struct {
  int dim;
  const double* s;
} fgrid;

static double fs(const fgrid* g, int x, int y, int z) { return g->s[((size_t)x * g->dim + y) * g->dim + z]; }
static int fin(const fgrid* g, int x, int y, int z) { return fs(g, x, y, z) < 0.0; }

/* central-difference gradient (one-sided at faces, as bmf_oracle.c) and its
 * stencil: g[a] = (s[hi] - s[lo]) * h */
static void fgrad(const fgrid* g, int x, int y, int z, double out[3], int lo[3][3], int hi[3][3], double h[3]) {
  int c[3] = {x, y, z};
  for (int a = 0; a < 3; ++a) {
    for (int k = 0; k < 3; ++k) lo[a][k] = hi[a][k] = c[k];
    h[a] = 0.5;
    if (c[a] > 0) lo[a][a]--; else h[a] = 1.0;
    if (c[a] < g->dim - 1) hi[a][a]++; else h[a] = 1.0;
    out[a] = (fs(g, hi[a][0], hi[a][1], hi[a][2]) - fs(g, lo[a][0], lo[a][1], lo[a][2])) * h[a];
  }
}

/* symmetric 3x3 eigen decomposition by cyclic Jacobi: A = V diag(w) V^T */
static void eig3(const double A_in[3][3], double w[3], double V[3][3]) {
  double A[3][3];
  memcpy(A, A_in, sizeof(A));
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) V[i][j] = (i == j);
  for (int sweep = 0; sweep < 30; ++sweep) {
    double off = fabs(A[0][1]) + fabs(A[0][2]) + fabs(A[1][2]);
    if (off < 1e-300) break;
    for (int p = 0; p < 2; ++p)
      for (int q = p + 1; q < 3; ++q) {
        if (A[p][q] == 0.0) continue;
        double tau = (A[q][q] - A[p][p]) / (2.0 * A[p][q]);
        double t = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
        double c = 1.0 / sqrt(1.0 + t * t), s = t * c;
        for (int k = 0; k < 3; ++k) {
          double akp = A[k][p], akq = A[k][q];
          A[k][p] = c * akp - s * akq;
          A[k][q] = s * akp + c * akq;
        }
        for (int k = 0; k < 3; ++k) {
          double apk = A[p][k], aqk = A[q][k];
          A[p][k] = c * apk - s * aqk;
          A[q][k] = s * apk + c * aqk;
        }
        for (int k = 0; k < 3; ++k) {
          double vkp = V[k][p], vkq = V[k][q];
          V[k][p] = c * vkp - s * vkq;
          V[k][q] = s * vkp + c * vkq;
        }
      }
  }
  for (int i = 0; i < 3; ++i) w[i] = A[i][i];
}

#define FIT_MAXE 12

typedef struct {
  int cx, cy, cz, mask, group;
  int ne;
  int edges[FIT_MAXE];
  int qef;            /* 1: QEF solution used, 0: mass point */
  double x[3];        /* placed position */
} fvert;

/* hermite point, normal and the quantities their adjoint needs */
typedef struct {
  int a0[3], a1[3], ax;
  double s0, s1, mu;
  double p[3], n[3], G[3], Glen, g0[3], g1[3];
  int lo0[3][3], hi0[3][3], lo1[3][3], hi1[3][3];
  double h0[3], h1[3];
} fherm;

static void fhermite(const fgrid* g, const fvert* v, int e, fherm* H) {
  int ca = fc_corner[e][0], cb = fc_corner[e][1];
  int c[3] = {v->cx, v->cy, v->cz};
  for (int k = 0; k < 3; ++k) {
    H->a0[k] = c[k] + ((ca >> (2 - k)) & 1);
    H->a1[k] = c[k] + ((cb >> (2 - k)) & 1);
  }
  H->ax = e >> 2;
  H->s0 = fs(g, H->a0[0], H->a0[1], H->a0[2]);
  H->s1 = fs(g, H->a1[0], H->a1[1], H->a1[2]);
  H->mu = (0.0 - H->s0) / (H->s1 - H->s0);
  for (int k = 0; k < 3; ++k) H->p[k] = (H->a1[k] - H->a0[k]) * H->mu + H->a0[k];
  fgrad(g, H->a0[0], H->a0[1], H->a0[2], H->g0, H->lo0, H->hi0, H->h0);
  fgrad(g, H->a1[0], H->a1[1], H->a1[2], H->g1, H->lo1, H->hi1, H->h1);
  for (int k = 0; k < 3; ++k) H->G[k] = H->g0[k] + (H->g1[k] - H->g0[k]) * H->mu;
  H->Glen = sqrt(H->G[0] * H->G[0] + H->G[1] * H->G[1] + H->G[2] * H->G[2]);
  for (int k = 0; k < 3; ++k) H->n[k] = H->G[k] / H->Glen;
}

typedef struct {
  double A[3][3], b[3], m[3], r[3], w[3], V[3][3], inv[3], y[3];
  int k;
} fqef;

static void fqef_solve(const fherm* H, int k, fqef* Q) {
  memset(Q, 0, sizeof(*Q));
  Q->k = k;
  for (int i = 0; i < k; ++i) {
    double d = H[i].n[0] * H[i].p[0] + H[i].n[1] * H[i].p[1] + H[i].n[2] * H[i].p[2];
    for (int r = 0; r < 3; ++r) {
      for (int c = 0; c < 3; ++c) Q->A[r][c] += H[i].n[r] * H[i].n[c];
      Q->b[r] += d * H[i].n[r];
      Q->m[r] += H[i].p[r];
    }
  }
  for (int r = 0; r < 3; ++r) Q->m[r] /= k;
  for (int r = 0; r < 3; ++r) Q->r[r] = Q->b[r] - (Q->A[r][0] * Q->m[0] + Q->A[r][1] * Q->m[1] + Q->A[r][2] * Q->m[2]);
  eig3(Q->A, Q->w, Q->V);
  for (int i = 0; i < 3; ++i) {
    double oo = 1.0 / Q->w[i];
    double mn = fabs(Q->w[i]) < fabs(oo) ? fabs(Q->w[i]) : fabs(oo);
    Q->inv[i] = mn >= 0.001 ? oo : 0.0;
  }
  for (int r = 0; r < 3; ++r) {
    Q->y[r] = 0.0;
    for (int c = 0; c < 3; ++c) {
      double P = 0.0;
      for (int i = 0; i < 3; ++i) P += Q->V[r][i] * Q->inv[i] * Q->V[c][i];
      Q->y[r] += P * Q->r[c];
    }
  }
}

static double sdf_box(const double* box, const double p[3], double grad[3]) {
  /* box: centre (3), half extents (3), corner radius */
  double q[3], sp[3], mq[3], l2 = 0.0;
  for (int k = 0; k < 3; ++k) {
    double d = p[k] - box[k];
    sp[k] = d >= 0 ? 1.0 : -1.0;
    q[k] = fabs(d) - box[3 + k] + box[6];
    mq[k] = q[k] > 0 ? q[k] : 0.0;
    l2 += mq[k] * mq[k];
  }
  double len = sqrt(l2);
  int am = 0;
  for (int k = 1; k < 3; ++k)
    if (q[k] > q[am]) am = k;
  double inner = q[am] < 0 ? q[am] : 0.0;
  if (grad) {
    for (int k = 0; k < 3; ++k) grad[k] = 0.0;
    if (len > 0) {
      for (int k = 0; k < 3; ++k) grad[k] = sp[k] * mq[k] / len;
    } else {
      grad[am] = sp[am];
    }
  }
  return len + inner - box[6];
}

/* target shape of the loss: a rounded box (centre, half extents, radius) or a
 * union of spheres (n rows of centre xyz, radius) */
typedef struct {
  int kind;
  const double* data;
  int n;
} ftarget;

static double sdf_spheres(const double* sph, int n, const double p[3], double grad[3], int* arg) {
  double best = 1e300;
  int bi = 0;
  for (int i = 0; i < n; ++i) {
    const double* c = sph + 4 * i;
    double dx = p[0] - c[0], dy = p[1] - c[1], dz = p[2] - c[2];
    double d = sqrt(dx * dx + dy * dy + dz * dz) - c[3];
    if (d < best) {
      best = d;
      bi = i;
    }
  }
  const double* c = sph + 4 * bi;
  double r[3] = {p[0] - c[0], p[1] - c[1], p[2] - c[2]};
  double len = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
  for (int k = 0; k < 3; ++k) grad[k] = len > 0 ? r[k] / len : 0.0;
  *arg = bi;
  return best;
}

static double fit_loss(int dim, const double* density, int iters, ftarget tgt, double* grad_density,
                       int64_t* out_counts, uint64_t* state_hash, unsigned char* near_branch);

double bmfo_fit_loss_f64(int dim, const double* density, int iters, const double* box, double* grad_density,
                         int64_t* out_counts, uint64_t* state_hash, unsigned char* near_branch) {
  ftarget t = {0, box, 1};
  return fit_loss(dim, density, iters, t, grad_density, out_counts, state_hash, near_branch);
}

double bmfo_fit_loss_spheres_f64(int dim, const double* density, int iters, const double* spheres, int n_spheres,
                                 double* grad_density, int64_t* out_counts, uint64_t* state_hash,
                                 unsigned char* near_branch) {
  ftarget t = {1, spheres, n_spheres};
  return fit_loss(dim, density, iters, t, grad_density, out_counts, state_hash, near_branch);
}

/* A vertex whose placement branch the float32 forward (bmf_oracle.c, the
 * reference's float QEF) takes differently from this FP64 one: a different
 * QEF / mass-point choice, or, when the QEF is used, an eigenvalue within 10%
 * of the 1e-3 truncation threshold (float eigenvalues are off by ~1e-6). */
static int fit_near_branch(const fqef* Q, int qef64, int qef32) {
  if (qef64 != qef32) return 1;
  if (!qef64) return 0;
  for (int i = 0; i < 3; ++i) {
    double a = fabs(Q->w[i]);
    if (a >= 0.9e-3 && a <= 1.1e-3) return 1;
  }
  return 0;
}

/* the samples a hermite pair reads: both ends and their gradient stencils */
static void fit_mark_stencil(unsigned char* mask, int dim, const fherm* h) {
#define FIT_MARK(q) (mask[((size_t)(q)[0] * dim + (q)[1]) * dim + (q)[2]] = 1)
  FIT_MARK(h->a0);
  FIT_MARK(h->a1);
  for (int a = 0; a < 3; ++a) {
    FIT_MARK(h->lo0[a]);
    FIT_MARK(h->hi0[a]);
    FIT_MARK(h->lo1[a]);
    FIT_MARK(h->hi1[a]);
  }
#undef FIT_MARK
}

static double fit_loss(int dim, const double* density, int iters, ftarget tgt, double* grad_density,
                       int64_t* out_counts, uint64_t* state_hash, unsigned char* near_branch) {
  uint64_t hsh = 1469598103934665603ull;
  float* fdens = NULL; /* the samples as the float forward reads them */
  if (near_branch) {
    memset(near_branch, 0, (size_t)dim * dim * dim);
    fdens = (float*)malloc((size_t)dim * dim * dim * sizeof(float));
    for (size_t i = 0; i < (size_t)dim * dim * dim; ++i) fdens[i] = (float)density[i];
  }
#define FIT_HASH(v) (hsh = (hsh ^ (uint64_t)(v)) * 1099511628211ull)
  fgrid G = {dim, density};
  const int nc = dim - 1;
  const size_t ncell = (size_t)nc * nc * nc;
  int* vbase = (int*)malloc(ncell * sizeof(int));
  int* cmask = (int*)malloc(ncell * sizeof(int));
  size_t vcap = 1024, nv = 0;
  fvert* V = (fvert*)malloc(vcap * sizeof(fvert));
  /* vertices: interior surface cells in linear order, groups in table order */
  for (int x = 0; x < nc; ++x)
    for (int y = 0; y < nc; ++y)
      for (int z = 0; z < nc; ++z) {
        size_t c = ((size_t)x * nc + y) * nc + z;
        int m = 0;
        for (int k = 0; k < 8; ++k) m |= fin(&G, x + ((k >> 2) & 1), y + ((k >> 1) & 1), z + (k & 1)) << k;
        cmask[c] = m;
        FIT_HASH(m);
        vbase[c] = (int)nv;
        uint64_t gw = kBmfGroupCases[m];
        int ng = (int)((gw >> 48) & 0xF);
        for (int gi = 0; gi < ng; ++gi) {
          if (nv == vcap) {
            vcap *= 2;
            V = (fvert*)realloc(V, vcap * sizeof(fvert));
          }
          fvert* v = &V[nv++];
          v->cx = x; v->cy = y; v->cz = z; v->mask = m; v->group = gi; v->ne = 0;
          for (int e = 0; e < 12; ++e)
            if ((int)((gw >> (4 * e)) & 0xF) == gi) v->edges[v->ne++] = e;
        }
      }
  /* quads (Mode Q rule of bmf_oracle.c) */
  size_t qcap = 1024, nq = 0;
  int* Q4 = (int*)malloc(qcap * 4 * sizeof(int));
  static const int ob[4] = {-1, 0, 0, -1}, oc[4] = {-1, -1, 0, 0};
  for (int x = 0; x < dim; ++x)
    for (int y = 0; y < dim; ++y)
      for (int z = 0; z < dim; ++z) {
        int s[3] = {x, y, z};
        int in0 = fin(&G, x, y, z);
        for (int a = 0; a < 3; ++a) {
          int b = (a + 1) % 3, cc = (a + 2) % 3;
          if (s[a] > dim - 2 || s[b] < 1 || s[b] > dim - 2 || s[cc] < 1 || s[cc] > dim - 2) continue;
          int t[3] = {x, y, z};
          t[a]++;
          if (fin(&G, t[0], t[1], t[2]) == in0) continue;
          int q[4];
          for (int k = 0; k < 4; ++k) {
            int cl[3] = {x, y, z}, lo[3] = {0, 0, 0};
            cl[b] += ob[k]; cl[cc] += oc[k];
            lo[b] = -ob[k]; lo[cc] = -oc[k];
            int e = a == 0 ? 2 * lo[1] + lo[2] : (a == 1 ? 4 + 2 * lo[0] + lo[2] : 8 + 2 * lo[0] + lo[1]);
            size_t ci = ((size_t)cl[0] * nc + cl[1]) * nc + cl[2];
            q[k] = vbase[ci] + (int)((kBmfGroupCases[cmask[ci]] >> (4 * e)) & 0xF);
          }
          if (!in0) { int tmp = q[1]; q[1] = q[3]; q[3] = tmp; }
          if (nq == qcap) {
            qcap *= 2;
            Q4 = (int*)realloc(Q4, qcap * 4 * sizeof(int));
          }
          memcpy(Q4 + 4 * nq, q, sizeof(q));
          ++nq;
        }
      }
  /* placement */
  double* P = (double*)malloc((nv ? nv : 1) * 3 * sizeof(double));
  for (size_t i = 0; i < nv; ++i) {
    fvert* v = &V[i];
    fherm H[FIT_MAXE];
    double mp[3] = {0, 0, 0};
    for (int j = 0; j < v->ne; ++j) {
      fhermite(&G, v, v->edges[j], &H[j]);
      for (int k = 0; k < 3; ++k) mp[k] += H[j].p[k];
    }
    for (int k = 0; k < 3; ++k) mp[k] /= v->ne;
    v->qef = 0;
    if (v->ne >= 2 && v->ne <= 12) {
      fqef Qs;
      fqef_solve(H, v->ne, &Qs);
      double xs[3] = {Qs.y[0] + Qs.m[0], Qs.y[1] + Qs.m[1], Qs.y[2] + Qs.m[2]};
      int ok = xs[0] >= v->cx && xs[0] <= v->cx + 1 && xs[1] >= v->cy && xs[1] <= v->cy + 1 && xs[2] >= v->cz &&
               xs[2] <= v->cz + 1;
      if (ok) {
        v->qef = 1;
        memcpy(v->x, xs, sizeof(xs));
      }
      if (near_branch) {
        float o32[3];
        int q32 = bmfo_place_q_f32(dim, fdens, v->cx, v->cy, v->cz, v->mask, v->group, o32);
        if (fit_near_branch(&Qs, ok, q32))
          for (int j = 0; j < v->ne; ++j) fit_mark_stencil(near_branch, dim, &H[j]);
      }
      FIT_HASH((Qs.inv[0] != 0.0) | ((Qs.inv[1] != 0.0) << 1) | ((Qs.inv[2] != 0.0) << 2));
    }
    FIT_HASH(v->qef);
    if (!v->qef) memcpy(v->x, mp, sizeof(mp));
    memcpy(P + 3 * i, v->x, sizeof(v->x));
  }
  /* smoothing: valence, boundary, adjacency */
  int* val = (int*)calloc(nv ? nv : 1, sizeof(int));
  unsigned char* bnd = (unsigned char*)malloc(nv ? nv : 1);
  for (size_t q = 0; q < 4 * nq; ++q) val[Q4[q]]++;
  for (size_t i = 0; i < nv; ++i)
    bnd[i] = V[i].cx == 0 || V[i].cy == 0 || V[i].cz == 0 || V[i].cx == nc - 1 || V[i].cy == nc - 1 ||
             V[i].cz == nc - 1;
  double* D = (double*)malloc((nq ? nq : 1) * 3 * sizeof(double));
  double* Pn = (double*)malloc((nv ? nv : 1) * 3 * sizeof(double));
  for (int it = 0; it < iters; ++it) {
    for (size_t t = 0; t < nq; ++t)
      for (int k = 0; k < 3; ++k)
        D[3 * t + k] = (P[3 * Q4[4 * t] + k] + P[3 * Q4[4 * t + 1] + k] + P[3 * Q4[4 * t + 2] + k] +
                        P[3 * Q4[4 * t + 3] + k]) / 4.0;
    memcpy(Pn, P, nv * 3 * sizeof(double));
    for (size_t i = 0; i < nv; ++i)
      if (val[i] > 0 && !bnd[i]) Pn[3 * i] = Pn[3 * i + 1] = Pn[3 * i + 2] = 0.0;
    for (size_t t = 0; t < nq; ++t)
      for (int k = 0; k < 4; ++k) {
        int v = Q4[4 * t + k];
        if (val[v] > 0 && !bnd[v])
          for (int c = 0; c < 3; ++c) Pn[3 * v + c] += D[3 * t + c] / val[v];
      }
    memcpy(P, Pn, nv * 3 * sizeof(double));
  }
  /* loss */
  double loss = 0.0;
  double* gP = (double*)calloc((nv ? nv : 1) * 3, sizeof(double));
  for (size_t i = 0; i < nv; ++i) {
    double gr[3], d;
    if (tgt.kind == 0) {
      d = sdf_box(tgt.data, P + 3 * i, gr);
      /* the loss's own branch: which box faces are active */
      FIT_HASH((gr[0] != 0.0) | ((gr[1] != 0.0) << 1) | ((gr[2] != 0.0) << 2) | ((gr[0] < 0.0) << 3) |
               ((gr[1] < 0.0) << 4) | ((gr[2] < 0.0) << 5));
    } else {
      int arg;
      d = sdf_spheres(tgt.data, tgt.n, P + 3 * i, gr, &arg);
      FIT_HASH(arg); /* the loss's own branch: the nearest sphere */
    }
    loss += d * d;
    for (int k = 0; k < 3; ++k) gP[3 * i + k] = 2.0 * d * gr[k] / (double)nv;
  }
  if (nv) loss /= (double)nv;
  if (grad_density) {
    memset(grad_density, 0, (size_t)dim * dim * dim * sizeof(double));
    /* smoothing adjoint: primal^T then dual^T, last sweep first */
    double* gD = (double*)malloc((nq ? nq : 1) * 3 * sizeof(double));
    double* gprev = (double*)malloc((nv ? nv : 1) * 3 * sizeof(double));
    for (int it = iters - 1; it >= 0; --it) {
      for (size_t t = 0; t < nq; ++t)
        for (int c = 0; c < 3; ++c) {
          double s = 0.0;
          for (int k = 0; k < 4; ++k) {
            int v = Q4[4 * t + k];
            if (val[v] > 0 && !bnd[v]) s += gP[3 * v + c] / val[v];
          }
          gD[3 * t + c] = s;
        }
      for (size_t i = 0; i < nv; ++i)
        for (int c = 0; c < 3; ++c) gprev[3 * i + c] = (val[i] > 0 && !bnd[i]) ? 0.0 : gP[3 * i + c];
      for (size_t t = 0; t < nq; ++t)
        for (int k = 0; k < 4; ++k)
          for (int c = 0; c < 3; ++c) gprev[3 * Q4[4 * t + k] + c] += gD[3 * t + c] / 4.0;
      memcpy(gP, gprev, nv * 3 * sizeof(double));
    }
    free(gD);
    free(gprev);
    /* placement adjoint */
    for (size_t i = 0; i < nv; ++i) {
      fvert* v = &V[i];
      const double* gx = gP + 3 * i;
      fherm H[FIT_MAXE];
      for (int j = 0; j < v->ne; ++j) fhermite(&G, v, v->edges[j], &H[j]);
      double gp[FIT_MAXE][3], gn[FIT_MAXE][3];
      memset(gp, 0, sizeof(gp));
      memset(gn, 0, sizeof(gn));
      const int k = v->ne;
      if (!v->qef) {
        for (int j = 0; j < k; ++j)
          for (int c = 0; c < 3; ++c) gp[j][c] = gx[c] / k;
      } else {
        fqef Qs;
        fqef_solve(H, k, &Qs);
        double gm[3] = {gx[0], gx[1], gx[2]}, gy[3] = {gx[0], gx[1], gx[2]};
        double gr[3], gA[3][3], Gs[3][3], M[3][3], F[3][3];
        for (int r = 0; r < 3; ++r) {  /* g_r = P g_y */
          gr[r] = 0.0;
          for (int c = 0; c < 3; ++c) {
            double Pc = 0.0;
            for (int q = 0; q < 3; ++q) Pc += Qs.V[r][q] * Qs.inv[q] * Qs.V[c][q];
            gr[r] += Pc * gy[c];
          }
        }
        for (int r = 0; r < 3; ++r)  /* G = sym(g_y r^T) */
          for (int c = 0; c < 3; ++c) Gs[r][c] = 0.5 * (gy[r] * Qs.r[c] + gy[c] * Qs.r[r]);
        for (int a = 0; a < 3; ++a)  /* M = V^T G V */
          for (int b2 = 0; b2 < 3; ++b2) {
            double s = 0.0;
            for (int r = 0; r < 3; ++r)
              for (int c = 0; c < 3; ++c) s += Qs.V[r][a] * Gs[r][c] * Qs.V[c][b2];
            M[a][b2] = s;
          }
        for (int a = 0; a < 3; ++a)
          for (int b2 = 0; b2 < 3; ++b2) {
            double fa = Qs.inv[a], fb = Qs.inv[b2], sa = Qs.w[a], sb = Qs.w[b2];
            /* f(s) = 1/s: (f_a - f_b)/(s_a - s_b) = -f_a f_b, and f'(s) = -f^2;
             * a truncated eigenvalue (f = 0) beside a kept one: the quotient */
            if (fa != 0.0 && fb != 0.0)
              F[a][b2] = -fa * fb;
            else if (a == b2 || fabs(sa - sb) <= 1e-12 * (fabs(sa) + fabs(sb) + 1e-300))
              F[a][b2] = 0.0;
            else
              F[a][b2] = (fa - fb) / (sa - sb);
          }
        for (int r = 0; r < 3; ++r)  /* g_A = V (F o M) V^T - sym(g_r m^T) */
          for (int c = 0; c < 3; ++c) {
            double s = 0.0;
            for (int a = 0; a < 3; ++a)
              for (int b2 = 0; b2 < 3; ++b2) s += Qs.V[r][a] * F[a][b2] * M[a][b2] * Qs.V[c][b2];
            gA[r][c] = s - 0.5 * (gr[r] * Qs.m[c] + gr[c] * Qs.m[r]);
          }
        for (int r = 0; r < 3; ++r)  /* r = b - A m  ->  g_m -= A g_r */
          gm[r] -= Qs.A[r][0] * gr[0] + Qs.A[r][1] * gr[1] + Qs.A[r][2] * gr[2];
        for (int j = 0; j < k; ++j) {
          const double* n = H[j].n;
          const double* p = H[j].p;
          double d = n[0] * p[0] + n[1] * p[1] + n[2] * p[2];
          double gd = gr[0] * n[0] + gr[1] * n[1] + gr[2] * n[2];
          for (int c = 0; c < 3; ++c) {
            gn[j][c] += 2.0 * (gA[c][0] * n[0] + gA[c][1] * n[1] + gA[c][2] * n[2]);
            gn[j][c] += d * gr[c] + gd * p[c];
            gp[j][c] += gd * n[c] + gm[c] / k;
          }
        }
      }
      for (int j = 0; j < k; ++j) { /* hermite adjoint */
        fherm* h = &H[j];
        double ndot = h->n[0] * gn[j][0] + h->n[1] * gn[j][1] + h->n[2] * gn[j][2];
        double gG[3], gmu = gp[j][h->ax];
        for (int c = 0; c < 3; ++c) gG[c] = (gn[j][c] - h->n[c] * ndot) / h->Glen;
        for (int c = 0; c < 3; ++c) gmu += gG[c] * (h->g1[c] - h->g0[c]);
        double den = (h->s1 - h->s0) * (h->s1 - h->s0);
        double* gs = grad_density;
#define GIDX(q) (((size_t)(q)[0] * dim + (q)[1]) * dim + (q)[2])
        gs[GIDX(h->a0)] += gmu * (-h->s1 / den);
        gs[GIDX(h->a1)] += gmu * (h->s0 / den);
        for (int a = 0; a < 3; ++a) {
          double w0 = gG[a] * (1.0 - h->mu) * h->h0[a], w1 = gG[a] * h->mu * h->h1[a];
          gs[GIDX(h->hi0[a])] += w0;
          gs[GIDX(h->lo0[a])] -= w0;
          gs[GIDX(h->hi1[a])] += w1;
          gs[GIDX(h->lo1[a])] -= w1;
        }
#undef GIDX
      }
    }
  }
  if (state_hash) *state_hash = hsh;
#undef FIT_HASH
  if (out_counts) {
    out_counts[0] = (int64_t)nv;
    out_counts[1] = (int64_t)nq;
    int64_t nqef = 0;
    for (size_t i = 0; i < nv; ++i) nqef += V[i].qef;
    out_counts[2] = nqef;
  }
  free(vbase); free(cmask); free(V); free(Q4); free(P); free(val); free(bnd); free(D); free(Pn); free(gP);
  free(fdens);
  return loss;
}
