/*
 * nosh_oracle.c -- CPU FP64 restatement of nosh's NLS hot path.
 *
 * TEST INFRASTRUCTURE ONLY (parity oracle + timed CPU baseline); never part
 * of the product.  Each function names the reference file:line it restates.
 * Parity pins: tests/test_oracle_kat.py reproduces the constants of the
 * reference's own (disabled) rectangle / cube test cases.
 */
#define _GNU_SOURCE
#include "nosh_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* RNG: splitmix64 (Steele, Lea, Flood 2014).  The generator is part of the
 * synthetic-workload definition, not of the reference. */
uint64_t nor_splitmix64(uint64_t *state)
{
  uint64_t z = (*state += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

double nor_uniform(uint64_t *state, double lo, double hi)
{
  const double u = (double)(nor_splitmix64(state) >> 11) * 0x1.0p-53;
  return lo + (hi - lo) * u;
}

/* ------------------------------------------------------------------------ */
/* Synthetic meshes.  Interior vertices are jittered by U(-j*h, j*h) per
 * coordinate; boundary vertices only tangentially (a coordinate that sits on
 * the boundary is kept).  Draws happen in vertex-id order, one per
 * coordinate, whether used or not; psi draws follow the coordinate draws. */
void nor_gen_square(int s, uint64_t seed, double jitter, double *x,
                    int32_t *cells, double *psi)
{
  const double h = 1.0 / (double)(s - 1);
  uint64_t st = seed;
  for (int j = 0; j < s; j++) {
    for (int i = 0; i < s; i++) {
      const int64_t v = i + (int64_t)s * j;
      const double dx = nor_uniform(&st, -jitter * h, jitter * h);
      const double dy = nor_uniform(&st, -jitter * h, jitter * h);
      x[3 * v + 0] = i * h + ((i > 0 && i < s - 1) ? dx : 0.0);
      x[3 * v + 1] = j * h + ((j > 0 && j < s - 1) ? dy : 0.0);
      x[3 * v + 2] = 0.0;
    }
  }
  const int64_t N = (int64_t)s * s;
  for (int64_t v = 0; v < N; v++) {
    psi[2 * v + 0] = 1.0 + nor_uniform(&st, -0.01, 0.01);
    psi[2 * v + 1] = nor_uniform(&st, -0.01, 0.01);
  }
  int64_t c = 0;
  for (int j = 0; j < s - 1; j++) {
    for (int i = 0; i < s - 1; i++) {
      const int32_t v00 = i + s * j, v10 = v00 + 1, v01 = v00 + s,
                    v11 = v01 + 1;
      cells[3 * c + 0] = v00; cells[3 * c + 1] = v10; cells[3 * c + 2] = v11;
      c++;
      cells[3 * c + 0] = v00; cells[3 * c + 1] = v11; cells[3 * c + 2] = v01;
      c++;
    }
  }
}

void nor_gen_cube(int m, uint64_t seed, double jitter, double *x,
                  int32_t *cells, double *psi)
{
  const int n = m + 1;
  const double h = 1.0 / (double)m;
  uint64_t st = seed;
  for (int k = 0; k < n; k++)
    for (int j = 0; j < n; j++)
      for (int i = 0; i < n; i++) {
        const int64_t v = i + (int64_t)n * (j + (int64_t)n * k);
        const double dx = nor_uniform(&st, -jitter * h, jitter * h);
        const double dy = nor_uniform(&st, -jitter * h, jitter * h);
        const double dz = nor_uniform(&st, -jitter * h, jitter * h);
        x[3 * v + 0] = i * h + ((i > 0 && i < m) ? dx : 0.0);
        x[3 * v + 1] = j * h + ((j > 0 && j < m) ? dy : 0.0);
        x[3 * v + 2] = k * h + ((k > 0 && k < m) ? dz : 0.0);
      }
  const int64_t N = (int64_t)n * n * n;
  for (int64_t v = 0; v < N; v++) {
    psi[2 * v + 0] = 1.0 + nor_uniform(&st, -0.01, 0.01);
    psi[2 * v + 1] = nor_uniform(&st, -0.01, 0.01);
  }
  /* Kuhn split: one tet per axis permutation, walking 000 -> 111. */
  static const int perm[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2},
                                 {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
  int64_t c = 0;
  for (int k = 0; k < m; k++)
    for (int j = 0; j < m; j++)
      for (int i = 0; i < m; i++)
        for (int p = 0; p < 6; p++) {
          int o[3] = {0, 0, 0};
          int32_t *t = cells + 4 * c;
          t[0] = i + n * (j + n * k);
          for (int s2 = 0; s2 < 2; s2++) {
            o[perm[p][s2]] = 1;
            t[1 + s2] = (i + o[0]) + n * ((j + o[1]) + n * (k + o[2]));
          }
          t[3] = (i + 1) + n * ((j + 1) + n * (k + 1));
          c++;
        }
}

/* ------------------------------------------------------------------------ */
/* Edges.  Restates mesh::build_entity_relations_ (src/mesh.cpp:631-691):
 * unique vertex pairs of all cells plus the cell->edge relation.  MOAB's
 * entity order is unavailable, so edges are the canonical sorted (v0<v1)
 * pairs in lexicographic order; orientation v0->v1. */
static const int TRI_PAIRS[3][2] = {{0, 1}, {0, 2}, {1, 2}};
static const int TET_PAIRS[6][2] = {{0, 1}, {0, 2}, {0, 3},
                                    {1, 2}, {1, 3}, {2, 3}};

int64_t nor_build_edges(int nvc, int64_t N, int64_t T, const int32_t *cells,
                        int32_t *edges, int32_t *cell_edges)
{
  const int ne = (nvc == 3) ? 3 : 6;
  const int(*pairs)[2] = (nvc == 3) ? TRI_PAIRS : TET_PAIRS;
  const int64_t M = T * ne;
  int64_t *cnt = (int64_t *)calloc((size_t)N + 1, sizeof(int64_t));
  int32_t *hi = (int32_t *)malloc((size_t)M * sizeof(int32_t));
  int64_t *slot = (int64_t *)malloc((size_t)M * sizeof(int64_t));
  for (int64_t c = 0; c < T; c++)
    for (int k = 0; k < ne; k++) {
      int32_t a = cells[nvc * c + pairs[k][0]], b = cells[nvc * c + pairs[k][1]];
      cnt[(a < b ? a : b) + 1]++;
    }
  for (int64_t i = 0; i < N; i++) cnt[i + 1] += cnt[i];
  int64_t *pos = (int64_t *)malloc((size_t)N * sizeof(int64_t));
  memcpy(pos, cnt, (size_t)N * sizeof(int64_t));
  for (int64_t c = 0; c < T; c++)
    for (int k = 0; k < ne; k++) {
      int32_t a = cells[nvc * c + pairs[k][0]], b = cells[nvc * c + pairs[k][1]];
      int32_t lo = a < b ? a : b, h = a < b ? b : a;
      int64_t q = pos[lo]++;
      hi[q] = h;
      slot[q] = c * ne + k;
    }
  int64_t E = 0;
  for (int64_t v = 0; v < N; v++) {
    /* insertion sort of the bucket by hi, ties by slot */
    for (int64_t q = cnt[v] + 1; q < cnt[v + 1]; q++) {
      int32_t hk = hi[q];
      int64_t sk = slot[q];
      int64_t r = q - 1;
      while (r >= cnt[v] && (hi[r] > hk || (hi[r] == hk && slot[r] > sk))) {
        hi[r + 1] = hi[r];
        slot[r + 1] = slot[r];
        r--;
      }
      hi[r + 1] = hk;
      slot[r + 1] = sk;
    }
    for (int64_t q = cnt[v]; q < cnt[v + 1]; q++) {
      if (q == cnt[v] || hi[q] != hi[q - 1]) {
        edges[2 * E + 0] = (int32_t)v;
        edges[2 * E + 1] = hi[q];
        E++;
      }
      cell_edges[slot[q]] = (int32_t)(E - 1);
    }
  }
  free(cnt);
  free(hi);
  free(slot);
  free(pos);
  return E;
}

/* Complex graph: restates mesh::build_complex_graph (src/mesh.cpp:789-882):
 * for every edge all 4x4 (complex: 2x2) index pairs are inserted, then
 * fillComplete sorts each row's columns.  Row i = {i} u neighbours(i). */
void nor_complex_graph(int64_t N, int64_t E, const int32_t *edges,
                       int32_t *row_ptr, int32_t *cols)
{
  int32_t *deg = (int32_t *)calloc((size_t)N, sizeof(int32_t));
  for (int64_t e = 0; e < E; e++) {
    deg[edges[2 * e]]++;
    deg[edges[2 * e + 1]]++;
  }
  row_ptr[0] = 0;
  for (int64_t i = 0; i < N; i++) row_ptr[i + 1] = row_ptr[i] + deg[i] + 1;
  int32_t *fill = (int32_t *)malloc((size_t)N * sizeof(int32_t));
  for (int64_t i = 0; i < N; i++) {
    cols[row_ptr[i]] = (int32_t)i;
    fill[i] = row_ptr[i] + 1;
  }
  for (int64_t e = 0; e < E; e++) {
    int32_t a = edges[2 * e], b = edges[2 * e + 1];
    cols[fill[a]++] = b;
    cols[fill[b]++] = a;
  }
  for (int64_t i = 0; i < N; i++) {
    for (int32_t q = row_ptr[i] + 1; q < row_ptr[i + 1]; q++) {
      int32_t k = cols[q], r = q - 1;
      while (r >= row_ptr[i] && cols[r] > k) {
        cols[r + 1] = cols[r];
        r--;
      }
      cols[r + 1] = k;
    }
  }
  free(deg);
  free(fill);
}

/* ------------------------------------------------------------------------ */
/* small vector helpers */
static inline void sub3(const double *a, const double *b, double *r)
{
  r[0] = a[0] - b[0]; r[1] = a[1] - b[1]; r[2] = a[2] - b[2];
}
static inline double dot3(const double *a, const double *b)
{
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
static inline void cross3(const double *a, const double *b, double *r)
{
  r[0] = a[1] * b[2] - a[2] * b[1];
  r[1] = a[2] * b[0] - a[0] * b[2];
  r[2] = a[0] * b[1] - a[1] * b[0];
}
static inline double norm3(const double *a) { return sqrt(dot3(a, a)); }

/* Dense solve with partial pivoting (n <= 6).  Eigen's fullPivLu gives the
 * same solution to roundoff for these SPD systems. */
static void dense_solve(int n, double *A, double *b, double *x)
{
  int piv[6];
  for (int i = 0; i < n; i++) piv[i] = i;
  for (int k = 0; k < n; k++) {
    int p = k;
    double best = fabs(A[piv[k] * n + k]);
    for (int i = k + 1; i < n; i++)
      if (fabs(A[piv[i] * n + k]) > best) {
        best = fabs(A[piv[i] * n + k]);
        p = i;
      }
    int t = piv[k]; piv[k] = piv[p]; piv[p] = t;
    const double *rk = A + piv[k] * n;
    for (int i = k + 1; i < n; i++) {
      double *ri = A + piv[i] * n;
      const double f = ri[k] / rk[k];
      ri[k] = f;
      for (int j = k + 1; j < n; j++) ri[j] -= f * rk[j];
      b[piv[i]] -= f * b[piv[k]];
    }
  }
  for (int k = n - 1; k >= 0; k--) {
    const double *rk = A + piv[k] * n;
    double s = b[piv[k]];
    for (int j = k + 1; j < n; j++) s -= rk[j] * x[j];
    x[k] = s / rk[k];
  }
}

/* Edge coefficients of one simplex: solve
 *   sum_j (e_i.e_j)^2 c_j = |simplex| |e_i|^2
 * (src/mesh_tri.cpp:107-151, src/mesh_tetra.cpp:107-160). */
static void edge_coefficients(int ne, const double (*ev)[3], double vol,
                              double *coef)
{
  double A[36], rhs[6];
  for (int i = 0; i < ne; i++) {
    const double a = dot3(ev[i], ev[i]);
    rhs[i] = vol * a;
    A[i * ne + i] = a * a;
    for (int j = i + 1; j < ne; j++) {
      const double d = dot3(ev[i], ev[j]);
      A[i * ne + j] = d * d;
      A[j * ne + i] = d * d;
    }
  }
  dense_solve(ne, A, rhs, coef);
}

/* Edge lengths and covolumes: mesh_tri::compute_edge_data_
 * (src/mesh_tri.cpp:46-103) and mesh_tetra::compute_edge_data_
 * (src/mesh_tetra.cpp:43-103): covolume[e] += coeff * length over cells. */
void nor_edge_data(int nvc, int64_t N, const double *x, int64_t E,
                   const int32_t *edges, int64_t T, const int32_t *cell_edges,
                   double *length, double *covolume)
{
  (void)N;
  const int ne = (nvc == 3) ? 3 : 6;
  double (*ecoords)[3] = (double(*)[3])malloc((size_t)E * sizeof(double[3]));
  for (int64_t e = 0; e < E; e++) {
    sub3(x + 3 * edges[2 * e], x + 3 * edges[2 * e + 1], ecoords[e]);
    length[e] = norm3(ecoords[e]);
    covolume[e] = 0.0;
  }
  for (int64_t c = 0; c < T; c++) {
    double ev[6][3], coef[6];
    for (int k = 0; k < ne; k++) {
      const double *s = ecoords[cell_edges[ne * c + k]];
      ev[k][0] = s[0]; ev[k][1] = s[1]; ev[k][2] = s[2];
    }
    double vol;
    if (ne == 3) {
      /* 0.5 |e0 x e1| (src/mesh_tri.cpp:121) */
      double cr[3];
      cross3(ev[0], ev[1], cr);
      vol = 0.5 * norm3(cr);
    } else {
      /* |e_a . (e_b x e_c)| / 6 over three non-coplanar edges
       * (src/mesh_tetra.cpp:120-128, 353-373).  Local edges 0,1,2 share
       * local vertex 0, so they are never coplanar. */
      double cr[3];
      cross3(ev[1], ev[2], cr);
      vol = fabs(dot3(ev[0], cr)) / 6.0;
    }
    edge_coefficients(ne, (const double(*)[3])ev, vol, coef);
    for (int k = 0; k < ne; k++) {
      const int32_t e = cell_edges[ne * c + k];
      covolume[e] += coef[k] * length[e];
    }
  }
  free(ecoords);
}

/* Triangle circumcenter (src/mesh.cpp:897-928). */
static void tri_circumcenter(const double *n0, const double *n1,
                             const double *n2, double *cc)
{
  double a[3], b[3], c[3], ab[3];
  sub3(n0, n1, a);
  sub3(n1, n2, b);
  sub3(n2, n0, c);
  cross3(a, b, ab);
  const double omega = 2.0 * dot3(ab, ab);
  const double al = -dot3(b, b) * dot3(a, c) / omega;
  const double be = -dot3(c, c) * dot3(b, a) / omega;
  const double ga = -dot3(a, a) * dot3(c, b) / omega;
  for (int k = 0; k < 3; k++) cc[k] = al * n0[k] + be * n1[k] + ga * n2[k];
}

/* Signed 2-D covolume (src/mesh.cpp:1005-1027). */
static double covolume2d(const double *cc, const double *x0, const double *x1,
                         const double *o0)
{
  double mp[3], d[3], u[3], v[3], w[3], cn[3], ccn[3];
  for (int k = 0; k < 3; k++) mp[k] = 0.5 * (x0[k] + x1[k]);
  sub3(mp, cc, d);
  const double len = norm3(d);
  sub3(o0, x0, u);
  sub3(mp, x0, v);
  cross3(u, v, cn);
  sub3(cc, x0, w);
  cross3(w, v, ccn);
  return copysign(len, dot3(ccn, cn));
}

/* Tetrahedron circumcenter (src/mesh_tetra.cpp:377-415). */
static void tet_circumcenter(const double (*v)[3], double *cc)
{
  double r0[3], r1[3], r2[3], c12[3], c20[3], c01[3];
  sub3(v[1], v[0], r0);
  sub3(v[2], v[0], r1);
  sub3(v[3], v[0], r2);
  cross3(r1, r2, c12);
  cross3(r2, r0, c20);
  cross3(r0, r1, c01);
  const double omega = 2.0 * dot3(r0, c12);
  const double al = dot3(r0, r0) / omega, be = dot3(r1, r1) / omega,
               ga = dot3(r2, r2) / omega;
  for (int k = 0; k < 3; k++)
    cc[k] = v[0][k] + al * c12[k] + be * c20[k] + ga * c01[k];
}

/* Signed 3-D covolume of one tet edge (src/mesh_tetra.cpp:275-331). */
static double covolume3d(const double *cc, const double *x0, const double *x1,
                         const double *o0, const double *o1)
{
  double mp[3], f0[3], f1[3], a[3], b[3], gauge[3], t[3], n[3];
  for (int k = 0; k < 3; k++) mp[k] = 0.5 * (x0[k] + x1[k]);
  tri_circumcenter(x0, x1, o0, f0);
  tri_circumcenter(x0, x1, o1, f1);
  sub3(o0, mp, a);
  sub3(o1, mp, b);
  cross3(a, b, gauge);
  double cov = 0.0;
  sub3(mp, f0, t);
  double h0 = norm3(t);
  sub3(f0, cc, t);
  double area0 = 0.5 * h0 * norm3(t);
  sub3(f0, mp, a);
  sub3(cc, mp, b);
  cross3(a, b, n);
  cov += copysign(area0, dot3(n, gauge));
  sub3(mp, f1, t);
  double h1 = norm3(t);
  sub3(f1, cc, t);
  double area1 = 0.5 * h1 * norm3(t);
  sub3(cc, mp, a);
  sub3(f1, mp, b);
  cross3(a, b, n);
  cov += copysign(area1, dot3(n, gauge));
  return cov;
}

/* Control volumes: mesh::compute_triangle_splitting_ (src/mesh.cpp:931-986)
 * with mesh_tri::compute_control_volumes_t_ (src/mesh_tri.cpp:187-210), and
 * mesh_tetra::compute_control_volumes_t_ (src/mesh_tetra.cpp:196-271). */
void nor_control_volumes(int nvc, int64_t N, const double *x, int64_t T,
                         const int32_t *cells, double *cv)
{
  for (int64_t i = 0; i < N; i++) cv[i] = 0.0;
  for (int64_t c = 0; c < T; c++) {
    const int32_t *cn = cells + nvc * c;
    double v[4][3];
    for (int k = 0; k < nvc; k++)
      for (int d = 0; d < 3; d++) v[k][d] = x[3 * cn[k] + d];
    double cc[3];
    if (nvc == 3) {
      tri_circumcenter(v[0], v[1], v[2], cc);
      for (int e0 = 0; e0 < 3; e0++)
        for (int e1 = e0 + 1; e1 < 3; e1++) {
          const int other = 3 - e0 - e1;
          double d[3];
          sub3(v[e1], v[e0], d);
          const double len = norm3(d);
          const double cov = covolume2d(cc, v[e0], v[e1], v[other]);
          const double pyr = 0.5 * len * cov / 2;
          cv[cn[e0]] += pyr;
          cv[cn[e1]] += pyr;
        }
    } else {
      tet_circumcenter((const double(*)[3])v, cc);
      for (int e0 = 0; e0 < 4; e0++)
        for (int e1 = e0 + 1; e1 < 4; e1++) {
          int o[2], no = 0;
          for (int k = 0; k < 4; k++)
            if (k != e0 && k != e1) o[no++] = k;
          double d[3];
          sub3(v[e1], v[e0], d);
          const double len = norm3(d);
          const double cov = covolume3d(cc, v[e0], v[e1], v[o[0]], v[o[1]]);
          const double pyr = 0.5 * len * cov / 3;
          cv[cn[e0]] += pyr;
          cv[cn[e1]] += pyr;
        }
    }
  }
}

/* Edge projection of an explicit vector field sampled per vertex:
 * p_e = 1/2 (A(x0) + A(x1)) . (x0 - x1)
 * (src/vector_field_explicit_values.cpp:14-50). */
void nor_edge_projection(int64_t E, const int32_t *edges, const double *x,
                         const double *A, double *p)
{
  for (int64_t e = 0; e < E; e++) {
    const int32_t a = edges[2 * e], b = edges[2 * e + 1];
    double av[3], d[3];
    for (int k = 0; k < 3; k++) av[k] = 0.5 * (A[3 * a + k] + A[3 * b + k]);
    sub3(x + 3 * a, x + 3 * b, d);
    p[e] = dot3(av, d);
  }
}

/* alpha_e = covolume/length * mean thickness
 * (keo::build_alpha_cache_, src/parameter_matrix_keo.cpp:221-228). */
void nor_alpha(int64_t E, const int32_t *edges, const double *length,
               const double *covolume, const double *thickness, double *alpha)
{
  for (int64_t e = 0; e < E; e++)
    alpha[e] = covolume[e] / length[e] * 0.5 *
               (thickness[edges[2 * e]] + thickness[edges[2 * e + 1]]);
}

/* ------------------------------------------------------------------------ */
static int64_t find_col(const int32_t *row_ptr, const int32_t *cols, int32_t r,
                        int32_t c)
{
  int32_t lo = row_ptr[r], hi = row_ptr[r + 1] - 1;
  while (lo <= hi) {
    int32_t mid = (lo + hi) / 2;
    if (cols[mid] == c) return mid;
    if (cols[mid] < c) lo = mid + 1;
    else hi = mid - 1;
  }
  return -1;
}

/* KEO values in the complex graph: keo::refill_
 * (src/parameter_matrix_keo.cpp:106-180).  Per edge v0->v1 with
 * a = mu*p_e: block (v0,v1) = [[v0,v1],[-v1,v0]] with v0=-alpha cos a,
 * v1=-alpha sin a, i.e. complex -alpha e^{-ia}; block (v1,v0) is its
 * transpose (the conjugate); +alpha on both diagonal blocks. */
void nor_keo_values(int64_t N, int64_t E, const int32_t *edges,
                    const double *alpha, const double *p, double mu,
                    const int32_t *row_ptr, const int32_t *cols, double *vals)
{
  memset(vals, 0, sizeof(double) * 2 * (size_t)row_ptr[N]);
  for (int64_t e = 0; e < E; e++) {
    const int32_t a = edges[2 * e], b = edges[2 * e + 1];
    double s, c;
    sincos(mu * p[e], &s, &c);
    const double v0 = -c * alpha[e], v1 = -s * alpha[e];
    int64_t q = find_col(row_ptr, cols, a, b);
    vals[2 * q] += v0;
    vals[2 * q + 1] += -v1;
    q = find_col(row_ptr, cols, b, a);
    vals[2 * q] += v0;
    vals[2 * q + 1] += v1;
    q = find_col(row_ptr, cols, a, a);
    vals[2 * q] += alpha[e];
    q = find_col(row_ptr, cols, b, b);
    vals[2 * q] += alpha[e];
  }
}

/* dK/dp values: DkeoDP::refill_ (src/parameter_matrix_dkeo_dp.cpp:96-151):
 * v0 = alpha dp sin a, v1 = -alpha dp cos a, zero diagonal. */
void nor_dkeo_values(int64_t N, int64_t E, const int32_t *edges,
                     const double *alpha, const double *p, const double *dp,
                     double mu, const int32_t *row_ptr, const int32_t *cols,
                     double *vals)
{
  memset(vals, 0, sizeof(double) * 2 * (size_t)row_ptr[N]);
  for (int64_t e = 0; e < E; e++) {
    const int32_t a = edges[2 * e], b = edges[2 * e + 1];
    double s, c;
    sincos(mu * p[e], &s, &c);
    const double v0 = dp[e] * s * alpha[e], v1 = -dp[e] * c * alpha[e];
    int64_t q = find_col(row_ptr, cols, a, b);
    vals[2 * q] += v0;
    vals[2 * q + 1] += -v1;
    q = find_col(row_ptr, cols, b, a);
    vals[2 * q] += v0;
    vals[2 * q + 1] += v1;
  }
}

/* y = K x, edge by edge (the 4x4 real block of keo::refill_ applied). */
void nor_keo_apply(int64_t N, int64_t E, const int32_t *edges,
                   const double *alpha, const double *p, double mu,
                   const double *x, double *y)
{
  memset(y, 0, sizeof(double) * 2 * (size_t)N);
  for (int64_t e = 0; e < E; e++) {
    const int32_t a = edges[2 * e], b = edges[2 * e + 1];
    double s, c;
    sincos(mu * p[e], &s, &c);
    const double v0 = -c * alpha[e], v1 = -s * alpha[e], al = alpha[e];
    const double xar = x[2 * a], xai = x[2 * a + 1];
    const double xbr = x[2 * b], xbi = x[2 * b + 1];
    /* rows of the 4x4 block (src/parameter_matrix_keo.cpp:155-160) */
    y[2 * a] += al * xar + v0 * xbr + v1 * xbi;
    y[2 * a + 1] += al * xai - v1 * xbr + v0 * xbi;
    y[2 * b] += v0 * xar - v1 * xai + al * xbr;
    y[2 * b + 1] += v1 * xar + v0 * xai + al * xbi;
  }
}

void nor_dkeo_apply(int64_t N, int64_t E, const int32_t *edges,
                    const double *alpha, const double *p, const double *dp,
                    double mu, const double *x, double *y)
{
  memset(y, 0, sizeof(double) * 2 * (size_t)N);
  for (int64_t e = 0; e < E; e++) {
    const int32_t a = edges[2 * e], b = edges[2 * e + 1];
    double s, c;
    sincos(mu * p[e], &s, &c);
    const double v0 = dp[e] * s * alpha[e], v1 = -dp[e] * c * alpha[e];
    const double xar = x[2 * a], xai = x[2 * a + 1];
    const double xbr = x[2 * b], xbi = x[2 * b + 1];
    y[2 * a] += v0 * xbr + v1 * xbi;
    y[2 * a + 1] += -v1 * xbr + v0 * xbi;
    y[2 * b] += v0 * xar - v1 * xai;
    y[2 * b + 1] += v1 * xar + v0 * xai;
  }
}

/* F(psi) = K psi + cv t (V + g|psi|^2) psi
 * (nls::compute_f_, src/model_evaluator_nls.cpp:536-625). */
void nor_compute_f(int64_t N, int64_t E, const int32_t *edges,
                   const double *alpha, const double *p, double mu, double g,
                   const double *cv, const double *t, const double *V,
                   const double *psi, double *f)
{
  nor_keo_apply(N, E, edges, alpha, p, mu, psi, f);
  for (int64_t k = 0; k < N; k++) {
    const double re = psi[2 * k], im = psi[2 * k + 1];
    const double a = cv[k] * t[k] * (V[k] + g * (re * re + im * im));
    f[2 * k] += a * re;
    f[2 * k + 1] += a * im;
  }
}

/* dF/dp (nls::computeDFDP_, src/model_evaluator_nls.cpp:632-695):
 * (dK/dp*) psi for the DkeoDP derivative parameter p*, plus
 * cv t |psi|^2 psi when p is "g", else cv t dV/dp psi. */
void nor_dfdp(int64_t N, int64_t E, const int32_t *edges, const double *alpha,
              const double *p, const double *dp, double mu, int param_is_g,
              const double *cv, const double *t, const double *dVdp,
              const double *psi, double *out)
{
  nor_dkeo_apply(N, E, edges, alpha, p, dp, mu, psi, out);
  for (int64_t k = 0; k < N; k++) {
    const double re = psi[2 * k], im = psi[2 * k + 1];
    const double a = param_is_g ? cv[k] * t[k] * (re * re + im * im)
                                : cv[k] * t[k] * dVdp[k];
    out[2 * k] += a * re;
    out[2 * k + 1] += a * im;
  }
}

/* jacobian_operator::rebuild_diags_ (src/jacobian_operator.cpp:184-197). */
void nor_jac_diags(int64_t N, const double *cv, const double *t,
                   const double *V, double g, const double *psi, double *d0,
                   double *d1b)
{
  for (int64_t k = 0; k < N; k++) {
    const double re = psi[2 * k], im = psi[2 * k + 1];
    const double al = cv[k] * t[k] * (V[k] + g * 2.0 * (re * re + im * im));
    const double rx2 = g * cv[k] * t[k] * (re * re - im * im);
    d0[2 * k] = al + rx2;
    d0[2 * k + 1] = al - rx2;
    d1b[k] = g * cv[k] * t[k] * (2.0 * re * im);
  }
}

/* jacobian_operator::apply (src/jacobian_operator.cpp:65-100). */
void nor_jac_apply(int64_t N, int64_t E, const int32_t *edges,
                   const double *alpha, const double *p, double mu,
                   const double *d0, const double *d1b, const double *x,
                   double *y)
{
  nor_keo_apply(N, E, edges, alpha, p, mu, x, y);
  for (int64_t k = 0; k < N; k++) {
    y[2 * k] += d0[2 * k] * x[2 * k] + d1b[k] * x[2 * k + 1];
    y[2 * k + 1] += d1b[k] * x[2 * k] + d0[2 * k + 1] * x[2 * k + 1];
  }
}

/* Regularized KEO: keo_regularized::rebuild (src/keo_regularized.cpp:
 * 196-258): K + g cv t [[2|psi|^2+gamma, beta],[beta, 2|psi|^2-gamma]]
 * (only when g > 0). */
void nor_kreg_apply(int64_t N, int64_t E, const int32_t *edges,
                    const double *alpha, const double *p, double mu, double g,
                    const double *cv, const double *t, const double *psi,
                    const double *x, double *y)
{
  nor_keo_apply(N, E, edges, alpha, p, mu, x, y);
  if (!(g > 0.0)) return;
  for (int64_t k = 0; k < N; k++) {
    const double re = psi[2 * k], im = psi[2 * k + 1];
    const double w = g * cv[k] * t[k];
    const double al = w * 2.0 * (re * re + im * im);
    const double be = w * (2.0 * re * im);
    const double ga = w * (re * re - im * im);
    y[2 * k] += (al + ga) * x[2 * k] + be * x[2 * k + 1];
    y[2 * k + 1] += be * x[2 * k] + (al - ga) * x[2 * k + 1];
  }
}

/* Free energy -sum cv|psi|^4 / sum cv: the value nls::gibbs_energy
 * (src/model_evaluator_nls.cpp:742-770) computes before its normalisation
 * (commented out there) and its `return 0.0`. */
double nor_energy(int64_t N, const double *cv, const double *psi)
{
  double e = 0.0, s = 0.0;
  for (int64_t k = 0; k < N; k++) {
    const double a = psi[2 * k] * psi[2 * k] + psi[2 * k + 1] * psi[2 * k + 1];
    e -= cv[k] * a * a;
    s += cv[k];
  }
  return e / s;
}

/* sum cv (Re phi Re psi + Im phi Im psi) / sum cv
 * (nls::inner_product, src/model_evaluator_nls.cpp:699-738). */
double nor_inner_product(int64_t N, const double *cv, const double *phi,
                         const double *psi)
{
  double r = 0.0, s = 0.0;
  for (int64_t k = 0; k < N; k++) {
    r += cv[k] * (phi[2 * k] * psi[2 * k] + phi[2 * k + 1] * psi[2 * k + 1]);
    s += cv[k];
  }
  return r / s;
}
