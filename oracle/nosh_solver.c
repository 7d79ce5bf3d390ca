/*
 * nosh_solver.c -- CPU FP64 Newton / preconditioned-MINRES / natural
 * continuation for the NLS problem, OpenMP over the host cores.
 *
 * TEST INFRASTRUCTURE ONLY: the timed CPU baseline (bench.py's reference arm
 * and cpu_baseline) and the oracle for the unpinned solver parts.  The
 * reference's own path (Belos MINRES + MueLu SA-AMG + NOX/LOCA, Trilinos)
 * cannot be built here; this restates the same algorithmic roles:
 *   - operators: KEO (src/parameter_matrix_keo.cpp:106-180), F
 *     (src/model_evaluator_nls.cpp:574-625), Jacobian diagonal blocks
 *     (src/jacobian_operator.cpp:184-197), regularised KEO
 *     (src/keo_regularized.cpp:233-258), all in complex-block CSR;
 *   - preconditioner: one V-cycle of a plain-aggregation AMG on the
 *     regularised KEO (the reference: one MueLu V-cycle,
 *     src/keo_regularized.cpp:106-108), block-Jacobi Chebyshev smoothing,
 *     dense coarse inverse;
 *   - MINRES (Paige-Saunders), full-step Newton with Eisenstat-Walker
 *     forcing (NOX, examples/conf.xml:77-191);
 *   - natural continuation with a phase-aligned secant predictor (LOCA,
 *     examples/conf.xml:35-75).
 */
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "nosh_oracle.h"

typedef struct {
  int64_t n, nnz;
  int32_t *rp, *ci;     /* off-diagonal CSR */
  double *off;          /* 2 per nonzero (complex) */
  double *dia;          /* 3 per node (d0r, d0i, d1b) */
  double *dinv;         /* 3 per node */
  double coef[8];       /* Chebyshev */
  /* transfer to the next level */
  int32_t *agg, *mem_ptr, *mem_idx, *seg_ptr, *seg_idx, *intra_ptr, *intra_idx;
  double *b, *x, *x2, *d, *res;
  double *dense; /* coarsest: inverse (2n)^2 */
} level_t;

typedef struct nor_solver {
  int64_t N, E;
  int32_t *rp, *ci;     /* fine off-diagonal CSR */
  int32_t *nz_edge;     /* edge of each nonzero (~e when the row is v1) */
  double *alpha, *p, *cv, *t, *V, *kdiag;
  double g, mu_keo;
  double *keo;          /* fine off-diagonal complex values */
  double *jd, *rd;      /* Jacobian / regularised diagonal blocks */
  int nlev;
  level_t lev[16];
  int deg;
  /* work */
  double *f, *b, *r1, *r2, *z0, *z1, *u, *w0, *w1, *w2, *dx, *xc, *xp;
} nor_solver;

static void *xcalloc(size_t n, size_t s) { return calloc(n ? n : 1, s); }

/* ---------------------------------------------------------------- setup */
nor_solver *nor_solver_create(int64_t N, int64_t E, const int32_t *edges, const double *alpha,
                              const double *p, const double *cv, const double *t, const double *V,
                              double g)
{
  nor_solver *s = (nor_solver *)xcalloc(1, sizeof(nor_solver));
  s->N = N; s->E = E; s->g = g; s->mu_keo = NAN; s->deg = 2;
  s->rp = (int32_t *)xcalloc(N + 1, 4);
  s->ci = (int32_t *)xcalloc(2 * E, 4);
  s->nz_edge = (int32_t *)xcalloc(2 * E, 4);
  int32_t *deg = (int32_t *)xcalloc(N, 4);
  for (int64_t e = 0; e < E; e++) { deg[edges[2 * e]]++; deg[edges[2 * e + 1]]++; }
  for (int64_t i = 0; i < N; i++) s->rp[i + 1] = s->rp[i] + deg[i];
  int32_t *fill = (int32_t *)xcalloc(N, 4);
  for (int64_t i = 0; i < N; i++) fill[i] = s->rp[i];
  /* edges are lexicographic: each row receives its lower neighbours in
   * increasing order first (as v1), then its upper ones (as v0) */
  for (int64_t e = 0; e < E; e++) {
    const int32_t a = edges[2 * e], b = edges[2 * e + 1];
    s->ci[fill[b]] = a; s->nz_edge[fill[b]++] = ~(int32_t)e;
  }
  for (int64_t e = 0; e < E; e++) {
    const int32_t a = edges[2 * e], b = edges[2 * e + 1];
    s->ci[fill[a]] = b; s->nz_edge[fill[a]++] = (int32_t)e;
  }
  free(deg); free(fill);
  size_t nb = sizeof(double);
  s->alpha = (double *)xcalloc(E, nb); memcpy(s->alpha, alpha, E * nb);
  s->p = (double *)xcalloc(E, nb); memcpy(s->p, p, E * nb);
  s->cv = (double *)xcalloc(N, nb); memcpy(s->cv, cv, N * nb);
  s->t = (double *)xcalloc(N, nb); memcpy(s->t, t, N * nb);
  s->V = (double *)xcalloc(N, nb); memcpy(s->V, V, N * nb);
  s->kdiag = (double *)xcalloc(N, nb);
  for (int64_t i = 0; i < N; i++) {
    double a = 0.0;
    for (int32_t k = s->rp[i]; k < s->rp[i + 1]; k++) {
      const int32_t e = s->nz_edge[k];
      a += alpha[e >= 0 ? e : ~e];
    }
    s->kdiag[i] = a;
  }
  s->keo = (double *)xcalloc(4 * E, nb);
  s->jd = (double *)xcalloc(3 * N, nb);
  s->rd = (double *)xcalloc(3 * N, nb);
  double **w[] = {&s->f, &s->b, &s->r1, &s->r2, &s->z0, &s->z1, &s->u, &s->w0, &s->w1, &s->w2,
                  &s->dx, &s->xc, &s->xp};
  for (size_t k = 0; k < sizeof(w) / sizeof(w[0]); k++) *w[k] = (double *)xcalloc(2 * N, nb);
  return s;
}

static void free_level(level_t *L, int own_graph)
{
  if (own_graph) { free(L->rp); free(L->ci); free(L->off); free(L->dia); }
  free(L->dinv); free(L->agg); free(L->mem_ptr); free(L->mem_idx); free(L->seg_ptr);
  free(L->seg_idx); free(L->intra_ptr); free(L->intra_idx); free(L->b); free(L->x);
  free(L->x2); free(L->d); free(L->res); free(L->dense);
}

void nor_solver_destroy(nor_solver *s)
{
  if (!s) return;
  for (int l = 0; l < s->nlev; l++) free_level(&s->lev[l], l > 0);
  free(s->rp); free(s->ci); free(s->nz_edge); free(s->alpha); free(s->p); free(s->cv);
  free(s->t); free(s->V); free(s->kdiag); free(s->keo); free(s->jd); free(s->rd);
  double *w[] = {s->f, s->b, s->r1, s->r2, s->z0, s->z1, s->u, s->w0, s->w1, s->w2, s->dx,
                 s->xc, s->xp};
  for (size_t k = 0; k < sizeof(w) / sizeof(w[0]); k++) free(w[k]);
  free(s);
}

int nor_num_threads(void)
{
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

int nor_set_num_threads(int n)
{
#ifdef _OPENMP
  const int prev = omp_get_max_threads();
  if (n >= 1) omp_set_num_threads(n);
  return prev;
#else
  (void)n;
  return 1;
#endif
}

/* ------------------------------------------------------------ operators */
static void keo_refill(nor_solver *s, double mu)
{
  if (s->mu_keo == mu) return;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < s->N; i++)
    for (int32_t k = s->rp[i]; k < s->rp[i + 1]; k++) {
      const int32_t e0 = s->nz_edge[k], e = e0 >= 0 ? e0 : ~e0;
      const double a = mu * s->p[e], al = s->alpha[e];
      /* -alpha e^{-ia} from v0 to v1, its conjugate from v1 to v0 */
      s->keo[2 * k] = -al * cos(a);
      s->keo[2 * k + 1] = (e0 >= 0 ? 1.0 : -1.0) * al * sin(a);
    }
  s->mu_keo = mu;
}

/* y = offdiag x + [[a, c], [c, b]] x_i  over one level's CSR */
static void block_apply(int64_t n, const int32_t *rp, const int32_t *ci, const double *off,
                        const double *dia, const double *x, double *y)
{
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; i++) {
    double sr = 0.0, si = 0.0;
    for (int32_t k = rp[i]; k < rp[i + 1]; k++) {
      const double vr = off[2 * k], vi = off[2 * k + 1];
      const double xr = x[2 * ci[k]], xi = x[2 * ci[k] + 1];
      sr += vr * xr - vi * xi;
      si += vr * xi + vi * xr;
    }
    const double xr = x[2 * i], xi = x[2 * i + 1];
    y[2 * i] = sr + dia[3 * i] * xr + dia[3 * i + 2] * xi;
    y[2 * i + 1] = si + dia[3 * i + 2] * xr + dia[3 * i + 1] * xi;
  }
}

static double compute_f_norm(nor_solver *s, const double *psi, double mu, double *f)
{
  keo_refill(s, mu);
  double n2 = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : n2)
  for (int64_t i = 0; i < s->N; i++) {
    double sr = 0.0, si = 0.0;
    for (int32_t k = s->rp[i]; k < s->rp[i + 1]; k++) {
      const double vr = s->keo[2 * k], vi = s->keo[2 * k + 1];
      const double xr = psi[2 * s->ci[k]], xi = psi[2 * s->ci[k] + 1];
      sr += vr * xr - vi * xi;
      si += vr * xi + vi * xr;
    }
    const double xr = psi[2 * i], xi = psi[2 * i + 1];
    const double a = s->kdiag[i] + s->cv[i] * s->t[i] * (s->V[i] + s->g * (xr * xr + xi * xi));
    f[2 * i] = sr + a * xr;
    f[2 * i + 1] = si + a * xi;
    n2 += f[2 * i] * f[2 * i] + f[2 * i + 1] * f[2 * i + 1];
  }
  return sqrt(n2);
}

static void rebuild_diags(nor_solver *s, const double *psi)
{
  const double g = s->g;
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < s->N; k++) {
    const double re = psi[2 * k], im = psi[2 * k + 1], w = s->cv[k] * s->t[k];
    const double al = w * (s->V[k] + g * 2.0 * (re * re + im * im));
    const double rx2 = g * w * (re * re - im * im);
    s->jd[3 * k] = s->kdiag[k] + al + rx2;
    s->jd[3 * k + 1] = s->kdiag[k] + al - rx2;
    s->jd[3 * k + 2] = g * w * 2.0 * re * im;
    double a = s->kdiag[k], b = s->kdiag[k], c = 0.0;
    if (g > 0.0) {
      const double wg = g * w;
      const double al2 = wg * 2.0 * (re * re + im * im), be = wg * 2.0 * re * im,
                   ga = wg * (re * re - im * im);
      a += al2 + ga; b += al2 - ga; c = be;
    }
    s->rd[3 * k] = a; s->rd[3 * k + 1] = b; s->rd[3 * k + 2] = c;
  }
}

/* ------------------------------------------------------------------ AMG */
#define THETA 0.05
#define CHEB_RATIO 30.0
#define COARSE_SIZE 64

static int64_t aggregate(const level_t *L, int32_t *agg)
{
  const int64_t n = L->n;
  double *scale = (double *)xcalloc(n, sizeof(double));
  for (int64_t i = 0; i < n; i++) {
    const double v = 0.5 * (L->dia[3 * i] + L->dia[3 * i + 1]);
    scale[i] = v > 1e-300 ? v : 1e-300;
  }
#define STRONG(i, k) \
  (hypot(L->off[2 * (k)], L->off[2 * (k) + 1]) >= THETA * sqrt(scale[i] * scale[L->ci[k]]))
  for (int64_t i = 0; i < n; i++) agg[i] = -1;
  int64_t na = 0;
  for (int64_t i = 0; i < n; i++) {
    if (agg[i] >= 0) continue;
    int free_ = 1;
    for (int32_t k = L->rp[i]; k < L->rp[i + 1] && free_; k++)
      if (STRONG(i, k) && agg[L->ci[k]] >= 0) free_ = 0;
    if (!free_) continue;
    agg[i] = (int32_t)na;
    for (int32_t k = L->rp[i]; k < L->rp[i + 1]; k++)
      if (STRONG(i, k)) agg[L->ci[k]] = (int32_t)na;
    na++;
  }
  int32_t *agg1 = (int32_t *)xcalloc(n, 4);
  memcpy(agg1, agg, n * 4);
  for (int64_t i = 0; i < n; i++) {
    if (agg1[i] >= 0) continue;
    double best = -1.0;
    int32_t to = -1;
    for (int32_t k = L->rp[i]; k < L->rp[i + 1]; k++) {
      const int32_t a = agg1[L->ci[k]];
      const double m = hypot(L->off[2 * k], L->off[2 * k + 1]);
      if (a >= 0 && m > best) { best = m; to = a; }
    }
    agg[i] = to;
  }
  for (int64_t i = 0; i < n; i++)
    if (agg[i] < 0) agg[i] = (int32_t)na++;
#undef STRONG
  free(agg1); free(scale);
  return na;
}

static int cmp_i32(const void *a, const void *b)
{
  const int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
  return (x > y) - (x < y);
}

/* structure of level l+1 from level l (values filled by amg_numeric) */
static void coarsen(level_t *F, level_t *C)
{
  const int64_t n = F->n;
  F->agg = (int32_t *)xcalloc(n, 4);
  const int64_t na = aggregate(F, F->agg);
  C->n = na;
  F->mem_ptr = (int32_t *)xcalloc(na + 1, 4);
  for (int64_t i = 0; i < n; i++) F->mem_ptr[F->agg[i] + 1]++;
  for (int64_t a = 0; a < na; a++) F->mem_ptr[a + 1] += F->mem_ptr[a];
  F->mem_idx = (int32_t *)xcalloc(n, 4);
  int32_t *fill = (int32_t *)xcalloc(na + 1, 4);
  memcpy(fill, F->mem_ptr, na * 4);
  for (int64_t i = 0; i < n; i++) F->mem_idx[fill[F->agg[i]]++] = (int32_t)i;
  /* coarse rows */
  C->rp = (int32_t *)xcalloc(na + 1, 4);
  int32_t *buf = (int32_t *)xcalloc(F->rp[n] + 1, 4);
  int64_t tot = 0;
  int32_t *rowstart = (int32_t *)xcalloc(na + 1, 4);
  for (int64_t a = 0; a < na; a++) {
    int64_t m = 0;
    int32_t *r = buf + tot;
    for (int32_t q = F->mem_ptr[a]; q < F->mem_ptr[a + 1]; q++) {
      const int32_t i = F->mem_idx[q];
      for (int32_t k = F->rp[i]; k < F->rp[i + 1]; k++) {
        const int32_t b = F->agg[F->ci[k]];
        if (b != a) r[m++] = b;
      }
    }
    qsort(r, m, 4, cmp_i32);
    int64_t u = 0;
    for (int64_t k = 0; k < m; k++)
      if (k == 0 || r[k] != r[k - 1]) r[u++] = r[k];
    rowstart[a] = (int32_t)tot;
    C->rp[a + 1] = C->rp[a] + (int32_t)u;
    tot += u;
  }
  C->ci = (int32_t *)xcalloc(C->rp[na] + 1, 4);
  for (int64_t a = 0; a < na; a++)
    memcpy(C->ci + C->rp[a], buf + rowstart[a], (C->rp[a + 1] - C->rp[a]) * 4);
  free(buf); free(rowstart);
  const int64_t nzc = C->rp[na];
  C->nnz = nzc;
  int32_t *target = (int32_t *)xcalloc(F->rp[n] + 1, 4);
  F->seg_ptr = (int32_t *)xcalloc(nzc + 1, 4);
  F->intra_ptr = (int32_t *)xcalloc(na + 1, 4);
  for (int64_t i = 0; i < n; i++) {
    const int32_t a = F->agg[i];
    for (int32_t k = F->rp[i]; k < F->rp[i + 1]; k++) {
      const int32_t b = F->agg[F->ci[k]];
      if (b == a) { target[k] = -1; F->intra_ptr[a + 1]++; }
      else {
        int32_t lo = C->rp[a], hi = C->rp[a + 1] - 1;
        while (lo < hi) { const int32_t mid = (lo + hi) / 2; if (C->ci[mid] < b) lo = mid + 1; else hi = mid; }
        target[k] = lo;
        F->seg_ptr[lo + 1]++;
      }
    }
  }
  for (int64_t q = 0; q < nzc; q++) F->seg_ptr[q + 1] += F->seg_ptr[q];
  for (int64_t a = 0; a < na; a++) F->intra_ptr[a + 1] += F->intra_ptr[a];
  F->seg_idx = (int32_t *)xcalloc(F->seg_ptr[nzc] + 1, 4);
  F->intra_idx = (int32_t *)xcalloc(F->intra_ptr[na] + 1, 4);
  int32_t *fs = (int32_t *)xcalloc(nzc + 1, 4), *fi = (int32_t *)xcalloc(na + 1, 4);
  memcpy(fs, F->seg_ptr, nzc * 4);
  memcpy(fi, F->intra_ptr, na * 4);
  for (int64_t i = 0; i < n; i++)
    for (int32_t k = F->rp[i]; k < F->rp[i + 1]; k++) {
      if (target[k] >= 0) F->seg_idx[fs[target[k]]++] = k;
      else F->intra_idx[fi[F->agg[i]]++] = k;
    }
  free(fs); free(fi); free(target); free(fill);
  C->off = (double *)xcalloc(2 * nzc + 2, sizeof(double));
  C->dia = (double *)xcalloc(3 * na, sizeof(double));
}

static void galerkin(const level_t *F, level_t *C)
{
#pragma omp parallel for schedule(static)
  for (int64_t q = 0; q < C->nnz; q++) {
    double sr = 0.0, si = 0.0;
    for (int32_t j = F->seg_ptr[q]; j < F->seg_ptr[q + 1]; j++) {
      sr += F->off[2 * F->seg_idx[j]];
      si += F->off[2 * F->seg_idx[j] + 1];
    }
    C->off[2 * q] = sr; C->off[2 * q + 1] = si;
  }
#pragma omp parallel for schedule(static)
  for (int64_t a = 0; a < C->n; a++) {
    double d0 = 0, d1 = 0, d2 = 0;
    for (int32_t j = F->mem_ptr[a]; j < F->mem_ptr[a + 1]; j++) {
      const int32_t i = F->mem_idx[j];
      d0 += F->dia[3 * i]; d1 += F->dia[3 * i + 1]; d2 += F->dia[3 * i + 2];
    }
    for (int32_t j = F->intra_ptr[a]; j < F->intra_ptr[a + 1]; j++) {
      const double re = F->off[2 * F->intra_idx[j]];
      d0 += re; d1 += re;
    }
    C->dia[3 * a] = d0; C->dia[3 * a + 1] = d1; C->dia[3 * a + 2] = d2;
  }
}

static void smoother_setup(level_t *L, int deg)
{
  double lmax = 0.0;
#pragma omp parallel for schedule(static) reduction(max : lmax)
  for (int64_t i = 0; i < L->n; i++) {
    const double a = L->dia[3 * i], d = L->dia[3 * i + 1], b = L->dia[3 * i + 2];
    const double det = a * d - b * b;
    L->dinv[3 * i] = d / det; L->dinv[3 * i + 1] = a / det; L->dinv[3 * i + 2] = -b / det;
    const double lmin = 0.5 * (a + d) - sqrt(0.25 * (a - d) * (a - d) + b * b);
    double s = 0.0;
    for (int32_t k = L->rp[i]; k < L->rp[i + 1]; k++) s += hypot(L->off[2 * k], L->off[2 * k + 1]);
    const double bound = (lmin > 0.0 && det > 0.0) ? 1.0 + s / lmin : 1e300;
    if (bound > lmax) lmax = bound;
  }
  const double hi = 1.1 * lmax, lo = lmax / CHEB_RATIO;
  const double theta = 0.5 * (hi + lo), delta = 0.5 * (hi - lo), sigma = theta / delta;
  double rho = 1.0 / sigma;
  L->coef[0] = 1.0 / theta;
  for (int k = 1; k < deg; k++) {
    const double rn = 1.0 / (2.0 * sigma - rho);
    L->coef[2 * k] = rn * rho;
    L->coef[2 * k + 1] = 2.0 * rn / delta;
    rho = rn;
  }
}

static int dense_inverse(level_t *L)
{
  const int64_t n = L->n, m = 2 * n;
  double *A = L->dense;
  memset(A, 0, m * m * sizeof(double));
  for (int64_t i = 0; i < n; i++) {
    A[(2 * i) * m + 2 * i] = L->dia[3 * i];
    A[(2 * i) * m + 2 * i + 1] = L->dia[3 * i + 2];
    A[(2 * i + 1) * m + 2 * i] = L->dia[3 * i + 2];
    A[(2 * i + 1) * m + 2 * i + 1] = L->dia[3 * i + 1];
    for (int32_t k = L->rp[i]; k < L->rp[i + 1]; k++) {
      const int64_t j = L->ci[k];
      const double vr = L->off[2 * k], vi = L->off[2 * k + 1];
      A[(2 * i) * m + 2 * j] = vr; A[(2 * i) * m + 2 * j + 1] = -vi;
      A[(2 * i + 1) * m + 2 * j] = vi; A[(2 * i + 1) * m + 2 * j + 1] = vr;
    }
  }
  for (int64_t k = 0; k < m; k++) {
    const double piv = A[k * m + k];
    if (!(piv > 0.0)) return NOSH_ERR_BREAKDOWN_ORACLE;
    const double ip = 1.0 / piv;
    for (int64_t j = 0; j < m; j++) A[k * m + j] = (j == k) ? ip : A[k * m + j] * ip;
    for (int64_t i = 0; i < m; i++) {
      if (i == k) continue;
      const double f = A[i * m + k];
      for (int64_t j = 0; j < m; j++) if (j != k) A[i * m + j] -= f * A[k * m + j];
      A[i * m + k] = -f * ip;
    }
  }
  return 0;
}

static void alloc_level_work(level_t *L)
{
  const int64_t n = L->n;
  L->dinv = (double *)xcalloc(3 * n, sizeof(double));
  double **w[] = {&L->b, &L->x, &L->x2, &L->d, &L->res};
  for (int k = 0; k < 5; k++) *w[k] = (double *)xcalloc(2 * n, sizeof(double));
}

/* build the hierarchy (first call) or refresh its values */
static int amg_refresh(nor_solver *s)
{
  level_t *L0 = &s->lev[0];
  if (s->nlev == 0) {
    L0->n = s->N; L0->nnz = s->rp[s->N];
    L0->rp = s->rp; L0->ci = s->ci; L0->off = s->keo; L0->dia = s->rd;
    alloc_level_work(L0);
    s->nlev = 1;
    while (s->nlev < 10 && s->lev[s->nlev - 1].n > COARSE_SIZE) {
      level_t *F = &s->lev[s->nlev - 1], *C = &s->lev[s->nlev];
      coarsen(F, C);
      galerkin(F, C);
      if (C->n >= F->n) { free_level(C, 1); memset(C, 0, sizeof(*C)); break; }
      alloc_level_work(C);
      s->nlev++;
    }
    level_t *Lc = &s->lev[s->nlev - 1];
    Lc->dense = (double *)xcalloc(4 * Lc->n * Lc->n, sizeof(double));
  }
  L0->off = s->keo; L0->dia = s->rd;
  for (int l = 1; l < s->nlev; l++) galerkin(&s->lev[l - 1], &s->lev[l]);
  for (int l = 0; l < s->nlev; l++) smoother_setup(&s->lev[l], s->deg);
  return dense_inverse(&s->lev[s->nlev - 1]);
}

/* Chebyshev step k with SpMV: x_out = x_in + d_k */
static void cheb_step(level_t *L, int k, const double *b, const double *xin, double *xout)
{
  const int64_t n = L->n;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; i++) {
    double sr = 0.0, si = 0.0;
    for (int32_t q = L->rp[i]; q < L->rp[i + 1]; q++) {
      const double vr = L->off[2 * q], vi = L->off[2 * q + 1];
      const double xr = xin[2 * L->ci[q]], xi = xin[2 * L->ci[q] + 1];
      sr += vr * xr - vi * xi;
      si += vr * xi + vi * xr;
    }
    const double xr = xin[2 * i], xi = xin[2 * i + 1];
    const double rr = b[2 * i] - (sr + L->dia[3 * i] * xr + L->dia[3 * i + 2] * xi);
    const double ri = b[2 * i + 1] - (si + L->dia[3 * i + 2] * xr + L->dia[3 * i + 1] * xi);
    const double zr = L->dinv[3 * i] * rr + L->dinv[3 * i + 2] * ri;
    const double zi = L->dinv[3 * i + 2] * rr + L->dinv[3 * i + 1] * ri;
    double dr, di;
    if (k == 0) { dr = L->coef[0] * zr; di = L->coef[0] * zi; }
    else {
      dr = L->coef[2 * k] * L->d[2 * i] + L->coef[2 * k + 1] * zr;
      di = L->coef[2 * k] * L->d[2 * i + 1] + L->coef[2 * k + 1] * zi;
    }
    L->d[2 * i] = dr; L->d[2 * i + 1] = di;
    xout[2 * i] = xr + dr; xout[2 * i + 1] = xi + di;
  }
}

static void vcycle(nor_solver *s, int l, const double *b, double *x)
{
  level_t *L = &s->lev[l];
  const int64_t n = L->n;
  if (l == s->nlev - 1) {
    const int64_t m = 2 * n;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < m; i++) {
      double a = 0.0;
      for (int64_t j = 0; j < m; j++) a += L->dense[i * m + j] * b[j];
      x[i] = a;
    }
    return;
  }
  const int deg = s->deg;
  double *cur = (deg % 2 == 1) ? x : L->x2, *oth = (deg % 2 == 1) ? L->x2 : x;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; i++) {
    const double br = b[2 * i], bi = b[2 * i + 1];
    const double dr = L->coef[0] * (L->dinv[3 * i] * br + L->dinv[3 * i + 2] * bi);
    const double di = L->coef[0] * (L->dinv[3 * i + 2] * br + L->dinv[3 * i + 1] * bi);
    L->d[2 * i] = dr; L->d[2 * i + 1] = di;
    cur[2 * i] = dr; cur[2 * i + 1] = di;
  }
  for (int k = 1; k < deg; k++) {
    cheb_step(L, k, b, cur, oth);
    double *t = cur; cur = oth; oth = t;
  }
  block_apply(n, L->rp, L->ci, L->off, L->dia, x, L->res);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < 2 * n; i++) L->res[i] = b[i] - L->res[i];
  level_t *C = &s->lev[l + 1];
#pragma omp parallel for schedule(static)
  for (int64_t a = 0; a < C->n; a++) {
    double sr = 0.0, si = 0.0;
    for (int32_t j = L->mem_ptr[a]; j < L->mem_ptr[a + 1]; j++) {
      sr += L->res[2 * L->mem_idx[j]];
      si += L->res[2 * L->mem_idx[j] + 1];
    }
    C->b[2 * a] = sr; C->b[2 * a + 1] = si;
  }
  vcycle(s, l + 1, C->b, C->x);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; i++) {
    x[2 * i] += C->x[2 * L->agg[i]];
    x[2 * i + 1] += C->x[2 * L->agg[i] + 1];
  }
  cur = x; oth = L->x2;
  for (int k = 0; k < deg; k++) {
    cheb_step(L, k, b, cur, oth);
    double *t = cur; cur = oth; oth = t;
  }
  if (cur != x) memcpy(x, cur, 2 * n * sizeof(double));
}

/* --------------------------------------------------------------- MINRES */
static double dot(int64_t n, const double *a, const double *b)
{
  double s = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : s)
  for (int64_t i = 0; i < n; i++) s += a[i] * b[i];
  return s;
}

static int minres(nor_solver *s, const double *b, double rtol, int maxit, double *x, int *its)
{
  const int64_t n2 = 2 * s->N;
  double *r1 = s->r1, *r2 = s->r2, *zc = s->z0, *zn = s->z1, *u = s->u;
  double *wa = s->w0, *wb = s->w1, *wc = s->w2;
  memcpy(r1, b, n2 * sizeof(double));
  memcpy(r2, b, n2 * sizeof(double));
  memset(x, 0, n2 * sizeof(double));
  memset(wa, 0, n2 * sizeof(double)); memset(wb, 0, n2 * sizeof(double)); memset(wc, 0, n2 * sizeof(double));
  vcycle(s, 0, r2, zc);
  double rz = dot(n2, r2, zc);
  *its = 0;
  if (!(rz >= 0.0)) return NOSH_ERR_BREAKDOWN_ORACLE;
  if (rz == 0.0) return 0;
  const double beta1 = sqrt(rz);
  double beta = beta1, oldb = 0.0, dbar = 0.0, epsln = 0.0, phibar = beta1, cs = -1.0, sn = 0.0;
  for (int itn = 0; itn < maxit; itn++) {
    block_apply(s->N, s->rp, s->ci, s->keo, s->jd, zc, u);
    const double zu = dot(n2, zc, u);
    const double alfa = zu / (beta * beta);
    const double a = 1.0 / beta, c = alfa / beta, bb = itn > 0 ? beta / oldb : 0.0;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n2; i++) r1[i] = a * u[i] - bb * r1[i] - c * r2[i];
    double *t = r1; r1 = r2; r2 = t;
    vcycle(s, 0, r2, zn);
    rz = dot(n2, r2, zn);
    oldb = beta;
    if (!(rz >= 0.0)) return NOSH_ERR_BREAKDOWN_ORACLE;
    beta = sqrt(rz);
    const double oldeps = epsln;
    const double delta = cs * dbar + sn * alfa;
    const double gbar = sn * dbar - cs * alfa;
    epsln = sn * beta;
    dbar = -cs * beta;
    double gamma = hypot(gbar, beta);
    if (gamma == 0.0) gamma = 2.2e-16;
    cs = gbar / gamma; sn = beta / gamma;
    const double phi = cs * phibar;
    phibar = sn * phibar;
    const double iv = 1.0 / oldb, ig = 1.0 / gamma;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n2; i++) {
      const double w = (zc[i] * iv - oldeps * wb[i] - delta * wc[i]) * ig;
      wa[i] = w;
      x[i] += phi * w;
    }
    double *tw = wa; wa = wb; wb = wc; wc = tw;
    t = zc; zc = zn; zn = t;
    *its = itn + 1;
    if (phibar <= rtol * beta1 || beta == 0.0) return 0;
  }
  return NOSH_ERR_NOT_CONVERGED_ORACLE;
}

/* ---------------------------------------------------------------- Newton */
int nor_newton(nor_solver *s, double *psi, double mu, double tol, int max_newton, int *newton_its,
               int *krylov_its, double *fnorm0, double *fnorm)
{
  const int64_t n2 = 2 * s->N;
  double fn = compute_f_norm(s, psi, mu, s->f), fn_prev = fn;
  *fnorm0 = fn;
  *newton_its = 0;
  *krylov_its = 0;
  for (int it = 0; it < max_newton && fn > tol; it++) {
    rebuild_diags(s, psi);
    int rc = amg_refresh(s);
    if (rc) return rc;
    for (int64_t i = 0; i < n2; i++) s->b[i] = -s->f[i];
    double ew = it == 0 ? 1e-2 : 0.9 * (fn / fn_prev) * (fn / fn_prev);
    double eta = ew > 0.5 * tol / fn ? ew : 0.5 * tol / fn;
    if (eta > 0.1) eta = 0.1;
    if (eta < 1e-12) eta = 1e-12;
    int its = 0;
    rc = minres(s, s->b, eta, 1000, s->dx, &its);
    *krylov_its += its;
    if (rc == NOSH_ERR_BREAKDOWN_ORACLE) return rc;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n2; i++) psi[i] += s->dx[i];
    fn_prev = fn;
    fn = compute_f_norm(s, psi, mu, s->f);
    *newton_its = it + 1;
  }
  *fnorm = fn;
  return fn <= tol ? 0 : NOSH_ERR_NOT_CONVERGED_ORACLE;
}

/* one natural continuation step with a phase-aligned secant predictor
 * (x_prev == NULL: the current state is the prediction) */
int nor_continuation_step(nor_solver *s, double *x, double *x_prev, double mu_new, double mu_cur,
                          double mu_prev, double tol, int *newton_its, int *krylov_its,
                          double *fnorm0, double *fnorm)
{
  const int64_t N = s->N;
  if (x_prev) {
    double cr = 0.0, ci = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : cr, ci)
    for (int64_t i = 0; i < N; i++) {
      cr += x_prev[2 * i] * x[2 * i] + x_prev[2 * i + 1] * x[2 * i + 1];
      ci += x_prev[2 * i] * x[2 * i + 1] - x_prev[2 * i + 1] * x[2 * i];
    }
    const double m = hypot(cr, ci), er = m > 0 ? cr / m : 1.0, ei = m > 0 ? ci / m : 0.0;
    const double r = (mu_new - mu_cur) / (mu_cur - mu_prev);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < N; i++) {
      const double pr = er * x_prev[2 * i] - ei * x_prev[2 * i + 1];
      const double pi = er * x_prev[2 * i + 1] + ei * x_prev[2 * i];
      const double ar = x[2 * i], ai = x[2 * i + 1];
      x_prev[2 * i] = ar; x_prev[2 * i + 1] = ai;
      x[2 * i] = ar + r * (ar - pr);
      x[2 * i + 1] = ai + r * (ai - pi);
    }
  }
  return nor_newton(s, x, mu_new, tol, 20, newton_its, krylov_its, fnorm0, fnorm);
}

int nor_amg_levels(const nor_solver *s, int64_t *sizes)
{
  for (int l = 0; l < s->nlev; l++) sizes[l] = s->lev[l].n;
  return s->nlev;
}
