/*
 * nosh_oracle.h -- CPU FP64 restatement of nosh's Ginzburg-Landau /
 * nonlinear-Schroedinger hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity oracle and the
 * timed CPU baseline.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline / reference arm may load it.  The product library
 * (nosh_gb300) never links, loads or calls it.
 *
 * Every routine cites the reference file:line it restates (paths relative to
 * the nosh source tree).  The reference itself (Trilinos/MOAB/Eigen) cannot
 * be built here; this restatement is pinned against the known-answer
 * constants of the reference's own tests (test/keo.cpp, test/jac.cpp,
 * test/compute_f.cpp, test/mesh.cpp) on the reconstructed "rectanglesmall"
 * and "cubesmall" meshes -- see tests/test_oracle_kat.py.
 *
 * Conventions
 *   - vertices 0..N-1, coordinates x[3*i+{0,1,2}]
 *   - cells: nvc = 3 (triangles) or 4 (tetrahedra) vertex ids per cell
 *   - edges: canonical (v0 < v1) pairs in lexicographic order
 *   - complex vectors interleaved [Re0, Im0, Re1, Im1, ...]
 *     (src/mesh.cpp:597-607, complexify_)
 *   - complex CSR ("block CSR"): one complex value per 2x2 real block,
 *     rows = vertices, sorted columns, diagonal included
 *     (src/mesh.cpp:789-882, build_complex_graph)
 */
#ifndef NOSH_ORACLE_H
#define NOSH_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- deterministic RNG (splitmix64) used by the synthetic mesh generator */
uint64_t nor_splitmix64(uint64_t *state);
double nor_uniform(uint64_t *state, double lo, double hi);

/* ---- synthetic structured meshes (jittered) ---------------------------- */
/* unit square, s x s vertices, each square cut into 2 right triangles.
 * x: 3*s*s, cells: 3*2*(s-1)^2, psi: 2*s*s (psi = 1 + U(-.01,.01) + iU(..)). */
void nor_gen_square(int s, uint64_t seed, double jitter, double *x,
                    int32_t *cells, double *psi);
/* unit cube, m^3 cubes each cut into 6 Kuhn tetrahedra.
 * x: 3*(m+1)^3, cells: 4*6*m^3, psi: 2*(m+1)^3 */
void nor_gen_cube(int m, uint64_t seed, double jitter, double *x,
                  int32_t *cells, double *psi);

/* ---- integer mesh work -------------------------------------------------- */
/* edges (2*cap ints, cap = T*ne) and cell->edge map (T*ne); returns E. */
int64_t nor_build_edges(int nvc, int64_t N, int64_t T, const int32_t *cells,
                        int32_t *edges, int32_t *cell_edges);
/* complex graph: row_ptr[N+1], cols[N+2E] */
void nor_complex_graph(int64_t N, int64_t E, const int32_t *edges,
                       int32_t *row_ptr, int32_t *cols);

/* ---- geometry ----------------------------------------------------------- */
void nor_edge_data(int nvc, int64_t N, const double *x, int64_t E,
                   const int32_t *edges, int64_t T, const int32_t *cell_edges,
                   double *length, double *covolume);
void nor_control_volumes(int nvc, int64_t N, const double *x, int64_t T,
                         const int32_t *cells, double *cv);
void nor_edge_projection(int64_t E, const int32_t *edges, const double *x,
                         const double *A, double *p);
void nor_alpha(int64_t E, const int32_t *edges, const double *length,
               const double *covolume, const double *thickness, double *alpha);

/* ---- operators (FP64) --------------------------------------------------- */
void nor_keo_values(int64_t N, int64_t E, const int32_t *edges,
                    const double *alpha, const double *p, double mu,
                    const int32_t *row_ptr, const int32_t *cols, double *vals);
void nor_dkeo_values(int64_t N, int64_t E, const int32_t *edges,
                     const double *alpha, const double *p, const double *dp,
                     double mu, const int32_t *row_ptr, const int32_t *cols,
                     double *vals);
void nor_keo_apply(int64_t N, int64_t E, const int32_t *edges,
                   const double *alpha, const double *p, double mu,
                   const double *x, double *y);
void nor_dkeo_apply(int64_t N, int64_t E, const int32_t *edges,
                    const double *alpha, const double *p, const double *dp,
                    double mu, const double *x, double *y);
void nor_compute_f(int64_t N, int64_t E, const int32_t *edges,
                   const double *alpha, const double *p, double mu, double g,
                   const double *cv, const double *t, const double *V,
                   const double *psi, double *f);
void nor_dfdp(int64_t N, int64_t E, const int32_t *edges, const double *alpha,
              const double *p, const double *dp, double mu, int param_is_g,
              const double *cv, const double *t, const double *dVdp,
              const double *psi, double *out);
void nor_jac_diags(int64_t N, const double *cv, const double *t,
                   const double *V, double g, const double *psi, double *d0,
                   double *d1b);
void nor_jac_apply(int64_t N, int64_t E, const int32_t *edges,
                   const double *alpha, const double *p, double mu,
                   const double *d0, const double *d1b, const double *x,
                   double *y);
void nor_kreg_apply(int64_t N, int64_t E, const int32_t *edges,
                    const double *alpha, const double *p, double mu, double g,
                    const double *cv, const double *t, const double *psi,
                    const double *x, double *y);
double nor_energy(int64_t N, const double *cv, const double *psi);
double nor_inner_product(int64_t N, const double *cv, const double *phi,
                         const double *psi);

/* ---- CPU solver (nosh_solver.c): Newton / MINRES / AMG / continuation -- */
#define NOSH_ERR_NOT_CONVERGED_ORACLE 3
#define NOSH_ERR_BREAKDOWN_ORACLE 5
typedef struct nor_solver nor_solver;
nor_solver *nor_solver_create(int64_t N, int64_t E, const int32_t *edges,
                              const double *alpha, const double *p,
                              const double *cv, const double *t,
                              const double *V, double g);
void nor_solver_destroy(nor_solver *s);
int nor_num_threads(void);
/* OpenMP threads of the solver calls that follow on the calling host thread
   (n >= 1; n < 1 leaves it unchanged); returns the previous maximum. */
int nor_set_num_threads(int n);
int nor_newton(nor_solver *s, double *psi, double mu, double tol,
               int max_newton, int *newton_its, int *krylov_its,
               double *fnorm0, double *fnorm);
int nor_continuation_step(nor_solver *s, double *x, double *x_prev,
                          double mu_new, double mu_cur, double mu_prev,
                          double tol, int *newton_its, int *krylov_its,
                          double *fnorm0, double *fnorm);
int nor_amg_levels(const nor_solver *s, int64_t *sizes);

#ifdef __cplusplus
}
#endif
#endif
