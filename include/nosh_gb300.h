/*
 * nosh_gb300.h -- C ABI of the GB300-native Newton-Krylov core for nosh's
 * finite-volume Ginzburg-Landau / nonlinear Schroedinger problem
 *
 *     0 = F(psi) = (K + V + g|psi|^2) psi .
 *
 * Each entry point names the reference (nschloe/nosh) interface it replaces,
 * as file:line within the nosh source tree.  The reference binds these
 * through Tpetra / Thyra objects; here every argument is a plain pointer plus
 * sizes so that any FFI (C++, ctypes, cgo, JNI) can bind it.
 *
 * Conventions
 *  - Return value: NOSH_OK (0) or one of the NOSH_ERR_* codes; a message is
 *    kept per thread in nosh_last_error().  No exception crosses the ABI.
 *  - Complex vectors are interleaved [Re0, Im0, Re1, Im1, ...] of length
 *    2*N doubles (the reference's complex map, src/mesh.cpp:597-607).
 *  - Vector arguments may live in host memory (pageable or pinned) or in
 *    device memory of the current CUDA device; the library detects which.
 *  - The parameter vector p follows the reference's sorted parameter names
 *    (src/model_evaluator_nls.cpp:102-130): p[0] = "g", p[1] = "mu".
 *  - Handles are not thread-safe (the reference's operators are mutated by
 *    rebuild()/refill_ too); use one handle per host thread.  Each nls
 *    handle owns one CUDA stream; calls return after their work on it is
 *    complete unless the name ends in _async.
 *  - There is no CPU fallback: on a machine without a usable GPU every
 *    compute entry point fails with NOSH_ERR_CUDA.
 */
#ifndef NOSH_GB300_H
#define NOSH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NOSH_OK 0
#define NOSH_ERR_INVALID 1       /* bad argument / size mismatch           */
#define NOSH_ERR_CUDA 2          /* CUDA runtime error, or no GPU          */
#define NOSH_ERR_NOT_CONVERGED 3 /* iteration limit reached                */
#define NOSH_ERR_NAN 4           /* NaN/Inf met in a reduction             */
#define NOSH_ERR_BREAKDOWN 5     /* Krylov breakdown (indefinite precond.) */
#define NOSH_ERR_UNSUPPORTED 6   /* e.g. apply() with mode/alpha/beta the
                                    reference rejects too                  */
#define NOSH_ERR_MESH 7          /* degenerate cell                        */
#define NOSH_ERR_NO_MEMORY 8

/* operator / Krylov precision */
#define NOSH_PREC_FP64 0  /* everything in FP64                             */
#define NOSH_PREC_MIXED 1 /* FP32 KEO/SpMV/MINRES/AMG, FP64 residual+scalars */

/* apply() mode, as Teuchos::ETransp */
#define NOSH_NO_TRANS 0
#define NOSH_TRANS 1

typedef struct nosh_mesh_s *nosh_mesh;
typedef struct nosh_nls_s *nosh_nls;

/* Last error message of the calling thread ("" when none). */
const char *nosh_last_error(void);
/* Library version (major*10000 + minor*100 + patch). */
int nosh_version(void);
/* Number of CUDA devices visible; 0 (and NOSH_ERR_CUDA) without a GPU. */
int nosh_device_count(int *count);

/* ------------------------------------------------------------------ mesh */
/* Builds the mesh and all its derived data.  Replaces nosh::read +
 * mesh_tri / mesh_tetra construction (src/mesh_reader.cpp:20-162,
 * src/mesh_tri.cpp:14-39, src/mesh_tetra.cpp:14-35): edges
 * (build_entity_relations_, src/mesh.cpp:631-691), edge data
 * (compute_edge_data_, src/mesh_tri.cpp:46-103 / src/mesh_tetra.cpp:43-103)
 * and control volumes (compute_control_volumes_t_, src/mesh_tri.cpp:187-210 /
 * src/mesh_tetra.cpp:196-271).  coords: 3*N doubles; cells: T*verts_per_cell
 * vertex ids, verts_per_cell = 3 (triangles) or 4 (tetrahedra).  Geometry is
 * computed on the GPU in FP64; integer work on the host. */
int nosh_mesh_create(const double *coords, int64_t num_vertices,
                     const int32_t *cells, int64_t num_cells,
                     int verts_per_cell, nosh_mesh *out);
int nosh_mesh_destroy(nosh_mesh mesh);
/* nnz_blocks = N + 2E, the number of 2x2 blocks of the KEO graph. */
int nosh_mesh_sizes(nosh_mesh mesh, int64_t *num_vertices, int64_t *num_edges,
                    int64_t *num_cells, int64_t *nnz_blocks);
/* Edge list (E x 2 vertex ids, v0 < v1, lexicographic): mesh::my_edges /
 * edge_lids (src/mesh.hpp:103-107, src/mesh.cpp:450-471). */
int nosh_mesh_edges(nosh_mesh mesh, int32_t *edges);
/* Complex global indices per edge (E x 4: 2g, 2g+1, 2h, 2h+1 with 1-based
 * vertex GIDs g, h): mesh::build_edge_gids_complex_ (src/mesh.cpp:514-537). */
int nosh_mesh_edge_gids_complex(nosh_mesh mesh, int32_t *idx);
/* Edge lengths and covolumes: mesh::get_edge_data (src/mesh.hpp:256-259). */
int nosh_mesh_edge_data(nosh_mesh mesh, double *length, double *covolume);
/* Control volumes (N): mesh::control_volumes (src/mesh.hpp:250-252). */
int nosh_mesh_control_volumes(nosh_mesh mesh, double *cv);
/* KEO graph in complex (2x2-block) form: row_ptr[N+1], cols[N+2E], sorted
 * columns, diagonal included.  Expanding each block into 2x2 real entries
 * gives mesh::build_complex_graph (src/mesh.cpp:789-882). */
int nosh_mesh_complex_graph(nosh_mesh mesh, int32_t *row_ptr, int32_t *cols);

/* ------------------------------------------------------ model evaluator */
/* nosh::model_evaluator::nls constructor (src/model_evaluator_nls.cpp:57-138)
 * together with its fields:
 *   mvp              3*N doubles: vector potential sampled per vertex, as
 *                    vector_field::explicit_values(mesh, "A", mu)
 *                    (src/vector_field_explicit_values.cpp:14-50);
 *   scalar_potential N doubles, V (scalar_field::explicit_values /
 *                    constant, src/scalar_field_constant.cpp:45-58);
 *   thickness        N doubles (likewise);
 *   g, mu            initial parameter values;
 *   deriv_parameter  "mu" or "g": the parameter DkeoDP differentiates by
 *                    (src/parameter_matrix_dkeo_dp.cpp:29-45).
 * The mesh must outlive the nls handle. */
int nosh_nls_create(nosh_mesh mesh, const double *mvp, double mu,
                    const double *scalar_potential, double g,
                    const double *thickness, const char *deriv_parameter,
                    nosh_nls *out);
int nosh_nls_destroy(nosh_nls nls);
/* Number of parameters and their sorted names (get_p_names,
 * src/model_evaluator_nls.cpp:196-205); name buffer gets a NUL-terminated
 * string. */
int nosh_nls_num_params(nosh_nls nls, int *num);
int nosh_nls_param_name(nosh_nls nls, int index, char *buf, size_t len);
/* Precision of J/K_reg applies and of the Krylov solver: NOSH_PREC_*. */
int nosh_nls_set_precision(nosh_nls nls, int precision);
int nosh_nls_get_precision(nosh_nls nls, int *precision);
/* Preconditioner options (the MueLu parameter list of
 * src/keo_regularized.cpp:296-315): maximum levels, coarsest size (nodes per
 * system), Chebyshev degree of pre- and post-smoothing, the reuse period
 * (numeric refreshes between two full Galerkin refreshes: 1 = every level
 * at every rebuild; the ones in between update the fine level only, like
 * MueLu "reuse: type full"), the strength threshold of the aggregation and
 * the Chebyshev eigenvalue ratio (smoothing interval [lmax / ratio,
 * 1.1 lmax]).  Defaults 10, 64, 2, 8 and, from sweeps, 0 and 15 on
 * tetrahedral meshes, 0.05 and 30 on triangular ones (a batched union of
 * many squares solved 12 % faster at threshold 0).  A connection (i, j) is
 * strong when |K_ij| >= threshold sqrt(d_i d_j), d_i the mean of the two
 * diagonal entries of the regularised operator's block at vertex i, at the
 * state of the first rebuild.  Drops the
 * current hierarchy; the next rebuild builds a new one. */
int nosh_nls_set_amg_options(nosh_nls nls, int max_levels, int coarse_size,
                             int smooth_degree, int reuse_period,
                             double strength_threshold, double cheb_ratio);
/* Batched independent solves (many meshes in one handle): the handle's
 * mesh is the disjoint union of num_systems meshes, system s owning the
 * vertices [vertex_offsets[s], vertex_offsets[s+1]) (no edge may join two
 * systems).  System s uses mu[s] in its KEO; the mu entry of the parameter
 * vector is then unused.  Every kernel runs over all systems at once, the
 * residual norms are per system (one CTA each), a Newton solve ends when
 * every system reaches ||F_s|| <= tol (stats->f_norm is the largest) and
 * converged systems receive zero Newton updates.  The AMG hierarchy keeps
 * systems apart (its coarsest level is block diagonal, one dense block per
 * system).  Continuation handles reject a batched handle: the gauge phase of
 * each system is its own. */
int nosh_nls_set_systems(nosh_nls nls, int64_t num_systems,
                         const int64_t *vertex_offsets, const double *mu);
/* Per-system Newton steps and MINRES iterations of the last Newton solve
 * (num_systems entries each; either pointer may be NULL).  Every system
 * runs its own MINRES recurrence; the batch's Krylov test is the union's
 * residual.  No counterpart in the reference (one nls per system there). */
int nosh_nls_system_iterations(nosh_nls nls, int *newton_iters, int *krylov_iters);
/* Per-system ||F_s||_2 of the last residual a Newton solve evaluated. */
int nosh_nls_system_norms(nosh_nls nls, double *norms);
/* The preconditioner hierarchy (after the first rebuild): number of
 * levels, their sizes (nodes; up to max_sizes entries) and the first level
 * run by the single-CTA tail kernel.  num_levels is 0 before the first
 * rebuild. */
int nosh_nls_amg_levels(nosh_nls nls, int *num_levels, int64_t *sizes,
                        int max_sizes, int *tail_level);
/* SpMV schedule of the handle's operators: NOSH_SPMV_AUTO (default: each
 * matrix times both schedules once and keeps the staged one unless the warp
 * schedule is at least 10 % faster), NOSH_SPMV_STAGED
 * (128-row blocks staged into shared memory by bulk copies) or
 * NOSH_SPMV_WARP (warp-cooperative, a half-warp per row).  Drops the
 * preconditioner hierarchy. */
#define NOSH_SPMV_AUTO 0
#define NOSH_SPMV_STAGED 1
#define NOSH_SPMV_WARP 2
int nosh_nls_set_spmv_schedule(nosh_nls nls, int schedule);
/* Newton's forcing (no counterpart in the reference, whose NOX forcing is
 * constant, examples/conf.xml:81): the Eisenstat-Walker term is never tighter
 * than what reaches the target in one step, eta >= aim * target / ||F||;
 * `aim` in (0, 1] is the fraction of the target a step aims at (default
 * 0.5; a larger aim takes fewer Krylov iterations per step and risks a
 * second Newton step). */
int nosh_nls_set_forcing_aim(nosh_nls nls, double aim);
/* Launch overlap (no counterpart in the reference): the kernels of a MINRES
 * iteration and of the V-cycle are launched with programmatic stream
 * serialisation, so each one is scheduled as its predecessor's CTAs exit,
 * before that kernel's completion is signalled, and waits on the device for
 * its predecessor's results before it reads them.  On by default; 0
 * launches them one after the other (for timing comparisons).  Drops the
 * preconditioner hierarchy and the captured MINRES graphs. */
int nosh_nls_set_launch_overlap(nosh_nls nls, int enable);
/* Diagnostics (no counterpart in the reference, whose Tpetra SpMV has no
 * bounded wait): the bound, in mbarrier polls, of the waits of the staged
 * SpMV schedule for the copies of its matrix rows into shared memory; the
 * default is 2^20, and polls < 0 restores it.  A wait that runs out leaves
 * its launch early and flags it; the call that ran that launch returns
 * NOSH_ERR_CUDA at its next synchronisation, and the handle stays usable.
 * polls = 0 makes every staged wait give up at once (tests of that path). */
int nosh_nls_set_stage_wait_limit(nosh_nls nls, int64_t polls);
/* Index-check mode (the reference's debug builds assert sizes on the host,
 * e.g. src/jacobian_operator.cpp:68-86; there is no device counterpart).
 * With enable != 0 the handle validates its KEO graph on the device before
 * every Newton solve, continuation step and operator apply of this ABI (and
 * once now): row ranges in order and within the entry count, column ids in
 * [0, N), off the diagonal and increasing along each row.  The first
 * offence is recorded in a device word (no trap, no out-of-range access)
 * and the call returns NOSH_ERR_INVALID naming its position.  Costs one
 * pass over the index arrays per call. */
int nosh_nls_set_index_checks(nosh_nls nls, int enable);
/* The same validation for a caller's off-diagonal CSR graph in device
 * memory (row_ptr[N+1], cols[nnz]), e.g. the one passed to
 * nosh_residual_norm_noalloc, which cannot read it on the host.  NOSH_OK or
 * NOSH_ERR_INVALID with the position of the first offence; work on
 * `stream`, waited for. */
int nosh_graph_check(int64_t num_vertices, int64_t nnz, const int32_t *row_ptr,
                     const int32_t *cols, void *stream);
/* Diagnostics (no counterpart in the reference): the achievable-bandwidth
 * probe.  Enqueues on `stream` one launch that streams `bytes` (a multiple
 * of 16) of the 16-byte aligned device buffer `buf` with 16-byte loads and
 * XOR-folds them into the 32-bit device word *out_word.  Timing it beside a
 * kernel that moves the same bytes shows what a single launch of that size
 * reaches at all on this GPU. */
int nosh_diag_stream_read(const void *buf, int64_t bytes, void *out_word, void *stream);
/* The CUDA stream the handle's work runs on (a cudaStream_t). */
int nosh_nls_stream(nosh_nls nls, void **stream);

/* F(x) at parameters p: nls::evalModelImpl with out_args.f set
 * (src/model_evaluator_nls.cpp:445-461) -> compute_f_ (:529-628).  FP64. */
int nosh_nls_compute_f(nosh_nls nls, const double *x, const double *p,
                       double *f);
/* Same, plus ||F||_2 (FP64 reduction) written to *norm (may be NULL). */
int nosh_nls_compute_f_norm(nosh_nls nls, const double *x, const double *p,
                            double *f, double *norm);
/* dF/dp for every parameter (num_params columns of 2N, column-major):
 * out_args.DfDp by column (src/model_evaluator_nls.cpp:463-489) ->
 * computeDFDP_ (:632-695). */
int nosh_nls_compute_dfdp(nosh_nls nls, const double *x, const double *p,
                          double *dfdp);
/* -sum cv |psi|^4 / sum cv: the value nls::gibbs_energy computes before its
 * "return 0.0" (src/model_evaluator_nls.cpp:742-770). */
int nosh_nls_gibbs_energy(nosh_nls nls, const double *psi, double *out);
/* sum cv (Re phi Re psi + Im phi Im psi) / sum cv (nls::inner_product,
 * src/model_evaluator_nls.cpp:699-738, normalised as its comment states). */
int nosh_nls_inner_product(nosh_nls nls, const double *phi, const double *psi,
                           double *out);

/* ---------------------------------------------------- parameter matrices */
/* keo::set_parameters -> refill_ (src/parameter_object.cpp:7-47,
 * src/parameter_matrix_keo.cpp:76-184): edge-parallel KEO assembly into the
 * device CSR at p ("mu" used).  Fills FP64 and FP32 copies. */
int nosh_keo_set_parameters(nosh_nls nls, const double *p);
/* Current KEO values in nosh_mesh_complex_graph order, complex interleaved
 * (2*(N+2E) doubles): one value z per 2x2 block [[Re z, -Im z], [Im z, Re z]]
 * (the blocks of src/parameter_matrix_keo.cpp:155-160). */
int nosh_keo_values(nosh_nls nls, double *vals);
/* Y = K X (Tpetra::CrsMatrix::apply as used at
 * src/model_evaluator_nls.cpp:537), FP64. */
int nosh_keo_apply(nosh_nls nls, const double *x, double *y);
/* DkeoDP::set_parameters -> refill_ (src/parameter_matrix_dkeo_dp.cpp:
 * 62-155), values and apply, as for the KEO. */
int nosh_dkeo_set_parameters(nosh_nls nls, const double *p);
int nosh_dkeo_values(nosh_nls nls, double *vals);
int nosh_dkeo_apply(nosh_nls nls, const double *x, double *y);

/* ---------------------------------------------------- jacobian operator */
/* jacobian_operator::rebuild (src/jacobian_operator.cpp:112-141): KEO refill
 * at p and the diagonal blocks from x (rebuild_diags_, :145-200). */
int nosh_jacobian_rebuild(nosh_nls nls, const double *p, const double *x);
/* jacobian_operator::apply (src/jacobian_operator.cpp:40-108) on
 * num_vectors columns of 2N (column-major).  Like the reference, only
 * mode = NOSH_NO_TRANS, alpha = 1, beta = 0 are accepted
 * (NOSH_ERR_UNSUPPORTED otherwise).  Runs in the handle's precision. */
int nosh_jacobian_apply(nosh_nls nls, const double *X, double *Y,
                        int num_vectors, int mode, double alpha, double beta);

/* -------------------------------------------------------- preconditioner */
/* keo_regularized::rebuild (src/keo_regularized.cpp:183-264): regularised
 * KEO K + g cv t [[2|x|^2+gamma, beta], [beta, 2|x|^2-gamma]] and its
 * aggregation-AMG hierarchy (the reference builds a MueLu SA-AMG,
 * :292-336). */
int nosh_keo_regularized_rebuild(nosh_nls nls, const double *p,
                                 const double *x);
/* keo_regularized::apply (src/keo_regularized.cpp:90-165): one V-cycle
 * (num_cycles == 1).  mode/alpha/beta as for nosh_jacobian_apply. */
int nosh_keo_regularized_apply(nosh_nls nls, const double *X, double *Y,
                               int num_vectors, int mode, double alpha,
                               double beta);
/* y = the fine level's Chebyshev smoothing sweep of the preconditioner,
 * from a zero initial guess on right-hand side x: y = p(D^-1 K_reg) D^-1 x,
 * D the 2x2 diagonal blocks of K_reg and p the Chebyshev polynomial of the
 * smoothing degree on [lmax / ratio, 1.1 lmax] (lmax a Gershgorin bound of
 * D^-1 K_reg).  In the handle's precision.  For checking: MueLu's smoother
 * inside the reference's V-cycle (src/keo_regularized.cpp:296-315) has no
 * call of its own.  Needs a hierarchy of two levels or more. */
int nosh_keo_regularized_smoother_apply(nosh_nls nls, const double *x,
                                        double *y);
/* The k smallest eigenvalues of the FP64 Jacobian J(psi, p) and their unit
 * eigenvectors: the stability test of a state, the role of Anasazi in the
 * reference's eigen tool (executables/nosh-eig/nosh-eig.cpp:57-) and of the
 * continuation's eigen analysis (examples/conf.xml:50-66).  LOBPCG on the
 * GPU with one AMG V-cycle of the regularised KEO as preconditioner; with
 * deflate_gauge the U(1) gauge mode i psi is projected out, so the values
 * are the physical ones.  guard: extra block vectors (< 0: max(2, k));
 * 3 (k + guard) <= 64.  Convergence: ||J x - lambda x|| <= tol * ||J||_est
 * for each of the k pairs, within maxit iterations (the estimates reached
 * are returned either way; compare *iterations with maxit).
 *   eigenvalues[k] (host, ascending); eigenvectors[k * 2N] (host or device,
 *   NULL to skip); seed: the random start block (splitmix64). */
int nosh_eig_lowest(nosh_nls nls, const double *psi, const double *p, int k,
                    double tol, int maxit, int guard, int deflate_gauge,
                    uint64_t seed, double *eigenvalues, double *eigenvectors,
                    int *iterations);
/* Y = K_reg X (the regularised operator itself, for checking). */
int nosh_keo_regularized_operator_apply(nosh_nls nls, const double *x,
                                        double *y);

/* ------------------------------------------------------------- solvers */
typedef struct {
  double tol;             /* ||F||_2 target (NOX NormF, examples/conf.xml:
                             178-189); default 1e-10                      */
  int max_newton;         /* NOX MaxIters (conf.xml:186-189); default 20  */
  double forcing;         /* relative MINRES tolerance per Newton step;
                             <= 0 selects Eisenstat-Walker "Type 1"
                             (sampleScripts/conf-parallel.xml:78)         */
  int max_krylov;         /* per linear solve; default 1000 (conf.xml:127)*/
  int precision;          /* NOSH_PREC_*                                  */
  int verbose;            /* 0 = silent                                   */
  double refine;          /* 0 (default) or a residual norm <= tol that
                             the solve aims at: a state with ||F|| above
                             4 refine gets at least one Newton step, whose
                             Eisenstat-Walker forcing aims at refine, and
                             iteration continues while ||F|| > tol.
                             States converged well below tol keep
                             high-order continuation predictors at their
                             truncation error                             */
  int phase_fix;          /* 0 (default) or 1: every Newton update is made
                             orthogonal to i psi, the U(1) gauge direction
                             (J(i psi) = i F).  This is the solution the
                             reference's bordered system gives,
                             [J, i psi; (i psi)^T, 0]
                             (src/bordering/ModelEvaluator_Bordered.cpp:
                             187-283): F is orthogonal to i psi, so the
                             border only removes the null direction     */
} nosh_newton_options;

typedef struct {
  int newton_iters;
  int krylov_iters;       /* total over the Newton steps                  */
  double f_norm;          /* final ||F||_2                                */
  double f_norm0;         /* initial ||F||_2                              */
  int status;             /* NOSH_OK / NOSH_ERR_NOT_CONVERGED / ...       */
  int residual_updates;   /* mixed path: Newton residuals evaluated from
                             the previous one's FP64 off-diagonal sums and
                             an FP32 product of the (small) update instead
                             of afresh; each deviates from the FP64
                             evaluation by at most the bound below, and is
                             only kept when it decides convergence with that
                             margin                                       */
  double f_norm_bound;    /* bound on |f_norm - FP64 ||F||_2| (0 when the
                             final residual was evaluated afresh)         */
} nosh_newton_stats;

/* Fills the defaults above. */
void nosh_newton_default_options(nosh_newton_options *opt);
/* Full-step inexact Newton with KEO-regularised-AMG-preconditioned MINRES
 * (NOX "Line Search Based" + "Full Step", examples/conf.xml:77-191; Belos
 * MINRES, test/linear-solve-test/linop-tester.cpp:288).  x is the initial
 * guess on entry and the solution on return. */
int nosh_newton_solve(nosh_nls nls, double *x, const double *p,
                      const nosh_newton_options *opt,
                      nosh_newton_stats *stats);

/* ---------------------------------------------------------- continuation */
#define NOSH_PREDICT_NONE 0    /* x(mu_new) = x(mu_cur)                      */
#define NOSH_PREDICT_SECANT 1  /* LOCA "Secant" (examples/conf.xml:39-41)    */
#define NOSH_PREDICT_TANGENT 2 /* LOCA "Tangent": x + dmu * (-J^-1 dF/dmu)   */
#define NOSH_PREDICT_QUADRATIC 3 /* 3-point polynomial extrapolation       */
#define NOSH_PREDICT_LEARNED 4   /* edge message-passing network on top of the
                                    secant, trained online; falls back to the
                                    secant when its residual is larger       */
#define NOSH_PREDICT_CUBIC 5     /* 4-point polynomial extrapolation       */

/* One natural-parameter continuation step (LOCA stepper semantics,
 * examples/conf.xml:35-75; driven by executables/nosh-cont/nosh-cont.cpp:
 * 226-345): predict the state at p_new[1] = mu_new from the states at
 * mu_cur and mu_prev, then Newton-correct it to opt->tol.
 *   x       in: x(mu_cur)             out: x(mu_new)
 *   x_prev  in: x(mu_prev)            out: x(mu_cur)     (secant only; may be
 *           NULL for the other predictors)
 * Predicted states are aligned in global phase first (the solutions are
 * defined up to the U(1) gauge psi -> e^{i phi} psi).  stats->f_norm0 is the
 * residual of the prediction. */
int nosh_continuation_step(nosh_nls nls, double *x, double *x_prev,
                           const double *p_new, double mu_cur, double mu_prev,
                           int predictor, const nosh_newton_options *opt,
                           nosh_newton_stats *stats);

/* A device-resident continuation run: the handle keeps the last converged
 * states (and the learned predictor) in HBM, so a step moves no state
 * through the host.  Same stepper semantics as nosh_continuation_step.
 * x0 is the converged state at mu0 (host or device). */
typedef struct nosh_continuation_s *nosh_continuation;
int nosh_continuation_create(nosh_nls nls, const double *x0, double mu0,
                             nosh_continuation *out);
int nosh_continuation_destroy(nosh_continuation c);
/* One natural step to mu_new with the given predictor (NOSH_PREDICT_*);
 * the polynomial predictors fall back to lower order while the history is
 * short.  stats->f_norm0 is the residual of the prediction actually used. */
int nosh_continuation_advance(nosh_continuation c, double mu_new, int predictor,
                              const nosh_newton_options *opt,
                              nosh_newton_stats *stats);
/* The current state (2N doubles, host or device) and its mu. */
int nosh_continuation_state(nosh_continuation c, double *x, double *mu);
/* One pseudo-arclength step (LOCA "Arc Length", examples/conf.xml:43) of
 * length ds in the norm ||(x, m)||^2 = x.x / (2N) + theta^2 m^2.  The unit
 * tangent at the current state is the TANGENT one (-J^-1 dF/dmu, mu
 * component 1, its U(1) gauge component removed) or the phase-aligned
 * SECANT of the last two states; it is oriented along the last secant (the
 * first step: towards larger mu for ds > 0).  The corrector is Newton on F
 * and the arclength constraint, solved by bordering (two MINRES solves per
 * Newton step with the same operators) in FP64 whatever the handle's
 * precision, at the relative tolerance opt->forcing, or 1e-8 when it is
 * <= 0: near a fold only the combination of the two solutions is small,
 * and looser or FP32 solves miss the fold.  On success the new state becomes
 * current (read mu with nosh_continuation_state); on failure the current
 * state is unchanged and the return code is the Newton status. */
int nosh_continuation_advance_arclength(nosh_continuation c, double ds,
                                        int predictor, double theta,
                                        const nosh_newton_options *opt,
                                        nosh_newton_stats *stats);
/* The mu component of the last unit arclength tangent (dmu/ds; its sign
 * flips past a fold) and the theta it was normalised with. */
int nosh_continuation_tangent(nosh_continuation c, double *tau_mu,
                              double *theta);
/* Learned predictor: creates the network (its readout starts at the cubic
 * extrapolation) and trains it online on the transitions of the next
 * `train_steps` steps, `iters_per_step` Adam iterations each, the step size
 * decaying linearly from `learning_rate` over the window.  NOSH_PREDICT_
 * LEARNED predicts with it once four states are known. */
int nosh_continuation_learning(nosh_continuation c, int train_steps,
                               int iters_per_step, double learning_rate);
/* After the training window the network's coefficient for the next learned
 * step is inferred on a second stream while the current step's Newton solve
 * runs.  With period p > 1 it is re-inferred on every p-th learned step
 * only and reused in between (default 1).  No counterpart in the reference
 * (its LOCA predictors have no network). */
int nosh_continuation_inference_period(nosh_continuation c, int period);
/* Diagnostics: ||F||_2 at mu_new of the secant, quadratic, cubic and learned
 * predictions (residuals[0..3]) formed from the handle's current history,
 * without advancing it (NaN where a predictor lacks history or the network
 * is not enabled).  The learned one uses a coefficient inferred from these
 * very features. */
int nosh_continuation_predictor_residuals(nosh_continuation c, double mu_new,
                                          double *residuals);
/* Predictor telemetry: which predictor the last advance used
 * (NOSH_PREDICT_*), the learned prediction's residual and the secant one's
 * (NaN when not evaluated: the secant is evaluated whenever the learned
 * prediction misses the tolerance, and the one with the smaller residual
 * starts Newton), the last training loss, and the learned coefficient w of
 * the last learned prediction (NaN if none). */
int nosh_continuation_last_prediction(nosh_continuation c, int *used,
                                      double *f_learned, double *f_secant,
                                      double *train_loss, double *coef);

/* The learned predictor's network, for inspection and gradient checks (the
 * continuation handle owns its own instance).  From the four newest states
 * it predicts one global coefficient w and the prediction is
 * quadratic + w c, c = cubic - quadratic extrapolation (w = 1 is the cubic
 * extrapolation, where the readout starts).  Parameters are one flat FP32
 * vector: encoder W [10x64] (row-major), b [64]; per layer l = 0..2:
 * W_a [64x64], W_b [64x64], W_c [4x64], b_m [64], W_u [128x64], b_u [64];
 * readout W_1 [64x32], b_1 [32], W_2 [32x1], b_2 [1].  Node features are
 * N x 10, edge features 2E x 4 in the order of the off-diagonal KEO graph
 * (the complex graph of nosh_mesh_complex_graph without its diagonal). */
typedef struct nosh_mpnn_s *nosh_mpnn;
int nosh_mpnn_create(nosh_nls nls, nosh_mpnn *out);
int nosh_mpnn_destroy(nosh_mpnn net);
int nosh_mpnn_num_params(nosh_mpnn net, int64_t *n);
/* copies the parameters out (get != NULL) and/or in (set != NULL) */
int nosh_mpnn_params(nosh_mpnn net, float *get, const float *set);
int nosh_mpnn_edge_features(nosh_mpnn net, float *ef);
/* the readout coefficient *w for node features X (N x 10) */
int nosh_mpnn_forward(nosh_mpnn net, const float *X, double *w);
/* the training loss (w^2 cc - 2 w cd + dd) / dd for Gram scalars gram =
 * [cc, cd, dd] (online training uses those of Jc and Jd: c = cubic -
 * quadratic, d = target - quadratic, J the Jacobian at the target, so the
 * loss is the linearised residual of the prediction relative to the
 * quadratic's), and its parameter gradient; the parameters are not
 * changed */
int nosh_mpnn_loss_grad(nosh_mpnn net, const float *X, const double *gram,
                        double *loss, float *grad);

/* ------------------------------------------------------ kernel timing */
#define NOSH_KERNEL_JACOBIAN 0 /* fine-level Jacobian apply (MINRES)       */
#define NOSH_KERNEL_SMOOTHER 1 /* fine-level AMG smoothing/residual SpMVs  */
#define NOSH_KERNEL_ALL 2      /* every kernel the handle launched (count
                                  only; always on)                         */
/* While enabled, every launch of the fine-level SpMV kernels is bracketed
 * by CUDA events on the handle's stream.  Inside a MINRES solve the launches
 * run from its captured graphs (captured anew when timing is switched), the
 * events are event-record nodes of those graphs, and only the launches that
 * did work are counted (not those that return at once after convergence
 * inside a captured part). */
int nosh_nls_profile_enable(nosh_nls nls, int enable);
/* Launch count, summed device time and summed algorithmic bytes (the bytes
 * the kernel must move at minimum: matrix, indices and the vectors it reads
 * and writes, once each) of one kernel class since the last read; resets
 * the counters.  For
 * NOSH_KERNEL_ALL only the launch count is returned. */
int nosh_nls_profile_read(nosh_nls nls, int kernel, int64_t *launches,
                          double *total_ms, double *bytes);

/* ------------------------------------------------ allocation-free residual */
/* F(psi) and ||F||_2 for callers that cannot allocate device memory: code
 * that runs inside a host framework owning the whole device memory pool,
 * plugins held to a fixed memory budget, or loops that must not pay the
 * implicit device synchronisation of cudaMalloc / cudaFree.  It has no
 * counterpart in the reference (whose F is compute_f_, reached through an
 * nls handle that owns its buffers).
 *
 * Every array is caller-owned device memory of the current device:
 *   row_ptr[N+1], cols[2E]  off-diagonal KEO graph (the complex graph of
 *                           nosh_mesh_complex_graph without the diagonal)
 *   keo_offdiag[2*2E]       its complex values (16-byte aligned)
 *   keo_diag[N]             real KEO diagonal, sum of the incident edge
 *                           coefficients
 *   cv_thickness[N], scalar_potential[N], g
 *   psi[2N] (in), f[2N] (out)  interleaved complex, 16-byte aligned
 *   norm[1] (out)           ||F||_2
 * Memory of another GPU, or host memory, is rejected with NOSH_ERR_INVALID;
 * managed memory is accepted.
 * The call cannot read the graph arrays on the host, so they must already be
 * a valid CSR: row_ptr non-decreasing with row_ptr[0] = 0 and row_ptr[N] =
 * the number of entries, and every cols[k] in [0, N).  Any other graph reads
 * out of bounds (undefined behaviour).  nosh_mesh_complex_graph with its
 * diagonal entries removed gives one that meets this.
 * The work is enqueued on `stream` (a cudaStream_t, NULL = default stream)
 * and the call returns without waiting for it.
 *
 * Limit: N <= 8,388,608 vertices (65,536 CTAs of 128 rows).  The reduction's
 * scratch is one fixed 512 KiB __device__ array inside the library, which
 * every GPU that loads the library holds until the process exits; larger
 * meshes are rejected with NOSH_ERR_INVALID (use nosh_nls_compute_f_norm).
 * The first call on a device looks up that array's device address, so make
 * the first call on each device before any stream capture.  All calls share
 * the one array: calls that overlap on the GPU (other streams, other host
 * threads) race and give wrong norms; serialise them.  No device memory is
 * allocated or freed by this call. */
int nosh_residual_norm_noalloc(int64_t num_vertices, const int32_t *row_ptr,
                               const int32_t *cols, const double *keo_offdiag,
                               const double *keo_diag,
                               const double *cv_thickness,
                               const double *scalar_potential, double g,
                               const double *psi, double *f, double *norm,
                               void *stream);

#ifdef __cplusplus
}
#endif
#endif /* NOSH_GB300_H */
