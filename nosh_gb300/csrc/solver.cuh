// Krylov / Newton solvers (solver.cu).
#pragma once

#include "amg.cuh"
#include "minres_state.cuh"
#include "nls.cuh"

namespace nosh {

// Preconditioned MINRES (Paige-Saunders) on J dx = b with the AMG V-cycle as
// the SPD preconditioner, vectors in T, scalars in FP64 (minres_state.cuh).
// Buffer roles repeat every kChunk iterations; the chunk is captured once as
// kParts CUDA graphs of kPart iterations (replayed in turn).  A solve
// launches as many parts as the previous solve needed before the host first
// polls the convergence flag, then one at a time; launches after
// convergence return at once (each such iteration still costs its kernels'
// launches, so parts are kept short).
template <typename T>
struct Minres {
  static constexpr int kChunk = 6;  // multiple of the 2- and 3-buffer rotations
  static constexpr int kParts = 3;
  static constexpr int kPart = kChunk / kParts;
  NlsImpl &s;
  int64_t n2;  // real length (2N)
  DevBuf<T> r[2], z[2], w[3], u, x;
  DevBuf<MinresScalars> sc;
  MinresScalars *h_sc = nullptr;  // pinned host mirror
  int *h_err = nullptr;
  cudaGraphExec_t part_exec[kParts] = {};
  // the captured prologue (initial V-cycle and recurrence set-up) for the
  // right-hand side pro_b; rtol and maxit reach it through `params`
  cudaGraphExec_t pro_exec = nullptr;
  const T *pro_b = nullptr;
  int64_t pro_kernels = 0;
  DevBuf<double> params;
  double *h_params = nullptr;
  int64_t part_kernels[kParts] = {};
  int last_its = 0;  // iterations of the previous solve
  // Kernel timing (the handle's timers on): the graphs are captured with
  // event-record nodes around the timed launches; the pairs of each
  // iteration of each part (per timer) and of the prologue, harvested after
  // a replay for the launches that did work
  bool graphs_timed = false;
  std::vector<KernelTimer::Pair> part_ev[kParts][kPart][2];
  std::vector<KernelTimer::Pair> pro_ev[2];
  explicit Minres(NlsImpl &nls);
  ~Minres();
  // b: device vector of T (2N); returns iterations; x holds the solution
  int solve(const T *b, double rtol, int maxit, int &status, double &rel_res);

 private:
  void iteration(int j);   // issue iteration j (0..kChunk-1) of a chunk
  void wx_final(int j);    // deferred w/x update of iteration j, the last issued
  void drop_graphs();
};

// Batched independent solves: one Paige-Saunders recurrence per system
// over the shared vectors (minres_sys.cu).
template <typename T>
struct MinresSys {
  NlsImpl &s;
  int64_t N, S;
  DevBuf<T> r[2], z[2], w[3], u, x;
  DevBuf<double> rowdot, cpart, rtol;
  DevBuf<MinresScalars> sc;
  DevBuf<int32_t> vsys, csys, schunk;
  DevBuf<int64_t> cstart;
  DevBuf<unsigned> counter;
  DevBuf<int> active;
  int nchunks = 0;
  std::vector<MinresScalars> h_sc;
  int *h_active = nullptr, *h_err = nullptr;
  double *h_eta = nullptr;
  DevBuf<double> eta;  // the batch's tolerance (read by the captured chunk)
  cudaGraphExec_t chunk_exec = nullptr;
  int64_t chunk_kernels = 0;
  int chunk_maxit = -1;
  explicit MinresSys(NlsImpl &nls);
  ~MinresSys();
  // b: device vector of T (2N); eta: the batch's relative tolerance (the
  // union's preconditioned residual); rtol: per system (a system stops early
  // at its own); its: iterations per system; returns the largest; x holds
  // the solution
  int solve(const T *b, double eta, const std::vector<double> &rtol, int maxit, std::vector<int> &its,
            int &status);

 private:
  void reduce(int mode, int maxit);
  void iteration(int j, int maxit);
};

// Newton work space of an nls handle (solver.cu)
struct NewtonState {
  DevBuf<double> psi, f, xc, xp, tmp;  // working state, residual, staged inputs
  DevBuf<float> b32;
  DevBuf<double> b64;
  DevBuf<double> red2;  // complex reduction (phase alignment)
  std::unique_ptr<Minres<float>> m32;
  std::unique_ptr<Minres<double>> m64;
  std::unique_ptr<MinresSys<float>> s32;
  std::unique_ptr<MinresSys<double>> s64;
  // batched solves: per-system Newton steps and MINRES iterations of the
  // last Newton solve
  std::vector<int> sys_newton, sys_krylov;
  // off-diagonal sums of K psi (FP64, 2N) for the current psi at soff_mu,
  // kept by the mixed-precision Newton steps (residual_update); soff_alt
  // holds a second candidate's (the learned step's two predictions)
  // the FP32 operators (diagonal blocks, preconditioner) already built for
  // this state buffer at (ops_g, ops_mu) by prebuild_operators32; the next
  // mixed-precision Newton step from it skips its first rebuild
  const double *ops_state = nullptr;
  double ops_g = 0.0, ops_mu = 0.0;
  DevBuf<double> soff, soff_alt;
  bool soff_valid = false, soff_fresh = false;  // fresh: from an FP64 evaluation, no update since
  double soff_mu = 0.0;
  void ensure_soff(int64_t n2) {
    if (soff.n < (size_t)n2) soff.alloc(n2);
    if (soff_alt.n < (size_t)n2) soff_alt.alloc(n2);
  }
};
NewtonState &state_of(NlsImpl &s);
// drop the AMG hierarchy (and the MINRES graphs that reference it); the next
// rebuild constructs it from the current options
void reset_preconditioner(NlsImpl &s);
// the AMG hierarchy with the handle's options, created when missing
Amg &ensure_preconditioner(NlsImpl &s);
// ||F(psi)||_2 (writes F into f; synchronises)
double residual_norm(NlsImpl &s, const double *psi, double g, double mu, double *f);
// Newton on state_of(s).psi in place.  With f0 >= 0, ns.f already holds
// F(psi) and f0 is its norm (no re-evaluation), and soff_ready says whether
// ns.soff holds the off-diagonal sums of K psi as well.
void newton_core(NlsImpl &s, NewtonState &ns, double g, double mu, const nosh_newton_options &opt,
                 nosh_newton_stats &st, double f0 = -1.0, bool soff_ready = false);

// The mixed-precision Newton step's operators at (psi, g, mu), enqueued
// ahead (e.g. while the host waits for a residual): psi must be the buffer
// that is ns.psi when newton_core runs.
void prebuild_operators32(NlsImpl &s, NewtonState &ns, const double *psi, double g, double mu);

// Relative MINRES tolerance of Newton step `it` (fixed forcing, else
// safeguarded Eisenstat-Walker), floored at what the Krylov precision resolves.
double forcing_term(const nosh_newton_options &opt, int it, double fn, double fn_prev, bool fp32,
                    double aim = 0.5);

// J(ns.psi, g, mu) x = rhs (2N reals, FP64 in/out) by preconditioned MINRES
// in `precision`; rebuilds the operators at (ns.psi, mu) when asked.
// Returns the iterations; status as Minres::solve.
int linear_solve(NlsImpl &s, NewtonState &ns, const double *rhs, double *x, double g, double mu, double rtol,
                 int maxit, int precision, bool rebuild, int &status);

// The k smallest eigenvalues of the FP64 Jacobian at psi (device, 2N) by
// LOBPCG with the AMG preconditioner, the gauge mode deflated (eig.cu);
// values[k] on the host, vectors (k x 2N, host or device) when non-null.
// guard < 0: max(2, k) extra block vectors.  Returns the iterations.
int lowest_eigenpairs(NlsImpl &s, const double *psi_dev, double g, double mu, int k, double tol, int maxit,
                      int guard, bool deflate_gauge, uint64_t seed, double *values, double *vectors);

void newton_solve(NlsImpl &s, double *x_user, double g, double mu,
                  const nosh_newton_options &opt, nosh_newton_stats &st);
void continuation_step(NlsImpl &s, double *x, double *x_prev, double g, double mu_new,
                       double mu_cur, double mu_prev, int predictor,
                       const nosh_newton_options &opt, nosh_newton_stats &st);

}  // namespace nosh
