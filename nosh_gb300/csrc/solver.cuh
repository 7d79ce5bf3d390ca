// Krylov / Newton solvers (solver.cu).
#pragma once

#include "amg.cuh"
#include "nls.cuh"

namespace nosh {

// MINRES recurrence state, resident in device memory (FP64 scalars).
struct MinresScalars {
  double beta1, beta, oldb, alfa, dbar, epsln, oldeps, phibar, phi, cs, sn, gamma, delta;
  double zu, rz;  // reduction slots: <z, J z>, <r, M r>
  int itn, done, flag, maxit;
  double rtol;
};

// Preconditioned MINRES (Paige-Saunders) on J dx = b with the AMG V-cycle as
// the SPD preconditioner, vectors in T, scalars in FP64.
template <typename T>
struct Minres {
  NlsImpl &s;
  int64_t n2;  // real length (2N)
  DevBuf<T> r1, r2, z0, z1, u, w0, w1, w2, x;
  DevBuf<MinresScalars> sc;
  MinresScalars *h_sc = nullptr;  // pinned host mirror
  explicit Minres(NlsImpl &nls);
  ~Minres();
  // b: device vector of T (2N); returns iterations; x holds the solution
  int solve(const T *b, double rtol, int maxit, int &status, double &rel_res);
};

void newton_solve(NlsImpl &s, double *x_user, double g, double mu,
                  const nosh_newton_options &opt, nosh_newton_stats &st);
void continuation_step(NlsImpl &s, double *x, double *x_prev, double g, double mu_new,
                       double mu_cur, double mu_prev, int predictor,
                       const nosh_newton_options &opt, nosh_newton_stats &st);

}  // namespace nosh
