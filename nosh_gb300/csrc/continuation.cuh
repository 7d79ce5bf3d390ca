// Device-resident continuation run (continuation.cu).
#pragma once

#include <memory>

#include "solver.cuh"

namespace nosh {

struct Mpnn;  // learned predictor (mpnn.cu)

struct ContinuationImpl {
  static constexpr int kHist = 5;  // newest converged states kept in HBM
  // relative MINRES tolerance of the arclength corrector's solves
  static constexpr double kArclengthForcing = 1e-8;
  NlsImpl &s;
  DevBuf<double> hist[kHist];
  double mu[kHist] = {0, 0, 0, 0, 0};
  int head = 0;   // slot of the newest state
  int count = 0;  // valid states
  DevBuf<double> dots;
  std::unique_ptr<Mpnn> net;
  int train_left = 0, train_steps = 0, iters_per_step = 0;
  double learning_rate = 0.0, train_loss = std::nan("");
  int last_used = NOSH_PREDICT_NONE;
  double f_learned = std::nan(""), f_secant = std::nan(""), coef = std::nan("");
  // Overlapped inference: once the weights are fixed (after the training
  // window) the network's coefficient for the next learned step runs on
  // `side` while this step's Newton solve runs on the handle's stream, from
  // this step's features (so the coefficient a step uses was inferred one
  // step earlier).  w_host: pinned copy of the coefficient used.
  cudaStream_t side = nullptr;
  cudaEvent_t ev_main = nullptr, ev_side = nullptr;
  bool w_pending = false;
  double *w_host = nullptr;
  // the network's coefficient is re-inferred on every infer_period-th
  // overlapped step and reused in between; w_valid: the device coefficient
  // belongs to the current weights
  int infer_period = 1, infer_count = 0;
  bool w_valid = false;
  void drain_side();              // handle stream waits for the side stream

  // pseudo-arclength: the last normalised tangent (tau, tau_mu) and the
  // parameter scale theta of the arclength norm
  DevBuf<double> tau, va, vb;
  double tau_mu = std::nan(""), theta = 1.0;

  ContinuationImpl(NlsImpl &nls, const double *x0, double mu0);
  ~ContinuationImpl();
  // k-th newest state (k = 0: current)
  double *slot(int k) { return hist[(head - k + kHist) % kHist].p; }
  double mu_of(int k) const { return mu[(head - k + kHist) % kHist]; }
  void extrapolate(int order, double mu_new, double *out);
  void advance(double mu_new, int predictor, const nosh_newton_options &opt, nosh_newton_stats &st);
  // one pseudo-arclength step of length ds (tangent or secant predictor,
  // bordered Newton corrector); on success the new state is pushed
  void advance_arclength(double ds, int predictor, double theta, const nosh_newton_options &opt,
                         nosh_newton_stats &st);
  // dpsi/dmu at the newest state (J^-1 of -dF/dmu, the U(1) gauge component
  // removed) into out, solved in `precision` to relative tolerance rtol;
  // returns the Krylov iterations
  int tangent_direction(const nosh_newton_options &opt, int precision, double rtol, double *out);
  void enable_learning(int train_steps, int iters, double lr);
  // diagnostics: ||F|| at mu_new of the secant, quadratic, cubic and learned
  // predictions from the current history (NaN where unavailable), without
  // advancing; the learned one uses a coefficient inferred from these
  // features
  void predictor_residuals(double mu_new, double out[4]);
};

}  // namespace nosh
