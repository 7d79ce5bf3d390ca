// Device-resident continuation run (continuation.cu).
#pragma once

#include <memory>

#include "solver.cuh"

namespace nosh {

struct Mpnn;  // learned predictor (mpnn.cu)

struct ContinuationImpl {
  static constexpr int kHist = 5;  // newest converged states kept in HBM
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

  ContinuationImpl(NlsImpl &nls, const double *x0, double mu0);
  ~ContinuationImpl();
  // k-th newest state (k = 0: current)
  double *slot(int k) { return hist[(head - k + kHist) % kHist].p; }
  double mu_of(int k) const { return mu[(head - k + kHist) % kHist]; }
  void extrapolate(int order, double mu_new, double *out);
  void advance(double mu_new, int predictor, const nosh_newton_options &opt, nosh_newton_stats &st);
  void enable_learning(int train_steps, int iters, double lr);
};

}  // namespace nosh
