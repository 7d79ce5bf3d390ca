// Learned continuation predictor: a 3-layer edge message-passing network
// (mpnn.cu).
#pragma once

#include "nls.cuh"

namespace nosh {

struct Mpnn {
  explicit Mpnn(NlsImpl &s);
  ~Mpnn();
  bool trained() const { return trained_; }
  void set_trained(bool t) { trained_ = t; }
  // out (in: secant prediction to mu_new) += learned correction, from the
  // newest states x0 (mu0), x1 (mu1), x2 (mu2)
  void predict(const double *x0, const double *x1, const double *x2, double mu0, double mu1, double mu2,
               double mu_new, double *out);
  // optimiser iterations on the transition (x0, x1, x2) -> target at mu_t;
  // returns the last relative loss
  double train(const double *x0, const double *x1, const double *x2, double mu0, double mu1, double mu2,
               const double *target, double mu_t, int iters, double lr);

  // inspection (gradient checks): flat FP32 parameters, per-nonzero edge
  // features (adjacency-CSR order), forward from given node features, and
  // loss + parameter gradient for given features and targets
  int64_t num_params() const;
  void get_params(float *h) const;
  void set_params(const float *h);
  void get_edge_features(float *h) const;
  void forward_features(const float *X, float *Y);
  double loss_and_grad(const float *X, const float *T, float *grad);

  struct Impl;
  std::unique_ptr<Impl> impl;

 private:
  bool trained_ = false;
};

}  // namespace nosh
