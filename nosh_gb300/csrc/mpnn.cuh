// Learned continuation predictor: a 3-layer edge message-passing network
// (mpnn.cu).
#pragma once

#include "nls.cuh"

namespace nosh {

struct Mpnn {
  explicit Mpnn(NlsImpl &s);
  ~Mpnn();
  // From the newest states x[0..3] at mu[0..3]: the secant prediction to
  // mu_new into `secant`, and out = secant + q + w c, the quadratic
  // prediction plus the learned multiple w of the cubic-minus-quadratic
  // field (returns w)
  double predict(const double *const x[4], const double mu[4], double mu_new, double *secant, double *out);
  // the same in parts, for an inference that overlaps the solver: node
  // features, prediction fields and the secant for mu_new (handle stream),
  // the network's coefficient w on stream `st` (it reads the features,
  // writes w), and out = secant + q + w c with the current w (handle stream;
  // w copied to w_host, a pinned scalar, when given)
  // (node_features = false: only the prediction fields and the secant, for
  // a step whose features feed no inference)
  void prepare(const double *const x[4], const double mu[4], double mu_new, double *secant,
               bool node_features = true);
  void infer(cudaStream_t st);
  void combine(const double *secant, double *out, double *w_host);
  // prepare(node_features = false) + combine in one pass over the states,
  // for a step whose features feed no inference: the secant into `secant`,
  // out = secant + q + w c with the current w (w copied to w_host)
  void predict_fields(const double *const x[4], const double mu[4], double mu_new, double *secant, double *out,
                      double *w_host);
  // optimiser iterations on the transition x[0..3] -> target at mu_t;
  // returns the last relative loss
  double train(const double *const x[4], const double mu[4], const double *target, double mu_t, int iters,
               double lr);

  // inspection (gradient checks): flat FP32 parameters, per-nonzero edge
  // features (adjacency-CSR order), the readout coefficient for given node
  // features, and loss + parameter gradient for given features and Gram
  // scalars [<c,c>, <c,d>, <d,d>]
  int64_t num_params() const;
  void get_params(float *h) const;
  void set_params(const float *h);
  void get_edge_features(float *h) const;
  void forward_features(const float *X, double *w);
  double loss_and_grad(const float *X, const double *gram, float *grad);

  struct Impl;
  std::unique_ptr<Impl> impl;
};

}  // namespace nosh
