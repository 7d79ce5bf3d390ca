// Device-resident natural continuation (LOCA stepper semantics,
// examples/conf.xml:35-75; the driver loop of
// executables/nosh-cont/nosh-cont.cpp:226-345): the last converged states stay
// in HBM, predictions are formed on the GPU and corrected by Newton.
#include <cmath>

#include "continuation.cuh"
#include "mpnn.cuh"
#include "spmv.cuh"

namespace nosh {

using namespace dev;

namespace {

// out = sum_k L_k e^{i phi_k} x_k (k <= order), the unit phase factors c
// (normalize_phases) aligning x_k with x0 (solutions are defined up to a
// global U(1) phase)
__global__ void extrapolate_kernel(int64_t n, int order, const double *__restrict__ c, double L0, double L1,
                                   double L2, double L3, const C2<double> *__restrict__ x0,
                                   const C2<double> *__restrict__ x1, const C2<double> *__restrict__ x2,
                                   const C2<double> *__restrict__ x3, C2<double> *__restrict__ out) {
  double er[3] = {1.0, 1.0, 1.0}, ei[3] = {0.0, 0.0, 0.0};
  for (int k = 0; k < order; k++) {
    er[k] = c[2 * k];
    ei[k] = c[2 * k + 1];
  }
  const double L[3] = {L1, L2, L3};
  const C2<double> *xs[3] = {x1, x2, x3};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const C2<double> a = x0[i];
    double r = L0 * a.x, im = L0 * a.y;
    for (int k = 0; k < order; k++) {
      const C2<double> p = xs[k][i];
      r += L[k] * (er[k] * p.x - ei[k] * p.y);
      im += L[k] * (er[k] * p.y + ei[k] * p.x);
    }
    out[i] = C2<double>{r, im};
  }
}

inline int vgrid(int64_t n) { return (int)std::min<int64_t>(div_up(n, 256), kNumSMs * 8); }

}  // namespace

ContinuationImpl::ContinuationImpl(NlsImpl &nls, const double *x0, double mu0) : s(nls) {
  for (auto &h : hist) h.alloc(2 * s.N);
  dots.alloc(8);
  NOSH_CUDA(cudaMemcpyAsync(hist[0].p, x0, 2 * s.N * sizeof(double), cudaMemcpyDefault, s.stream));
  mu[0] = mu0;
  head = 0;
  count = 1;
  s.sync();
}

ContinuationImpl::~ContinuationImpl() = default;

// phase-aligned Lagrange extrapolation of the newest (order+1) states to mu_new
void ContinuationImpl::extrapolate(int order, double mu_new, double *out) {
  cudaStream_t st = s.stream;
  double L[4] = {1.0, 0.0, 0.0, 0.0};
  for (int k = 0; k <= order; k++) {
    double v = 1.0;
    for (int q = 0; q <= order; q++)
      if (q != k) v *= (mu_new - mu_of(q)) / (mu_of(k) - mu_of(q));
    L[k] = v;
  }
  const int G = vgrid(s.N);
  if (order >= 1) {
    history_dots<<<G, 256, 0, st>>>(s.N, slot(0), slot(1), order >= 2 ? slot(2) : nullptr,
                                    order >= 3 ? slot(3) : nullptr, nullptr, order, s.red.partials.p, s.red.counter.p,
                                    dots.p);
    normalize_phases<<<1, 32, 0, st>>>(order, dots.p);
    s.launch_count += 2;
  }
  const double *x1 = order >= 1 ? slot(1) : slot(0), *x2 = order >= 2 ? slot(2) : slot(0),
               *x3 = order >= 3 ? slot(3) : slot(0);
  extrapolate_kernel<<<G, 256, 0, st>>>(s.N, order, dots.p, L[0], L[1], L[2], L[3], (const C2<double> *)slot(0),
                                        (const C2<double> *)x1, (const C2<double> *)x2, (const C2<double> *)x3,
                                        (C2<double> *)out);
  ++s.launch_count;
  NOSH_CUDA(cudaGetLastError());
}

void ContinuationImpl::advance(double mu_new, int predictor, const nosh_newton_options &opt,
                               nosh_newton_stats &st) {
  NOSH_CHECK(predictor == NOSH_PREDICT_NONE || predictor == NOSH_PREDICT_SECANT ||
                 predictor == NOSH_PREDICT_QUADRATIC || predictor == NOSH_PREDICT_CUBIC ||
                 predictor == NOSH_PREDICT_LEARNED,
             NOSH_ERR_INVALID, "continuation handles predict NONE, SECANT, QUADRATIC, CUBIC or LEARNED");
  NOSH_CHECK(mu_new != mu_of(0), NOSH_ERR_INVALID, "mu_new equals the current mu");
  NewtonState &ns = state_of(s);
  const double g = s.g0;
  int order = 0;
  if (predictor == NOSH_PREDICT_SECANT || predictor == NOSH_PREDICT_LEARNED) order = 1;
  if (predictor == NOSH_PREDICT_QUADRATIC) order = 2;
  if (predictor == NOSH_PREDICT_CUBIC) order = 3;
  order = std::min(order, count - 1);
  const int used_of[4] = {NOSH_PREDICT_NONE, NOSH_PREDICT_SECANT, NOSH_PREDICT_QUADRATIC, NOSH_PREDICT_CUBIC};
  last_used = used_of[order];
  f_learned = std::nan("");
  f_secant = std::nan("");
  coef = std::nan("");
  extrapolate(order, mu_new, ns.psi.p);
  double f0 = -1.0;
  if (predictor == NOSH_PREDICT_LEARNED && net && count >= 4) {
    // learned correction of the secant prediction; a prediction that already
    // meets the tolerance is taken as is, otherwise the one with the smaller
    // residual starts Newton (the secant is the fallback)
    NOSH_CUDA(cudaMemcpyAsync(ns.tmp.p, ns.psi.p, 2 * s.N * sizeof(double), cudaMemcpyDeviceToDevice, s.stream));
    const double *x[4] = {slot(0), slot(1), slot(2), slot(3)};
    const double m[4] = {mu_of(0), mu_of(1), mu_of(2), mu_of(3)};
    coef = net->predict(x, m, mu_new, ns.tmp.p);
    f_learned = residual_norm(s, ns.tmp.p, g, mu_new, ns.f.p);
    if (!(f_learned <= opt.tol)) f_secant = residual_norm(s, ns.psi.p, g, mu_new, ns.xc.p);
    if (f_learned <= opt.tol || f_learned < f_secant) {
      std::swap(ns.psi, ns.tmp);
      last_used = NOSH_PREDICT_LEARNED;
      f0 = f_learned;  // ns.f holds F of the learned prediction
    } else {
      std::swap(ns.f, ns.xc);
      f0 = f_secant;
    }
  }
  newton_core(s, ns, g, mu_new, opt, st, f0);
  if (st.status != NOSH_OK) return;
  // push the converged state
  head = (head + 1) % kHist;
  NOSH_CUDA(cudaMemcpyAsync(hist[head].p, ns.psi.p, 2 * s.N * sizeof(double), cudaMemcpyDeviceToDevice,
                            s.stream));
  mu[head] = mu_new;
  count = std::min(count + 1, kHist);
  // online training on the transition (x_{k-3}, ..., x_k) -> x_{k+1}
  if (net && train_left > 0 && count >= 5) {
    const double *x[4] = {slot(1), slot(2), slot(3), slot(4)};
    const double m[4] = {mu_of(1), mu_of(2), mu_of(3), mu_of(4)};
    // the step size decays linearly over the training window
    const double lr = learning_rate * train_left / std::max(train_steps, 1);
    train_loss = net->train(x, m, slot(0), mu_of(0), iters_per_step, lr);
    train_left--;
  }
  s.sync();
}

void ContinuationImpl::enable_learning(int train_steps, int iters, double lr) {
  if (!net) net.reset(new Mpnn(s));
  train_left = train_steps;
  this->train_steps = train_steps;
  iters_per_step = iters;
  learning_rate = lr;
}

}  // namespace nosh
