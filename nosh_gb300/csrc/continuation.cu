// Device-resident continuation (LOCA stepper semantics, examples/conf.xml:35-75;
// the driver loop of executables/nosh-cont/nosh-cont.cpp:226-345): natural
// steps in mu and pseudo-arclength steps.  The last converged states stay in
// HBM, predictions are formed on the GPU and corrected by Newton.
#include <cmath>
#include <cstdio>

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

// Up to six real inner products of complex vectors in one pass:
// out[j] = sum_i Re(conj(a_j[i]) * b_j[i]), or with i*b_j[i] when rot[j]
// (the U(1) gauge direction).
struct DotSet {
  const C2<double> *a[6] = {}, *b[6] = {};
  bool rot[6] = {};
  int k = 0;
  void add(const double *x, const double *y, bool r = false) {
    a[k] = (const C2<double> *)x;
    b[k] = (const C2<double> *)y;
    rot[k] = r;
    k++;
  }
};

__global__ void dot_set_kernel(int64_t n, DotSet d, double *partials, unsigned *counter, double *out) {
  double v[6] = {0, 0, 0, 0, 0, 0};
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int j = 0; j < 6; j++) {
      if (j < d.k) {
        const C2<double> a = d.a[j][i], b = d.b[j][i];
        v[j] += d.rot[j] ? a.y * b.x - a.x * b.y : a.x * b.x + a.y * b.y;
      }
    }
  }
  dev::grid_reduce_n<6>(v, d.k, partials, counter, out);
}

// y = c0 x0 + c1 x1 + c2 (rot2 ? i x2 : x2); y may alias x0 or x1
__global__ void lin3_kernel(int64_t n, C2<double> *y, double c0, const C2<double> *x0, double c1,
                            const C2<double> *x1, double c2, const C2<double> *x2, bool rot2) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    C2<double> r = x0[i];
    r.x *= c0;
    r.y *= c0;
    if (x1) {
      const C2<double> a = x1[i];
      r.x += c1 * a.x;
      r.y += c1 * a.y;
    }
    if (x2) {
      const C2<double> a = x2[i];
      r.x += c2 * (rot2 ? -a.y : a.x);
      r.y += c2 * (rot2 ? a.x : a.y);
    }
    y[i] = r;
  }
}

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

ContinuationImpl::~ContinuationImpl() {
  // the network's buffers outlive any inference still running on the side
  if (side) cudaStreamSynchronize(side);
  if (ev_main) cudaEventDestroy(ev_main);
  if (ev_side) cudaEventDestroy(ev_side);
  if (side) cudaStreamDestroy(side);
  if (w_host) cudaFreeHost(w_host);
}

void ContinuationImpl::drain_side() {
  if (w_pending) NOSH_CUDA(cudaStreamWaitEvent(s.stream, ev_side, 0));
  w_pending = false;
}

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
    history_dots<<<reduce_grid(s.N), 256, 0, st>>>(s.N, slot(0), slot(1), order >= 2 ? slot(2) : nullptr,
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

namespace {
double *dots_host(NlsImpl &s, const DotSet &d, int64_t n, double *dev_out, double *host) {
  dot_set_kernel<<<reduce_grid(n), 256, 0, s.stream>>>(n, d, s.red.partials.p, s.red.counter.p, dev_out);
  ++s.launch_count;
  NOSH_CUDA(cudaGetLastError());
  NOSH_CUDA(cudaMemcpyAsync(host, dev_out, d.k * sizeof(double), cudaMemcpyDeviceToHost, s.stream));
  s.sync();
  return host;
}
void lin3(NlsImpl &s, int64_t n, double *y, double c0, const double *x0, double c1 = 0.0,
          const double *x1 = nullptr, double c2 = 0.0, const double *x2 = nullptr, bool rot2 = false) {
  lin3_kernel<<<vgrid(n), 256, 0, s.stream>>>(n, (C2<double> *)y, c0, (const C2<double> *)x0, c1,
                                              (const C2<double> *)x1, c2, (const C2<double> *)x2, rot2);
  ++s.launch_count;
  NOSH_CUDA(cudaGetLastError());
}
inline bool solve_failed(int status) { return status == NOSH_ERR_NAN || status == NOSH_ERR_BREAKDOWN; }
}  // namespace

int ContinuationImpl::tangent_direction(const nosh_newton_options &opt, int precision, double rtol, double *out) {
  // LOCA's tangent predictor: J dpsi/dmu = -dF/dmu at the converged state,
  // dF/dmu = (dK/dmu) psi (src/model_evaluator_nls.cpp:632-695).  J is
  // singular along the gauge direction i psi0 (J(i psi) = i F); the
  // component of the solution along it is arbitrary and is removed, which
  // makes the tangent, and the arclength norm built on it, unique.
  NewtonState &ns = state_of(s);
  const double g = s.g0, mu0 = mu_of(0);
  NOSH_CUDA(cudaMemcpyAsync(ns.psi.p, slot(0), 2 * s.N * sizeof(double), cudaMemcpyDeviceToDevice, s.stream));
  s.dfdp64(ns.psi.p, g, mu0, 1, ns.tmp.p);
  int status = 0;
  const int its = linear_solve(s, ns, ns.tmp.p, out, g, mu0, rtol, opt.max_krylov, precision, true, status);
  NOSH_CHECK(!solve_failed(status), status, "tangent solve failed");
  DotSet d;
  d.add(slot(0), out, true);  // <psi0, i v> = -<i psi0, v>
  d.add(slot(0), slot(0));
  double h[6];
  dots_host(s, d, s.N, dots.p, h);
  NOSH_CHECK(h[1] > 0.0, NOSH_ERR_BREAKDOWN, "tangent at a zero state");
  const double kappa = -h[0] / h[1];
  // out = -(v - kappa i psi0)
  lin3(s, s.N, out, -1.0, out, 0.0, nullptr, kappa, slot(0), true);
  return its;
}

void ContinuationImpl::advance_arclength(double ds, int predictor, double theta_in,
                                         const nosh_newton_options &opt, nosh_newton_stats &st) {
  // Pseudo-arclength continuation (Keller), LOCA "Arc Length" stepper
  // (examples/conf.xml:38-46) with the bordering solve of the extended
  // system.  With <a, b>_s = a.b / n (n = 2N reals) and
  // ||(x, m)||^2 = <x, x>_s + theta^2 m^2, the unit tangent (tau, tau_mu)
  // at (psi0, mu0) and the step length ds define the constraint
  //   c(psi, mu) = <tau, psi - psi0>_s + theta^2 tau_mu (mu - mu0) - ds = 0.
  // Predictor: (psi0, mu0) + ds (tau, tau_mu) (which satisfies c = 0).
  // Corrector: Newton on (F, c); each step solves J a = F and J b = dF/dmu
  // with the same operators and takes
  //   dmu = <tau, a>_s / (theta^2 tau_mu - <tau, b>_s),  dpsi = -a - dmu b,
  // which keeps c = 0 exactly, so convergence is ||F|| <= tol.
  NOSH_CHECK(predictor == NOSH_PREDICT_TANGENT || predictor == NOSH_PREDICT_SECANT, NOSH_ERR_INVALID,
             "arclength steps predict TANGENT or SECANT");
  NOSH_CHECK(std::isfinite(ds) && ds != 0.0, NOSH_ERR_INVALID, "ds must be finite and nonzero");
  NOSH_CHECK(std::isfinite(theta_in) && theta_in > 0.0, NOSH_ERR_INVALID, "theta must be positive");
  theta = theta_in;
  drain_side();  // a pending coefficient serves only the next learned step
  NewtonState &ns = state_of(s);
  const double g = s.g0, mu0 = mu_of(0);
  const int64_t N = s.N, n2 = 2 * N;
  const double inv_n = 1.0 / (double)n2, th2 = theta * theta;
  for (DevBuf<double> *b : {&tau, &va, &vb})
    if (b->n < (size_t)n2) b->alloc(n2);
  st = nosh_newton_stats{};
  f_learned = f_secant = coef = std::nan("");
  const bool have_secant = count >= 2;
  const int G = vgrid(N);
  if (have_secant) {
    // phase-aligned secant psi0 - e^{i phi} psi1 into va
    history_dots<<<reduce_grid(N), 256, 0, s.stream>>>(N, slot(0), slot(1), nullptr, nullptr, nullptr, 1,
                                                        s.red.partials.p,
                                          s.red.counter.p, dots.p);
    normalize_phases<<<1, 32, 0, s.stream>>>(1, dots.p);
    extrapolate_kernel<<<G, 256, 0, s.stream>>>(N, 1, dots.p, 1.0, -1.0, 0.0, 0.0, (const C2<double> *)slot(0),
                                                (const C2<double> *)slot(1), (const C2<double> *)slot(0),
                                                (const C2<double> *)slot(0), (C2<double> *)va.p);
    s.launch_count += 3;
    NOSH_CUDA(cudaGetLastError());
  }
  double tmu;
  if (predictor == NOSH_PREDICT_TANGENT || !have_secant) {
    st.krylov_iters += tangent_direction(opt, NOSH_PREC_FP64, 1e-10, tau.p);
    tmu = 1.0;
    last_used = NOSH_PREDICT_TANGENT;
  } else {
    NOSH_CUDA(cudaMemcpyAsync(tau.p, va.p, n2 * sizeof(double), cudaMemcpyDeviceToDevice, s.stream));
    tmu = mu0 - mu_of(1);
    last_used = NOSH_PREDICT_SECANT;
  }
  double h[6];
  {
    DotSet d;
    d.add(tau.p, tau.p);
    if (have_secant) d.add(tau.p, va.p);
    dots_host(s, d, N, dots.p, h);
  }
  const double t2 = h[0] * inv_n + th2 * tmu * tmu;
  NOSH_CHECK(t2 > 0.0 && std::isfinite(t2), NOSH_ERR_BREAKDOWN, "zero or non-finite tangent");
  double sc = 1.0 / std::sqrt(t2);
  // orientation: along the last secant (the direction of travel)
  if (have_secant && h[1] * inv_n + th2 * tmu * (mu0 - mu_of(1)) < 0.0) sc = -sc;
  lin3(s, N, tau.p, sc, tau.p);
  tmu *= sc;
  tau_mu = tmu;
  // predictor
  lin3(s, N, ns.psi.p, 1.0, slot(0), ds, tau.p);
  double mc = mu0 + ds * tmu;
  double fn = residual_norm(s, ns.psi.p, g, mc, ns.f.p);
  st.f_norm0 = st.f_norm = fn;
  NOSH_CHECK(!std::isnan(fn), NOSH_ERR_NAN, "predicted residual is NaN");
  // Constant forcing (the reference's NOX setting, "Forcing Term Method"
  // Constant, examples/conf.xml:81) and FP64 Krylov whatever the handle's
  // precision: near a fold J is nearly singular along the tangent, a and b
  // are both large there and only their combination is small, so loose
  // (Eisenstat-Walker) or FP32 solves stall the corrector or skip the fold
  // (an 8x8 square, 97^2 vertices: both turned away from the fold at
  // mu = 0.4097 that FP64 solves at 1e-8 follow).
  const double eta = opt.forcing > 0.0 ? opt.forcing : kArclengthForcing;
  for (int it = 0; it < opt.max_newton && fn > opt.tol; it++) {
    int status = 0;
    st.krylov_iters += linear_solve(s, ns, ns.f.p, va.p, g, mc, eta, opt.max_krylov, NOSH_PREC_FP64, true, status);
    if (solve_failed(status)) {
      st.status = status;
      return;
    }
    s.dfdp64(ns.psi.p, g, mc, 1, ns.tmp.p);
    st.krylov_iters += linear_solve(s, ns, ns.tmp.p, vb.p, g, mc, eta, opt.max_krylov, NOSH_PREC_FP64, false, status);
    if (solve_failed(status)) {
      st.status = status;
      return;
    }
    DotSet d;
    d.add(tau.p, va.p);
    d.add(tau.p, vb.p);
    dots_host(s, d, N, dots.p, h);
    const double den = th2 * tmu - h[1] * inv_n;
    if (!(std::isfinite(den) && den != 0.0)) {
      st.status = NOSH_ERR_BREAKDOWN;  // singular bordered system
      return;
    }
    const double dmu = h[0] * inv_n / den;
    lin3(s, N, ns.psi.p, 1.0, ns.psi.p, -1.0, va.p, -dmu, vb.p);
    mc += dmu;
    fn = residual_norm(s, ns.psi.p, g, mc, ns.f.p);
    st.newton_iters = it + 1;
    st.f_norm = fn;
    if (opt.verbose)
      std::fprintf(stderr, "arclength newton %2d  mu = %.12f  ||F|| = %.3e  eta %.1e\n", it + 1, mc, fn, eta);
    if (std::isnan(fn)) {
      st.status = NOSH_ERR_NAN;
      return;
    }
  }
  if (!(fn <= opt.tol)) {
    st.status = NOSH_ERR_NOT_CONVERGED;
    return;
  }
  head = (head + 1) % kHist;
  NOSH_CUDA(cudaMemcpyAsync(hist[head].p, ns.psi.p, n2 * sizeof(double), cudaMemcpyDeviceToDevice, s.stream));
  mu[head] = mc;
  count = std::min(count + 1, kHist);
  s.sync();
}

void ContinuationImpl::advance(double mu_new, int predictor, const nosh_newton_options &opt,
                               nosh_newton_stats &st) {
  NOSH_CHECK(predictor == NOSH_PREDICT_NONE || predictor == NOSH_PREDICT_SECANT ||
                 predictor == NOSH_PREDICT_TANGENT || predictor == NOSH_PREDICT_QUADRATIC ||
                 predictor == NOSH_PREDICT_CUBIC || predictor == NOSH_PREDICT_LEARNED,
             NOSH_ERR_INVALID, "continuation handles predict NONE, SECANT, TANGENT, QUADRATIC, CUBIC or LEARNED");
  NOSH_CHECK(mu_new != mu_of(0), NOSH_ERR_INVALID, "mu_new equals the current mu");
  NewtonState &ns = state_of(s);
  const double g = s.g0;
  if (predictor == NOSH_PREDICT_TANGENT) {
    drain_side();  // a pending coefficient serves only the next learned step
    // psi0 + (mu_new - mu0) dpsi/dmu
    if (tau.n < (size_t)(2 * s.N)) tau.alloc(2 * s.N);
    // a predictor only: FP32 solves are accurate enough
    const bool fp64 = opt.precision == NOSH_PREC_FP64;
    const int its = tangent_direction(opt, opt.precision, fp64 ? 1e-10 : 1e-5, tau.p);
    lin3(s, s.N, ns.psi.p, 1.0, slot(0), mu_new - mu_of(0), tau.p);
    last_used = NOSH_PREDICT_TANGENT;
    f_learned = f_secant = coef = std::nan("");
    newton_core(s, ns, g, mu_new, opt, st, -1.0);
    st.krylov_iters += its;
    if (st.status != NOSH_OK) return;
    head = (head + 1) % kHist;
    NOSH_CUDA(cudaMemcpyAsync(hist[head].p, ns.psi.p, 2 * s.N * sizeof(double), cudaMemcpyDeviceToDevice,
                              s.stream));
    mu[head] = mu_new;
    count = std::min(count + 1, kHist);
    s.sync();
    return;
  }
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
  const bool learned = predictor == NOSH_PREDICT_LEARNED && net && count >= 4;
  // (a learned step forms the secant with its features)
  if (!learned) extrapolate(order, mu_new, ns.psi.p);
  double f0 = -1.0;
  // the weights change (training) or the network is not used: no inference
  // may still be running
  const bool overlap = learned && train_left == 0;
  if (!overlap) drain_side();
  if (learned) {
    // learned correction of the secant prediction: the secant into ns.psi
    // (the fallback), the learned prediction into ns.tmp
    const double *x[4] = {slot(0), slot(1), slot(2), slot(3)};
    const double m[4] = {mu_of(0), mu_of(1), mu_of(2), mu_of(3)};
    bool compare;
    if (overlap) {
      if (!side) {
        int lo = 0, hi = 0;
        NOSH_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
        NOSH_CUDA(cudaStreamCreateWithPriority(&side, cudaStreamNonBlocking, lo));  // below the solver
        NOSH_CUDA(cudaEventCreateWithFlags(&ev_main, cudaEventDisableTiming));
        NOSH_CUDA(cudaEventCreateWithFlags(&ev_side, cudaEventDisableTiming));
        NOSH_CUDA(cudaMallocHost(&w_host, sizeof(double)));
      }
      // the coefficient inferred during an earlier step (or now, on the
      // first overlapped step)
      const bool have_w = w_pending || w_valid;
      drain_side();
      // the node features only when an inference reads them; otherwise the
      // prediction straight from the states
      if (!have_w || infer_count + 1 >= infer_period) {
        net->prepare(x, m, mu_new, ns.psi.p, true);
        if (!have_w) net->infer(s.stream);
        net->combine(ns.psi.p, ns.tmp.p, w_host);
      } else {
        net->predict_fields(x, m, mu_new, ns.psi.p, ns.tmp.p, w_host);
      }
      w_valid = true;
      // the next coefficient from these features, under this Newton
      if (++infer_count >= infer_period) {
        infer_count = 0;
        NOSH_CUDA(cudaEventRecord(ev_main, s.stream));
        NOSH_CUDA(cudaStreamWaitEvent(side, ev_main, 0));
        net->infer(side);
        NOSH_CUDA(cudaEventRecord(ev_side, side));
        w_pending = true;
      }
    } else {
      coef = net->predict(x, m, mu_new, ns.psi.p, ns.tmp.p);
      w_valid = false;  // the weights may change before the next step
    }
    // F of the learned prediction and of the secant in one pass over the
    // KEO (syncs: w_host is valid after it); a prediction that meets the
    // tolerance is taken as is, otherwise the one with the smaller residual
    // starts Newton: the plain secant is the fallback whenever the
    // network's starting residual is worse
    double nrm[2];
    ns.ensure_soff(2 * s.N);
    s.residual_pair(ns.tmp.p, ns.psi.p, g, mu_new, ns.f.p, ns.xc.p, nrm, ns.soff_alt.p, ns.soff.p, false);
    // while the host waits for the two norms, the GPU builds the mixed
    // Newton step's operators at the learned prediction (the usual winner;
    // a secant that wins is rebuilt for in the Newton loop)
    if (opt.precision != NOSH_PREC_FP64) prebuild_operators32(s, ns, ns.tmp.p, g, mu_new);
    s.residual_pair_norms(nrm);
    if (overlap) coef = *w_host;
    f_learned = nrm[0];
    f_secant = nrm[1];
    compare = !(f_learned <= opt.tol);
    if (!compare || f_learned < f_secant) {
      std::swap(ns.psi, ns.tmp);
      std::swap(ns.soff, ns.soff_alt);
      last_used = NOSH_PREDICT_LEARNED;
      f0 = f_learned;  // ns.f holds F of the learned prediction
    } else {
      std::swap(ns.f, ns.xc);
      f0 = f_secant;
    }
    ns.soff_valid = ns.soff_fresh = true;  // ns.soff: K's off-diagonal sums at the chosen prediction
    ns.soff_mu = mu_new;
  }
  newton_core(s, ns, g, mu_new, opt, st, f0, learned);
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

void ContinuationImpl::predictor_residuals(double mu_new, double out[4]) {
  NOSH_CHECK(mu_new != mu_of(0), NOSH_ERR_INVALID, "mu_new equals the current mu");
  drain_side();
  NewtonState &ns = state_of(s);
  const double g = s.g0;
  for (int q = 0; q < 4; q++) out[q] = std::nan("");
  for (int order = 1; order <= 3; order++)
    if (count > order) {
      extrapolate(order, mu_new, ns.tmp.p);
      out[order - 1] = residual_norm(s, ns.tmp.p, g, mu_new, ns.f.p);
    }
  if (net && count >= 4) {
    const double *x[4] = {slot(0), slot(1), slot(2), slot(3)};
    const double m[4] = {mu_of(0), mu_of(1), mu_of(2), mu_of(3)};
    net->predict(x, m, mu_new, ns.xc.p, ns.tmp.p);
    w_valid = false;  // the device coefficient now belongs to these features
    out[3] = residual_norm(s, ns.tmp.p, g, mu_new, ns.f.p);
  }
}

void ContinuationImpl::enable_learning(int train_steps, int iters, double lr) {
  drain_side();
  w_valid = false;
  if (!net) net.reset(new Mpnn(s));
  train_left = train_steps;
  this->train_steps = train_steps;
  iters_per_step = iters;
  learning_rate = lr;
}

}  // namespace nosh
