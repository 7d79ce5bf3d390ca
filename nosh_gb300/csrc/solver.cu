// Preconditioned MINRES and inexact Newton on the GPU.
//
// MINRES follows Paige & Saunders (1975) in the preconditioned form used by
// Belos MINRES (the solver the reference's README and
// test/linear-solve-test/linop-tester.cpp:288 pair with KeoRegularized).
// Vectors live in HBM in the operator precision (FP32 in the mixed path,
// FP64 in the plain path); every recurrence scalar is FP64 and stays in
// device memory: the reductions finish in the last CTA of the producing
// kernel, and one single-thread kernel advances the Givens recurrence, so
// the host only polls a convergence flag.
//
// Newton: full step (NOX "Line Search Based" / "Full Step",
// examples/conf.xml:168-174), NormF two-norm test (conf.xml:178-189) on the
// FP64 residual, Eisenstat-Walker style forcing.
#include <cmath>
#include <cstdio>

#include "solver.cuh"
#include "spmv.cuh"

namespace nosh {

using namespace dev;

namespace {

template <typename T>
__global__ void dot_kernel(int64_t n, const T *__restrict__ a, const T *__restrict__ b,
                           double *partials, unsigned *counter, double *out) {
  double v = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    v += (double)a[i] * (double)b[i];
  grid_reduce(v, partials, counter, out);
}

__global__ void minres_init(MinresScalars *s, double rtol, int maxit) {
  const double rz = s->rz;
  s->rtol = rtol;
  s->maxit = maxit;
  s->itn = 0;
  s->flag = 0;
  s->done = 0;
  s->oldb = 0.0;
  s->dbar = 0.0;
  s->epsln = 0.0;
  s->oldeps = 0.0;
  s->cs = -1.0;
  s->sn = 0.0;
  s->phi = 0.0;
  s->gamma = 1.0;
  s->delta = 0.0;
  s->alfa = 0.0;
  if (!(rz >= 0.0) || isinf(rz)) {  // indefinite preconditioner or NaN
    s->flag = isnan(rz) || isinf(rz) ? NOSH_ERR_NAN : NOSH_ERR_BREAKDOWN;
    s->done = 2;
    s->beta1 = s->beta = s->phibar = 0.0;
    return;
  }
  s->beta1 = sqrt(rz);
  s->beta = s->beta1;
  s->phibar = s->beta1;
  if (rz == 0.0) s->done = 2;  // b == 0: x = 0
}

// r_new = J z / beta - (beta/oldb) r1 - (alfa/beta) r2, written over r1
template <typename T>
__global__ void lanczos_update(int64_t n, const MinresScalars *__restrict__ s, const T *__restrict__ u,
                               T *__restrict__ r1, const T *__restrict__ r2) {
  if (s->done) return;
  const double beta = s->beta, alfa = s->zu / (beta * beta);
  const T a = (T)(1.0 / beta), c = (T)(alfa / beta);
  const T bb = s->itn > 0 ? (T)(beta / s->oldb) : (T)0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    r1[i] = a * u[i] - bb * r1[i] - c * r2[i];
}

// Givens recurrence (scipy / Paige-Saunders variable names)
__global__ void minres_scalars(MinresScalars *s) {
  if (s->done) {
    s->done = 2;  // 2: frozen, 1: converged during the last update
    return;
  }
  const double beta = s->beta;
  const double alfa = s->zu / (beta * beta);
  const double rz = s->rz;
  s->alfa = alfa;
  s->oldb = beta;
  if (!(rz >= 0.0) || isinf(rz) || isnan(alfa)) {
    s->flag = (isnan(rz) || isinf(rz) || isnan(alfa)) ? NOSH_ERR_NAN : NOSH_ERR_BREAKDOWN;
    s->done = 2;
    return;
  }
  const double nb = sqrt(rz);
  s->beta = nb;
  s->oldeps = s->epsln;
  const double delta = s->cs * s->dbar + s->sn * alfa;
  const double gbar = s->sn * s->dbar - s->cs * alfa;
  s->epsln = s->sn * nb;
  s->dbar = -s->cs * nb;
  double gamma = hypot(gbar, nb);
  if (gamma == 0.0) gamma = 2.2e-16;
  s->cs = gbar / gamma;
  s->sn = nb / gamma;
  s->phi = s->cs * s->phibar;
  s->phibar = s->sn * s->phibar;
  s->gamma = gamma;
  s->delta = delta;
  s->itn += 1;
  if (s->phibar <= s->rtol * s->beta1 || nb == 0.0) s->done = 1;
  else if (s->itn >= s->maxit) {
    s->done = 1;
    s->flag = NOSH_ERR_NOT_CONVERGED;
  }
}

// w_new = (z/oldb - oldeps w2 - delta w) / gamma over the w1 buffer;
// x += phi w_new
template <typename T>
__global__ void minres_wx(int64_t n, const MinresScalars *__restrict__ s, const T *__restrict__ z,
                          T *__restrict__ wa, const T *__restrict__ wb, const T *__restrict__ wc,
                          T *__restrict__ x) {
  if (s->done == 2) return;
  const T iv = (T)(1.0 / s->oldb), e = (T)s->oldeps, d = (T)s->delta, ig = (T)(1.0 / s->gamma),
          ph = (T)s->phi;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const T w = (z[i] * iv - e * wb[i] - d * wc[i]) * ig;
    wa[i] = w;
    x[i] += ph * w;
  }
}

template <typename T>
__global__ void neg_cast(int64_t n, const double *__restrict__ f, T *__restrict__ b) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (T)(-f[i]);
}

template <typename T>
__global__ void axpy_cast(int64_t n, const T *__restrict__ dx, double *__restrict__ x) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] += (double)dx[i];
}

inline int vec_grid(int64_t n) { return std::min<int64_t>(div_up(n, 256), kNumSMs * 8); }

}  // namespace

template <typename T>
Minres<T>::Minres(NlsImpl &nls) : s(nls), n2(2 * nls.N) {
  for (DevBuf<T> *b : {&r1, &r2, &z0, &z1, &u, &w0, &w1, &w2, &x}) b->alloc(n2);
  sc.alloc(1);
  NOSH_CUDA(cudaMallocHost(&h_sc, sizeof(MinresScalars)));
}

template <typename T>
Minres<T>::~Minres() {
  if (h_sc) cudaFreeHost(h_sc);
}

template <typename T>
int Minres<T>::solve(const T *b, double rtol, int maxit, int &status, double &rel_res) {
  cudaStream_t st = s.stream;
  const int G = vec_grid(n2);
  const size_t bytes = n2 * sizeof(T);
  MinresScalars *d = sc.p;
  // r1 = r2 = b, x = w = 0, z = M b, beta1^2 = <b, z>
  NOSH_CUDA(cudaMemcpyAsync(r2.p, b, bytes, cudaMemcpyDeviceToDevice, st));
  NOSH_CUDA(cudaMemcpyAsync(r1.p, b, bytes, cudaMemcpyDeviceToDevice, st));
  for (DevBuf<T> *q : {&x, &w0, &w1, &w2}) NOSH_CUDA(cudaMemsetAsync(q->p, 0, bytes, st));
  T *zc = z0.p, *zn = z1.p, *pr1 = r1.p, *pr2 = r2.p;
  T *wa = w0.p, *wb = w1.p, *wc = w2.p;  // (w1, w2, w) of the recurrence
  s.amg->apply<T>(pr2, zc);
  dot_kernel<T><<<G, 256, 0, st>>>(n2, pr2, zc, s.red.partials.p, s.red.counter.p, &d->rz);
  minres_init<<<1, 1, 0, st>>>(d, rtol, maxit);
  NOSH_CUDA(cudaGetLastError());
  const int check_every = 4;
  int it = 0;
  for (;;) {
    for (int k = 0; k < check_every; k++, it++) {
      // u = J z, <z, u>
      s.jac_apply<T>(zc, u.p, &d->zu);
      lanczos_update<T><<<G, 256, 0, st>>>(n2, d, u.p, pr1, pr2);
      std::swap(pr1, pr2);  // r2 = r_new, r1 = previous r2
      s.amg->apply<T>(pr2, zn);
      dot_kernel<T><<<G, 256, 0, st>>>(n2, pr2, zn, s.red.partials.p, s.red.counter.p, &d->rz);
      minres_scalars<<<1, 1, 0, st>>>(d);
      minres_wx<T><<<G, 256, 0, st>>>(n2, d, zc, wa, wb, wc, x.p);
      // (w1, w2, w) <- (w2, w, w_new)
      T *t = wa;
      wa = wb;
      wb = wc;
      wc = t;
      std::swap(zc, zn);
    }
    NOSH_CUDA(cudaGetLastError());
    NOSH_CUDA(cudaMemcpyAsync(h_sc, d, sizeof(MinresScalars), cudaMemcpyDeviceToHost, st));
    NOSH_CUDA(cudaStreamSynchronize(st));
    if (h_sc->done || it >= maxit + check_every) break;
  }
  status = h_sc->flag;
  rel_res = h_sc->beta1 > 0 ? h_sc->phibar / h_sc->beta1 : 0.0;
  return h_sc->itn;
}

template struct Minres<float>;
template struct Minres<double>;

// ------------------------------------------------------------------ Newton
namespace {
struct NewtonState {
  DevBuf<double> psi, f;
  DevBuf<float> b32;
  DevBuf<double> b64;
  std::unique_ptr<Minres<float>> m32;
  std::unique_ptr<Minres<double>> m64;
};
}  // namespace

static NewtonState &state_of(NlsImpl &s) {
  if (!s.solver_state) {
    auto *ns = new NewtonState();
    ns->psi.alloc(2 * s.N);
    ns->f.alloc(2 * s.N);
    s.solver_state = std::shared_ptr<void>(ns, [](void *p) { delete (NewtonState *)p; });
  }
  return *(NewtonState *)s.solver_state.get();
}

static double residual_norm(NlsImpl &s, const double *psi, double g, double mu, double *f) {
  s.compute_f64(psi, g, mu, f, 0);
  double n2 = 0.0;
  s.red.out.download(&n2, 1, s.stream);
  s.sync();
  return std::sqrt(n2);
}

template <typename T>
static void newton_loop(NlsImpl &s, NewtonState &ns, double g, double mu,
                        const nosh_newton_options &opt, nosh_newton_stats &st,
                        std::unique_ptr<Minres<T>> &mr, DevBuf<T> &b) {
  if (!mr) mr.reset(new Minres<T>(s));
  if (b.n < (size_t)(2 * s.N)) b.alloc(2 * s.N);
  const int64_t n2 = 2 * s.N;
  const int G = vec_grid(n2);
  // FP32 Krylov cannot resolve relative residuals much below ~1e-6
  const double eta_min = sizeof(T) == 4 ? 1e-6 : 1e-12;
  double fn = st.f_norm0, fn_prev = fn;
  for (int it = 0; it < opt.max_newton && fn > opt.tol; it++) {
    s.jac_rebuild(ns.psi.p, g, mu);
    s.reg_rebuild(ns.psi.p, g, mu);
    if (!s.amg) s.amg.reset(new Amg(s));
    s.amg->refresh<T>();
    neg_cast<T><<<G, 256, 0, s.stream>>>(n2, ns.f.p, b.p);
    double eta;
    if (opt.forcing > 0) {
      eta = opt.forcing;
    } else {
      // Eisenstat-Walker choice 2 (gamma 0.9, alpha 2), safeguarded, and no
      // tighter than needed to reach the target in one step
      const double ew = it == 0 ? 1e-2 : 0.9 * (fn / fn_prev) * (fn / fn_prev);
      eta = std::min(0.1, std::max(ew, 0.5 * opt.tol / fn));
    }
    eta = std::max(eta, eta_min);
    int status = 0;
    double rel = 0.0;
    const int its = mr->solve(b.p, eta, opt.max_krylov, status, rel);
    st.krylov_iters += its;
    if (status == NOSH_ERR_NAN || status == NOSH_ERR_BREAKDOWN) {
      st.status = status;
      return;
    }
    axpy_cast<T><<<G, 256, 0, s.stream>>>(n2, mr->x.p, ns.psi.p);
    fn_prev = fn;
    fn = residual_norm(s, ns.psi.p, g, mu, ns.f.p);
    st.newton_iters = it + 1;
    st.f_norm = fn;
    if (opt.verbose)
      std::fprintf(stderr, "newton %2d  ||F|| = %.3e  minres its %4d  eta %.1e  rel %.1e\n", it + 1, fn, its,
                   eta, rel);
    if (std::isnan(fn)) {
      st.status = NOSH_ERR_NAN;
      return;
    }
  }
}

void newton_solve(NlsImpl &s, double *x_user, double g, double mu, const nosh_newton_options &opt,
                  nosh_newton_stats &st) {
  NewtonState &ns = state_of(s);
  const size_t bytes = 2 * s.N * sizeof(double);
  NOSH_CUDA(cudaMemcpyAsync(ns.psi.p, x_user, bytes, cudaMemcpyDefault, s.stream));
  st = nosh_newton_stats{};
  st.f_norm0 = residual_norm(s, ns.psi.p, g, mu, ns.f.p);
  st.f_norm = st.f_norm0;
  NOSH_CHECK(!std::isnan(st.f_norm0), NOSH_ERR_NAN, "initial residual is NaN");
  if (opt.precision == NOSH_PREC_FP64) newton_loop<double>(s, ns, g, mu, opt, st, ns.m64, ns.b64);
  else newton_loop<float>(s, ns, g, mu, opt, st, ns.m32, ns.b32);
  NOSH_CUDA(cudaMemcpyAsync(x_user, ns.psi.p, bytes, cudaMemcpyDefault, s.stream));
  s.sync();
  if (st.status == NOSH_OK && !(st.f_norm <= opt.tol)) st.status = NOSH_ERR_NOT_CONVERGED;
}

}  // namespace nosh
