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
#include <algorithm>
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
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  // two elements per pass, their loads issued first (the per-thread order
  // stays i, i + stride, ...)
  for (; i + stride < n; i += 2 * stride) {
    const T a0 = a[i], b0 = b[i], a1 = a[i + stride], b1 = b[i + stride];
    v += (double)a0 * (double)b0;
    v += (double)a1 * (double)b1;
  }
  for (; i < n; i += stride) v += (double)a[i] * (double)b[i];
  grid_reduce(v, partials, counter, out);
}

// params = {rtol, maxit} (device memory, written before each solve so the
// captured prologue graph stays valid)
__global__ void minres_init(MinresScalars *s, const double *params) {
  const double rz = s->rz;
  s->rtol = params[0];
  s->maxit = (int)params[1];
  s->itn = 0;
  s->flag = 0;
  s->done = 0;
  s->wx_pending = 0;
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

// u = J z and <z, u>, with the deferred w/x update of the previous Lanczos
// step folded into the epilogue (element-wise, rows are independent).
template <typename T>
struct JacMinresOp {
  static constexpr bool kReduce = true;
  static constexpr bool kHook = true;
  const T *d;  // Jacobian diagonal blocks, 3 per vertex
  const C2<T> *x;
  C2<T> *y;
  const MinresScalars *s;
  const T *zprev;
  T *wa;
  const T *wb, *wc;
  T *xsol;
  const int *halt;  // &s->done
  struct Pre {
    C2<T> xi;
    T d0r, d0i, d1b;
    C2<T> zp, wbv, wcv, xs;  // deferred w/x update operands (when pending)
    bool wx;
  };
  __device__ Pre load(int i) const {
    Pre p;
    p.xi = x[i];
    p.d0r = d[3 * i];
    p.d0i = d[3 * i + 1];
    p.d1b = d[3 * i + 2];
    p.wx = s->wx_pending != 0;
    if (p.wx) {
      p.zp = reinterpret_cast<const C2<T> *>(zprev)[i];
      p.wbv = reinterpret_cast<const C2<T> *>(wb)[i];
      p.wcv = reinterpret_cast<const C2<T> *>(wc)[i];
      p.xs = reinterpret_cast<const C2<T> *>(xsol)[i];
    }
    return p;
  }
  __device__ double finish(int i, T sr, T si, const Pre &p) const {
    const T yr = sr + p.d0r * p.xi.x + p.d1b * p.xi.y;
    const T yi = si + p.d1b * p.xi.x + p.d0i * p.xi.y;
    y[i] = C2<T>{yr, yi};
    if (p.wx) {
      // w = (z c0 - c1 w2 - c2 w) c3 over the w1 buffer, x += c4 w
      const T *c = wx_coef<T>(s);
      const C2<T> w{(p.zp.x * c[0] - c[1] * p.wbv.x - c[2] * p.wcv.x) * c[3],
                    (p.zp.y * c[0] - c[1] * p.wbv.y - c[2] * p.wcv.y) * c[3]};
      reinterpret_cast<C2<T> *>(wa)[i] = w;
      reinterpret_cast<C2<T> *>(xsol)[i] = C2<T>{p.xs.x + c[4] * w.x, p.xs.y + c[4] * w.y};
    }
    return (double)(p.xi.x * yr + p.xi.y * yi);
  }
  // the finishing thread turns <z, J z> into the Lanczos coefficients
  __device__ void hook(double total) const { minres_lanczos_coefs(const_cast<MinresScalars *>(s), total); }
};

template <typename T>
__global__ void minres_wx(int64_t n, const MinresScalars *__restrict__ s, const T *__restrict__ z,
                          T *__restrict__ wa, const T *__restrict__ wb, const T *__restrict__ wc,
                          T *__restrict__ x) {
  if (!s->wx_pending) return;
  const T *c = wx_coef<T>(s);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    minres_wx_elem<T>(c, i, z, wa, wb, wc, x);
}

__global__ void clear_wx_pending(MinresScalars *s) { s->wx_pending = 0; }

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
  for (DevBuf<T> *b : {&r[0], &r[1], &z[0], &z[1], &w[0], &w[1], &w[2], &u, &x}) b->alloc(n2);
  sc.alloc(1);
  NOSH_CUDA(cudaMallocHost(&h_sc, sizeof(MinresScalars)));
  NOSH_CUDA(cudaMallocHost(&h_err, 2 * sizeof(int)));
  NOSH_CUDA(cudaMallocHost(&h_params, 2 * sizeof(double)));
  params.alloc(2);
  NOSH_CUDA(cudaFuncSetAttribute(row_block_apply<T, JacMinresOp<T>>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024));
}

template <typename T>
void Minres<T>::drop_graphs() {
  for (cudaGraphExec_t &e : part_exec) {
    if (e) cudaGraphExecDestroy(e);
    e = nullptr;
  }
  if (pro_exec) cudaGraphExecDestroy(pro_exec);
  pro_exec = nullptr;
  pro_b = nullptr;
  for (auto &part : part_ev)
    for (auto &it : part)
      for (auto &v : it) KernelTimer::release(v);
  for (auto &v : pro_ev) KernelTimer::release(v);
}

template <typename T>
Minres<T>::~Minres() {
  drop_graphs();
  if (h_params) cudaFreeHost(h_params);
  if (h_sc) cudaFreeHost(h_sc);
  if (h_err) cudaFreeHost(h_err);
}

// Iteration j of a chunk.  Buffer roles rotate with period 2 (z, r) and 3
// (w: the (w1, w2, w) triple of the recurrence), so a chunk of 6 iterations
// always starts from the same assignment.
template <typename T>
void Minres<T>::iteration(int j) {
  cudaStream_t st = s.stream;
  MinresScalars *d = sc.p;
  T *zc = z[j % 2].p, *zn = z[(j + 1) % 2].p;
  T *r_old = r[j % 2].p, *r_cur = r[(j + 1) % 2].p;
  // deferred w/x update of step j-1: its z is zn, its (w1, w2, w) buffers
  const int jm = (j + kChunk - 1) % 3;
  T *wa = w[jm].p, *wb = w[(jm + 1) % 3].p, *wc = w[(jm + 2) % 3].p;
  const int cap = sizeof(T) == 4 ? s.cap32 : s.cap64;
  const C2<T> *val = sizeof(T) == 4 ? (const C2<T> *)s.d_keo32.p : (const C2<T> *)s.d_keo64.p;
  const T *jd = sizeof(T) == 4 ? (const T *)s.d_jd32.p : (const T *)s.d_jd64.p;
  JacMinresOp<T> op{jd, (const C2<T> *)zc, (C2<T> *)u.p, d, zn, wa, wb, wc, x.p, &d->done};
  s.timers[NOSH_KERNEL_JACOBIAN].begin(st);
  // overlaps the previous iteration's last V-cycle launch (the KEO values
  // were assembled before the solve)
  const bool overlap = s.overlap_launches && !s.timers[NOSH_KERNEL_JACOBIAN].on;
  launch_spmv<T>(sizeof(T) == 4 ? s.warp32 : s.warp64, (int)s.N, s.mesh->d_rp.p, s.mesh->d_ci.p, val,
                 (const C2<T> *)zc, cap, op, s.red.partials.p, s.red.counter.p, &d->zu, st, overlap);
  ++s.launch_count;
  // values per vertex: z (2) and the diagonal block (3) read, u (2) written;
  // the fused w/x update reads z_prev, w2, w, x and writes w1, x (12).  The
  // first launch of a solve has no update pending (7: see the harvest)
  s.timers[NOSH_KERNEL_JACOBIAN].end(st, s.spmv_bytes(2 * sizeof(T), 19 * sizeof(T)));
  s.amg->apply_minres<T>(d, u.p, r_old, r_cur, zn);
}

template <typename T>
void Minres<T>::wx_final(int j) {
  // the update iteration j + 1 would have fused: z = z[j % 2], (w1, w2, w) =
  // (w[j % 3], w[(j + 1) % 3], w[(j + 2) % 3])
  const int G = std::min<int64_t>(div_up(n2, 256), kNumSMs * 8);
  minres_wx<T><<<G, 256, 0, s.stream>>>(n2, sc.p, z[j % 2].p, w[j % 3].p, w[(j + 1) % 3].p, w[(j + 2) % 3].p,
                                        x.p);
  clear_wx_pending<<<1, 1, 0, s.stream>>>(sc.p);
  s.launch_count += 2;
}

template <typename T>
int Minres<T>::solve(const T *b, double rtol, int maxit, int &status, double &rel_res) {
  cudaStream_t st = s.stream;
  const int G = vec_grid(n2);
  const size_t bytes = n2 * sizeof(T);
  MinresScalars *d = sc.p;
  // with kernel timing on, the graphs carry event-record nodes around the
  // timed launches: captured anew when timing is switched
  const bool timed = s.timers[NOSH_KERNEL_JACOBIAN].on || s.timers[NOSH_KERNEL_SMOOTHER].on;
  if (timed != graphs_timed) {
    NOSH_CUDA(cudaStreamSynchronize(st));
    drop_graphs();
    graphs_timed = timed;
  }
  h_params[0] = rtol;
  h_params[1] = (double)maxit;
  NOSH_CUDA(cudaMemcpyAsync(params.p, h_params, 2 * sizeof(double), cudaMemcpyHostToDevice, st));
  // prologue: r_old = r_cur = b, x = w = 0, z = M b, beta1^2 = <b, z>; one
  // captured graph for a given right-hand-side buffer
  auto prologue = [&] {
    NOSH_CUDA(cudaMemcpyAsync(r[0].p, b, bytes, cudaMemcpyDeviceToDevice, st));
    NOSH_CUDA(cudaMemcpyAsync(r[1].p, b, bytes, cudaMemcpyDeviceToDevice, st));
    for (DevBuf<T> *q : {&x, &w[0], &w[1], &w[2]}) NOSH_CUDA(cudaMemsetAsync(q->p, 0, bytes, st));
    s.amg->apply<T>(r[1].p, z[0].p);
    dot_kernel<T><<<reduce_grid(n2), 256, 0, st>>>(n2, r[1].p, z[0].p, s.red.partials.p, s.red.counter.p,
                                                    &d->rz);
    minres_init<<<1, 1, 0, st>>>(d, params.p);
    s.launch_count += 2;
  };
  {
    if (!pro_exec || pro_b != b) {
      if (pro_exec) {
        NOSH_CUDA(cudaStreamSynchronize(st));
        NOSH_CUDA(cudaGraphExecDestroy(pro_exec));
      }
      for (auto &v : pro_ev) KernelTimer::release(v);
      cudaGraph_t g;
      const int64_t before = s.launch_count;
      NOSH_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      prologue();
      NOSH_CUDA(cudaStreamEndCapture(st, &g));
      for (int k = 0; k < 2; k++) pro_ev[k] = s.timers[k].take();
      pro_kernels = s.launch_count - before;
      s.launch_count = before;
      NOSH_CUDA(cudaGraphInstantiate(&pro_exec, g, 0));
      NOSH_CUDA(cudaGraphDestroy(g));
      pro_b = b;
    }
    NOSH_CUDA(cudaGraphLaunch(pro_exec, st));
    s.launch_count += pro_kernels;
  }
  NOSH_CUDA(cudaGetLastError());
  if (!part_exec[0]) {
    for (int h = 0; h < kParts; h++) {
      cudaGraph_t g;
      const int64_t before = s.launch_count;
      NOSH_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      for (int j = h * kPart; j < (h + 1) * kPart; j++) {
        iteration(j);
        for (int k = 0; k < 2; k++) part_ev[h][j - h * kPart][k] = s.timers[k].take();
      }
      NOSH_CUDA(cudaStreamEndCapture(st, &g));
      part_kernels[h] = s.launch_count - before;
      s.launch_count = before;
      NOSH_CUDA(cudaGraphInstantiate(&part_exec[h], g, 0));
      NOSH_CUDA(cudaGraphDestroy(g));
    }
  }
  auto launch_part = [&](int h) {
    NOSH_CUDA(cudaGraphLaunch(part_exec[h], st));
    s.launch_count += part_kernels[h];
  };
  // first batch: as many parts as the previous solve used (one chunk at
  // first); one part per poll when timing, so that every replay's events
  // are read before the part is replayed again
  int batch = timed ? 1 : last_its > 0 ? (last_its + kPart - 1) / kPart : kParts;
  int it = 0, h = 0;
  bool first = true;
  for (;;) {
    const int it0 = it, h0 = h;
    for (int q = 0; q < batch; q++, h = (h + 1) % kParts, it += kPart) launch_part(h);
    batch = 1;
    NOSH_CUDA(cudaGetLastError());
    NOSH_CUDA(cudaMemcpyAsync(h_sc, d, sizeof(MinresScalars), cudaMemcpyDeviceToHost, st));
    NOSH_CUDA(cudaMemcpyAsync(h_err, s.amg->error_flag_ptr(), sizeof(int), cudaMemcpyDeviceToHost, st));
    NOSH_CUDA(cudaMemcpyAsync(h_err + 1, s.red.counter.p + kStageErrorSlot, sizeof(int), cudaMemcpyDeviceToHost,
                              st));
    NOSH_CUDA(cudaStreamSynchronize(st));
    if (timed) {
      // the launches that did work: iteration g's Jacobian apply runs unless
      // the recurrence was frozen before it (it runs in the iteration after
      // convergence, which applies the last w/x update), its V-cycle unless
      // the solve converged before it (then itn <= g)
      if (first)
        for (int k = 0; k < 2; k++)
          for (const auto &p : pro_ev[k]) s.timers[k].harvest(p);
      const int jac_end = h_sc->itn + (h_sc->done ? 1 : 0);
      // the solve's first Jacobian apply has no deferred w/x update to apply
      const double jac_first = s.spmv_bytes(2 * sizeof(T), 7 * sizeof(T));
      for (int jj = 0; jj < kPart; jj++) {
        const int g = it0 + jj;
        if (g < jac_end)
          for (const auto &p : part_ev[h0][jj][NOSH_KERNEL_JACOBIAN])
            s.timers[NOSH_KERNEL_JACOBIAN].harvest(p, g == 0 ? jac_first : -1.0);
        if (g < h_sc->itn)
          for (const auto &p : part_ev[h0][jj][NOSH_KERNEL_SMOOTHER]) s.timers[NOSH_KERNEL_SMOOTHER].harvest(p);
      }
    }
    first = false;
    if (h_sc->done || h_err[1] != 0 || it >= maxit + kChunk) break;
  }
  // converged on the last issued iteration: its w/x update is still due
  // (h is the next part; the last issued iteration ends the part before it)
  if (h_sc->wx_pending) wx_final(((h + kParts - 1) % kParts + 1) * kPart - 1);
  if (h_err[1] != 0) s.stage_failure();
  if (h_err[0] != 0) {
    s.amg->clear_error();
    throw Error(NOSH_ERR_BREAKDOWN,
                "the regularised KEO or a level of its AMG hierarchy is not positive definite "
                "(a diagonal block or a coarsest pivot)");
  }
  status = h_sc->flag;
  rel_res = h_sc->beta1 > 0 ? h_sc->phibar / h_sc->beta1 : 0.0;
  last_its = h_sc->itn;
  return h_sc->itn;
}

template struct Minres<float>;
template struct Minres<double>;

// ------------------------------------------------------------------ Newton
namespace {

// c = sum conj(a_i) b_i (complex), deterministic two-slot reduction
__global__ void cdot_kernel(int64_t n, const C2<double> *__restrict__ a,
                            const C2<double> *__restrict__ b, double *partials,
                            unsigned *counter, double *out) {
  double re = 0.0, im = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const C2<double> x = a[i], y = b[i];
    re += x.x * y.x + x.y * y.y;
    im += x.x * y.y - x.y * y.x;
  }
  const double v[2] = {re, im};
  grid_reduce_n<2>(v, 2, partials, counter, out);
}

// secant prediction x_new = x + r (x - e^{i phi} x_prev), e^{i phi} = c (the
// unit phase factor aligning x_prev to x); x_prev <- x
__global__ void secant_kernel(int64_t n, const double *__restrict__ c, double r,
                              C2<double> *__restrict__ xn, C2<double> *__restrict__ x,
                              C2<double> *__restrict__ xp) {
  const double er = c[0], ei = c[1];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const C2<double> a = x[i], p = xp[i];
    const double pr = er * p.x - ei * p.y, pi = er * p.y + ei * p.x;
    xn[i] = C2<double>{a.x + r * (a.x - pr), a.y + r * (a.y - pi)};
    xp[i] = a;
  }
}

template <typename T>
__global__ void cast_to(int64_t n, const double *__restrict__ a, T *__restrict__ b) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (T)a[i];
}
template <typename T>
__global__ void cast_from(int64_t n, const T *__restrict__ a, double *__restrict__ b) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (double)a[i];
}

// <i psi, x> and |psi|^2 over complex entries (x in the Krylov precision)
template <typename T>
__global__ void gauge_dots(int64_t n, const T *__restrict__ x, const double *__restrict__ psi, double *partials,
                           unsigned *counter, double *out) {
  double a = 0.0, b = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double pr = psi[2 * i], pi = psi[2 * i + 1];
    a += pr * (double)x[2 * i + 1] - pi * (double)x[2 * i];
    b += pr * pr + pi * pi;
  }
  const double v[2] = {a, b};
  grid_reduce_n<2>(v, 2, partials, counter, out);
}

// x -= (<i psi, x> / |psi|^2) i psi, the coefficients from gauge_dots
template <typename T>
__global__ void gauge_remove(int64_t n, T *__restrict__ x, const double *__restrict__ psi,
                             const double *__restrict__ d) {
  const double k = d[1] > 0.0 ? d[0] / d[1] : 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[2 * i] = (T)((double)x[2 * i] + k * psi[2 * i + 1]);
    x[2 * i + 1] = (T)((double)x[2 * i + 1] - k * psi[2 * i]);
  }
}

template <typename T>
__global__ void axpy_to(int64_t n, double a, const T *__restrict__ t, const double *__restrict__ x,
                        double *__restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = x[i] + a * (double)t[i];
}
}  // namespace

void reset_preconditioner(NlsImpl &s) {
  // the MINRES graphs capture the hierarchy's buffers: drop them with it
  if (s.solver_state) {
    NewtonState &ns = *(NewtonState *)s.solver_state.get();
    ns.m32.reset();
    ns.m64.reset();
    ns.s32.reset();
    ns.s64.reset();
  }
  s.amg.reset();
}

NewtonState &state_of(NlsImpl &s) {
  if (!s.solver_state) {
    auto *ns = new NewtonState();
    for (DevBuf<double> *b : {&ns->psi, &ns->f, &ns->xc, &ns->xp, &ns->tmp}) b->alloc(2 * s.N);
    ns->red2.alloc(2);
    s.solver_state = std::shared_ptr<void>(ns, [](void *p) { delete (NewtonState *)p; });
  }
  return *(NewtonState *)s.solver_state.get();
}

double residual_norm(NlsImpl &s, const double *psi, double g, double mu, double *f) {
  s.compute_f64(psi, g, mu, f, 0);
  double n2 = 0.0;
  s.red.out.download(&n2, 1, s.stream);
  s.sync();
  return std::sqrt(n2);
}

// The same for ns.psi, keeping the off-diagonal sums of K psi in ns.soff
static double residual_norm_kept(NlsImpl &s, NewtonState &ns, double g, double mu) {
  ns.ensure_soff(2 * s.N);
  s.compute_f64(ns.psi.p, g, mu, ns.f.p, 0, ns.soff.p);
  double n2 = 0.0;
  s.red.out.download(&n2, 1, s.stream);
  s.sync();
  ns.soff_valid = true;
  ns.soff_fresh = true;
  ns.soff_mu = mu;
  return std::sqrt(n2);
}

// psi += dx (FP64 += FP32), and ||dx||_2^2 into *out: the per-thread sums
// in FP32 (the norm only scales a rounding bound), the grid sum in FP64
template <typename T>
__global__ void axpy_cast_norm(int64_t n, const T *__restrict__ dx, double *__restrict__ x, double *partials,
                               unsigned *counter, double *out) {
  float v = 0.0f;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const T d = dx[i];
    x[i] += (double)d;
    v += (float)d * (float)d;
  }
  grid_reduce((double)v, partials, counter, out);
}

// ns.psi += dx, then F and ||F|| of the updated state.
//
// On the mixed path, when ns.soff holds the off-diagonal sums of K psi from
// a fresh FP64 evaluation at this mu and the state is close to converged
// (||F|| <= 100 tol before the step), the update is evaluated from them:
// soff += K dx by an FP32 SpMV of the FP32 update, F = soff + the per-vertex
// FP64 terms (ResidualUpdateOp).  Beyond FP64 rounding, it deviates from
// the FP64 evaluation by the FP32 product's error alone: per real component
// of row i, at most gamma_{2n} (one rounding per real multiply-add of the
// row's 2n, n <= n_max off-diagonal nonzeros) plus 2^-24 (K32 is K rounded
// per component) times sum_j |K_ij| |dx_j|, since |a x| + |b y| <= |K_ij|
// |dx_j| for K_ij = a + ib, dx_j = x + iy.  Over the 2N components, with
// || |K| ||_2 <= R (the largest row sum of |K|, |K| symmetric), that is
// sqrt(2) (2 n_max + 1) 2^-24 R ||dx||_2, taken as e = 3 (n_max + 1) 2^-24 R
// ||dx||_2 (the margin covers gamma's denominator and the FP32 sums of
// ||dx||^2).
// The estimate is kept when it decides convergence either way with margin
// e (||F|| <= tol - e, or ||F|| > tol + e with e <= ||F|| / 100, so that
// it serves as the next step's right-hand side); otherwise F is evaluated
// afresh in FP64.  Only one update follows each fresh evaluation.
template <typename T>
static double residual_after_update(NlsImpl &s, NewtonState &ns, const T *dx, double g, double mu, double fn_prev,
                                    double tol, double &bound) {
  bound = 0.0;
  const int64_t n2 = 2 * s.N;
  const bool try_update = sizeof(T) == 4 && ns.soff_valid && ns.soff_fresh && ns.soff_mu == mu &&
                          fn_prev <= 100.0 * tol;
  if (!try_update) {
    axpy_cast<T><<<vec_grid(n2), 256, 0, s.stream>>>(n2, dx, ns.psi.p);
    ++s.launch_count;
    return residual_norm_kept(s, ns, g, mu);
  }
  axpy_cast_norm<T><<<vec_grid(n2), 256, 0, s.stream>>>(n2, dx, ns.psi.p, s.red.partials.p, s.red.counter.p,
                                                        s.red.out.p + 1);
  ++s.launch_count;
  s.residual_update(ns.psi.p, (const float *)dx, g, mu, ns.f.p, ns.soff.p);
  double sq[2] = {0.0, 0.0};  // ||F||^2, ||dx||^2
  s.red.out.download(sq, 2, s.stream);
  s.sync();
  const double fn = std::sqrt(sq[0]);
  const double e = 3.0 * (s.max_row_nnz() + 1) * std::ldexp(1.0, -24) * s.keo_abs_rowmax() * std::sqrt(sq[1]);
  if (fn <= tol - e || (fn > tol + e && e <= 0.01 * fn)) {
    ns.soff_fresh = false;
    bound = e;
    return fn;
  }
  return residual_norm_kept(s, ns, g, mu);
}

Amg &ensure_preconditioner(NlsImpl &s) {
  if (!s.amg) {
    AmgOptions o;
    o.max_levels = s.amg_max_levels;
    o.coarse_size = s.amg_coarse_size;
    o.smooth_degree = s.amg_smooth_degree;
    o.reuse_period = s.amg_reuse_period;
    o.strength_threshold = s.amg_theta;
    o.cheb_ratio = s.amg_cheb_ratio;
    s.amg.reset(new Amg(s, o));
  }
  return *s.amg;
}

// Refresh the Jacobian and the preconditioner at (psi, g, mu) in precision T.
template <typename T>
static void rebuild_operators(NlsImpl &s, const double *psi, double g, double mu) {
  if constexpr (sizeof(T) == 4) {
    // the preconditioner's one-time setup (the host aggregation's strength
    // test) reads the FP64 regularised diagonal, which the mixed rebuild
    // does not write: fill it at this state first
    if (!s.amg) s.reg_rebuild(psi, g, mu);
    s.operators32_rebuild(psi, g, mu);
  } else {
    s.jac_rebuild(psi, g, mu);
    s.reg_rebuild(psi, g, mu);
  }
  ensure_preconditioner(s).refresh<T>();
}

void prebuild_operators32(NlsImpl &s, NewtonState &ns, const double *psi, double g, double mu) {
  rebuild_operators<float>(s, psi, g, mu);
  ns.ops_state = psi;
  ns.ops_g = g;
  ns.ops_mu = mu;
}

template <typename T>
static Minres<T> &minres_of(NlsImpl &s, NewtonState &ns);
template <>
Minres<float> &minres_of<float>(NlsImpl &s, NewtonState &ns) {
  if (!ns.m32) ns.m32.reset(new Minres<float>(s));
  if (ns.b32.n < (size_t)(2 * s.N)) ns.b32.alloc(2 * s.N);
  return *ns.m32;
}
template <>
Minres<double> &minres_of<double>(NlsImpl &s, NewtonState &ns) {
  if (!ns.m64) ns.m64.reset(new Minres<double>(s));
  if (ns.b64.n < (size_t)(2 * s.N)) ns.b64.alloc(2 * s.N);
  return *ns.m64;
}
template <typename T> static DevBuf<T> &rhs_of(NewtonState &ns);
template <> DevBuf<float> &rhs_of<float>(NewtonState &ns) { return ns.b32; }
template <> DevBuf<double> &rhs_of<double>(NewtonState &ns) { return ns.b64; }

double forcing_term(const nosh_newton_options &opt, int it, double fn, double fn_prev, bool fp32, double aim) {
  // FP32 Krylov cannot resolve relative residuals much below ~1e-6
  const double eta_min = fp32 ? 1e-6 : 1e-12;
  double eta;
  if (opt.forcing > 0) {
    eta = opt.forcing;
  } else {
    // Eisenstat-Walker choice 2 (gamma 0.9, alpha 2), safeguarded, no
    // tighter than needed to reach the target (refine, else tol) in one
    // step, and at most 0.3 (a sweep of 0.1 against 0.3 at 64^3: 1.58
    // against 1.41 ms per quadratic-predictor continuation step, same
    // Newton steps)
    const double target = opt.refine > 0.0 ? opt.refine : opt.tol;
    const double ew = it == 0 ? 1e-2 : 0.9 * (fn / fn_prev) * (fn / fn_prev);
    // (the margin `aim` < 1 keeps a one-step target reachable when the cap
    // is the binding term: the step's residual is about eta * fn)
    eta = std::min(0.3, std::max(ew, aim * target / fn));
  }
  return std::max(eta, eta_min);
}

template <typename T>
static MinresSys<T> &minres_sys_of(NlsImpl &s, NewtonState &ns);
template <>
MinresSys<float> &minres_sys_of<float>(NlsImpl &s, NewtonState &ns) {
  if (!ns.s32 || ns.s32->S != s.nsys()) ns.s32.reset(new MinresSys<float>(s));
  if (ns.b32.n < (size_t)(2 * s.N)) ns.b32.alloc(2 * s.N);
  return *ns.s32;
}
template <>
MinresSys<double> &minres_sys_of<double>(NlsImpl &s, NewtonState &ns) {
  if (!ns.s64 || ns.s64->S != s.nsys()) ns.s64.reset(new MinresSys<double>(s));
  if (ns.b64.n < (size_t)(2 * s.N)) ns.b64.alloc(2 * s.N);
  return *ns.s64;
}

// Newton for batched independent systems: one MINRES recurrence per system;
// a converged system gets a zero right-hand side (its update is zero: the
// Jacobian is block diagonal).
template <typename T>
static void newton_loop_systems(NlsImpl &s, NewtonState &ns, double g, double mu, const nosh_newton_options &opt,
                                nosh_newton_stats &st) {
  MinresSys<T> &mr = minres_sys_of<T>(s, ns);
  DevBuf<T> &b = rhs_of<T>(ns);
  const int64_t n2 = 2 * s.N, S = s.nsys();
  const int G = vec_grid(n2);
  ns.sys_newton.assign(S, 0);
  ns.sys_krylov.assign(S, 0);
  std::vector<double> fcur = s.h_sys_norm, rtol(S, sizeof(T) == 4 ? 1e-6 : 1e-12);
  std::vector<int> its;
  double fn = st.f_norm0, fn_prev = fn;
  ns.ops_state = nullptr;
  for (int it = 0; it < opt.max_newton && fn > opt.tol; it++) {
    rebuild_operators<T>(s, ns.psi.p, g, mu);
    s.mask_converged(ns.f.p, opt.tol);
    neg_cast<T><<<G, 256, 0, s.stream>>>(n2, ns.f.p, b.p);
    ++s.launch_count;
    // one Eisenstat-Walker forcing term from the largest residual is the
    // batch's test (the union's residual relative to its right-hand side);
    // a system that reaches the Krylov precision's floor on its own stops
    // early.  (The same term as each system's own test made the slowest
    // system of the 256-square workload take 7 Newton steps and the batch
    // 704 MINRES iterations; per-system terms, 11 Newton steps.)
    const double eta = forcing_term(opt, it, fn, fn_prev, sizeof(T) == 4, s.forcing_aim);
    int status = 0;
    st.krylov_iters += mr.solve(b.p, eta, rtol, opt.max_krylov, its, status);
    for (int64_t q = 0; q < S; q++)
      if (fcur[q] > opt.tol) {
        ns.sys_newton[q]++;
        ns.sys_krylov[q] += its[q];
      }
    if (status == NOSH_ERR_NAN || status == NOSH_ERR_BREAKDOWN) {
      s.amg->clear_error();
      st.status = status;
      return;
    }
    axpy_cast<T><<<G, 256, 0, s.stream>>>(n2, mr.x.p, ns.psi.p);
    ++s.launch_count;
    residual_norm(s, ns.psi.p, g, mu, ns.f.p);
    ns.soff_valid = false;
    fn_prev = fn;
    fn = s.system_norms(ns.f.p);
    fcur = s.h_sys_norm;
    st.newton_iters = it + 1;
    st.f_norm = fn;
    if (opt.verbose)
      std::fprintf(stderr, "newton %2d  max ||F_s|| = %.3e  minres its (largest over systems) %4d\n", it + 1, fn,
                   *std::max_element(its.begin(), its.end()));
    if (std::isnan(fn)) {
      st.status = NOSH_ERR_NAN;
      return;
    }
  }
}

// Newton on ns.psi (device), residual already in ns.f with norm st.f_norm0.
template <typename T>
static void newton_loop(NlsImpl &s, NewtonState &ns, double g, double mu,
                        const nosh_newton_options &opt, nosh_newton_stats &st) {
  if (!s.sys_off.empty() && !opt.phase_fix) {
    newton_loop_systems<T>(s, ns, g, mu, opt, st);
    return;
  }
  Minres<T> &mr = minres_of<T>(s, ns);
  DevBuf<T> &b = rhs_of<T>(ns);
  const int64_t n2 = 2 * s.N;
  const int G = vec_grid(n2);
  double fn = st.f_norm0, fn_prev = fn;
  // with a refine target, a state above 4 refine gets at least one step
  const bool polish = opt.refine > 0.0 && fn > 4.0 * opt.refine;
  const bool prebuilt = sizeof(T) == 4 && ns.ops_state == ns.psi.p && ns.ops_g == g && ns.ops_mu == mu;
  ns.ops_state = nullptr;
  for (int it = 0; it < opt.max_newton && (fn > opt.tol || (it == 0 && polish)); it++) {
    if (!(it == 0 && prebuilt)) rebuild_operators<T>(s, ns.psi.p, g, mu);
    // batched systems: converged ones get a zero right-hand side (their
    // Newton update is zero: the Jacobian is block diagonal)
    if (!s.sys_off.empty()) s.mask_converged(ns.f.p, opt.tol);
    neg_cast<T><<<G, 256, 0, s.stream>>>(n2, ns.f.p, b.p);
    ++s.launch_count;
    const double eta = forcing_term(opt, it, fn, fn_prev, sizeof(T) == 4, s.forcing_aim);
    int status = 0;
    double rel = 0.0;
    const int its = mr.solve(b.p, eta, opt.max_krylov, status, rel);
    st.krylov_iters += its;
    if (status == NOSH_ERR_NAN || status == NOSH_ERR_BREAKDOWN) {
      // the hierarchy's coarse operators are rebuilt in full next time, so
      // a later solve does not inherit the failed ones
      s.amg->clear_error();
      st.status = status;
      return;
    }
    if (opt.phase_fix) {
      // the bordered system's update: no component along i psi
      const int Gc = vec_grid(s.N);
      gauge_dots<T><<<reduce_grid(s.N), 256, 0, s.stream>>>(s.N, mr.x.p, ns.psi.p, s.red.partials.p, s.red.counter.p,
                                               ns.red2.p);
      gauge_remove<T><<<Gc, 256, 0, s.stream>>>(s.N, mr.x.p, ns.psi.p, ns.red2.p);
      s.launch_count += 2;
    }
    fn_prev = fn;
    if (s.sys_off.empty()) {
      double bound = 0.0;
      fn = residual_after_update<T>(s, ns, mr.x.p, g, mu, fn_prev, opt.tol, bound);
      st.f_norm_bound = bound;
      if (bound > 0.0) ++st.residual_updates;
    } else {
      axpy_cast<T><<<G, 256, 0, s.stream>>>(n2, mr.x.p, ns.psi.p);
      ++s.launch_count;
      residual_norm(s, ns.psi.p, g, mu, ns.f.p);
      ns.soff_valid = false;
      fn = s.system_norms(ns.f.p);
    }
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

void newton_core(NlsImpl &s, NewtonState &ns, double g, double mu, const nosh_newton_options &opt,
                 nosh_newton_stats &st, double f0, bool soff_ready) {
  st = nosh_newton_stats{};
  if (f0 >= 0.0) {
    if (!soff_ready) ns.soff_valid = false;
    st.f_norm0 = f0;
  } else {
    st.f_norm0 = residual_norm_kept(s, ns, g, mu);
  }
  // batched systems: the largest per-system norm decides convergence
  if (!s.sys_off.empty()) st.f_norm0 = s.system_norms(ns.f.p);
  st.f_norm = st.f_norm0;
  NOSH_CHECK(!std::isnan(st.f_norm0), NOSH_ERR_NAN, "initial residual is NaN");
  if (opt.precision == NOSH_PREC_FP64) newton_loop<double>(s, ns, g, mu, opt, st);
  else newton_loop<float>(s, ns, g, mu, opt, st);
  if (st.status == NOSH_OK && !(st.f_norm <= opt.tol)) st.status = NOSH_ERR_NOT_CONVERGED;
}

void newton_solve(NlsImpl &s, double *x_user, double g, double mu, const nosh_newton_options &opt,
                  nosh_newton_stats &st) {
  NewtonState &ns = state_of(s);
  const size_t bytes = 2 * s.N * sizeof(double);
  NOSH_CUDA(cudaMemcpyAsync(ns.psi.p, x_user, bytes, cudaMemcpyDefault, s.stream));
  newton_core(s, ns, g, mu, opt, st);
  NOSH_CUDA(cudaMemcpyAsync(x_user, ns.psi.p, bytes, cudaMemcpyDefault, s.stream));
  s.sync();
}

template <typename T>
static void tangent_predict(NlsImpl &s, NewtonState &ns, double g, double mu_cur, double dmu,
                            const nosh_newton_options &opt, nosh_newton_stats &st) {
  // dx/dmu = -J^-1 dF/dmu at (x, mu_cur) (LOCA tangent predictor; dF/dmu is
  // DkeoDP x, src/model_evaluator_nls.cpp:632-695)
  Minres<T> &mr = minres_of<T>(s, ns);
  DevBuf<T> &b = rhs_of<T>(ns);
  const int64_t n2 = 2 * s.N;
  const int G = vec_grid(n2);
  rebuild_operators<T>(s, ns.xc.p, g, mu_cur);
  s.dfdp64(ns.xc.p, g, mu_cur, 1, ns.tmp.p);
  neg_cast<T><<<G, 256, 0, s.stream>>>(n2, ns.tmp.p, b.p);
  ++s.launch_count;
  int status = 0;
  double rel = 0.0;
  st.krylov_iters += mr.solve(b.p, sizeof(T) == 4 ? 1e-5 : 1e-8, opt.max_krylov, status, rel);
  NOSH_CHECK(status != NOSH_ERR_NAN && status != NOSH_ERR_BREAKDOWN, status, "tangent solve failed");
  axpy_to<T><<<G, 256, 0, s.stream>>>(n2, dmu, mr.x.p, ns.xc.p, ns.psi.p);
  ++s.launch_count;
}

// J(psi at ns.psi, g, mu) x = rhs (FP64 in and out, 2N reals), solved by the
// preconditioned MINRES in the requested precision to relative tolerance
// rtol; the operators are rebuilt at (ns.psi, mu) when `rebuild`.
template <typename T>
static int linear_solve_t(NlsImpl &s, NewtonState &ns, const double *rhs, double *x, double g, double mu,
                          double rtol, int maxit, bool rebuild, int &status) {
  Minres<T> &mr = minres_of<T>(s, ns);
  DevBuf<T> &b = rhs_of<T>(ns);
  const int64_t n2 = 2 * s.N;
  const int G = vec_grid(n2);
  if (rebuild) rebuild_operators<T>(s, ns.psi.p, g, mu);
  cast_to<T><<<G, 256, 0, s.stream>>>(n2, rhs, b.p);
  ++s.launch_count;
  double rel = 0.0;
  const int its = mr.solve(b.p, rtol, maxit, status, rel);
  cast_from<T><<<G, 256, 0, s.stream>>>(n2, mr.x.p, x);
  ++s.launch_count;
  NOSH_CUDA(cudaGetLastError());
  return its;
}

int linear_solve(NlsImpl &s, NewtonState &ns, const double *rhs, double *x, double g, double mu, double rtol,
                 int maxit, int precision, bool rebuild, int &status) {
  return precision == NOSH_PREC_FP64 ? linear_solve_t<double>(s, ns, rhs, x, g, mu, rtol, maxit, rebuild, status)
                                     : linear_solve_t<float>(s, ns, rhs, x, g, mu, rtol, maxit, rebuild, status);
}

void continuation_step(NlsImpl &s, double *x, double *x_prev, double g, double mu_new, double mu_cur,
                       double mu_prev, int predictor, const nosh_newton_options &opt,
                       nosh_newton_stats &st) {
  NewtonState &ns = state_of(s);
  const size_t bytes = 2 * s.N * sizeof(double);
  const int64_t n2 = 2 * s.N;
  const int G = vec_grid(n2);
  cudaStream_t st_ = s.stream;
  NOSH_CUDA(cudaMemcpyAsync(ns.xc.p, x, bytes, cudaMemcpyDefault, st_));
  nosh_newton_stats pst{};
  if (predictor == NOSH_PREDICT_SECANT && x_prev && mu_cur != mu_prev && !std::isnan(mu_prev)) {
    NOSH_CUDA(cudaMemcpyAsync(ns.xp.p, x_prev, bytes, cudaMemcpyDefault, st_));
    cdot_kernel<<<reduce_grid(s.N), 256, 0, st_>>>(s.N, (const C2<double> *)ns.xp.p, (const C2<double> *)ns.xc.p,
                                    s.red.partials.p, s.red.counter.p, ns.red2.p);
    normalize_phases<<<1, 32, 0, st_>>>(1, ns.red2.p);
    s.launch_count += 2;
    secant_kernel<<<G, 256, 0, st_>>>(s.N, ns.red2.p, (mu_new - mu_cur) / (mu_cur - mu_prev),
                                      (C2<double> *)ns.psi.p, (C2<double> *)ns.xc.p,
                                      (C2<double> *)ns.xp.p);
    ++s.launch_count;
    NOSH_CUDA(cudaGetLastError());
    NOSH_CUDA(cudaMemcpyAsync(x_prev, ns.xp.p, bytes, cudaMemcpyDefault, st_));
  } else if (predictor == NOSH_PREDICT_TANGENT) {
    if (opt.precision == NOSH_PREC_FP64) tangent_predict<double>(s, ns, g, mu_cur, mu_new - mu_cur, opt, pst);
    else tangent_predict<float>(s, ns, g, mu_cur, mu_new - mu_cur, opt, pst);
    if (x_prev) NOSH_CUDA(cudaMemcpyAsync(x_prev, ns.xc.p, bytes, cudaMemcpyDefault, st_));
  } else {
    NOSH_CUDA(cudaMemcpyAsync(ns.psi.p, ns.xc.p, bytes, cudaMemcpyDeviceToDevice, st_));
    if (x_prev) NOSH_CUDA(cudaMemcpyAsync(x_prev, ns.xc.p, bytes, cudaMemcpyDefault, st_));
  }
  newton_core(s, ns, g, mu_new, opt, st);
  st.krylov_iters += pst.krylov_iters;
  NOSH_CUDA(cudaMemcpyAsync(x, ns.psi.p, bytes, cudaMemcpyDefault, st_));
  s.sync();
}

}  // namespace nosh
