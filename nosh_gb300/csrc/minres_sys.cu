// Per-system preconditioned MINRES for batched independent solves.
//
// The handle's mesh is the disjoint union of S systems (nosh_nls_set_systems):
// the Jacobian and the AMG V-cycle are block diagonal by system.  This solver
// runs S Paige-Saunders recurrences over the shared vectors -- one
// MinresScalars per system -- so each system's Krylov polynomial is its own
// (a recurrence over the union would apply one polynomial to every block).
// Every launch still covers all systems:
//   u = J z              row-block SpMV whose epilogue also writes each
//                        vertex's <z_i, u_i> (rowdot)
//   <z, J z>_s           segmented reduction of rowdot over fixed chunks of
//                        each system's vertices; the last chunk of a system
//                        to finish sums the system's chunk partials in order
//                        (deterministic) and advances that system's scalars
//   r_new                per-vertex coefficients of the vertex's system
//   V-cycle              amg.cu (block diagonal: a frozen system's zero
//                        residual stays zero)
//   <r_new, z_new>_s     as above, then the Givens step of each system
//   w, x update          per-system coefficients
// A system that reaches its own relative tolerance is frozen: its residual
// block is set to zero, so the remaining launches leave its solution
// unchanged.  The batch stops as a whole once the preconditioned residual of
// the union is below eta times its right-hand side, the test one recurrence
// over the union would make (the per-system recurrences meet it in no more
// iterations in exact arithmetic, since each minimises its own block).  The
// host polls the number of running systems.
#include <algorithm>
#include <cmath>

#include "solver.cuh"
#include "spmv.cuh"

namespace nosh {

using namespace dev;

namespace {

constexpr int64_t kChunk = 4096;  // vertices per reduction chunk

// u = J z (diagonal blocks included); rowdot[i] = <z_i, u_i>
template <typename T>
struct JacRowDotOp {
  static constexpr bool kReduce = false;
  const T *d;
  const C2<T> *x;
  C2<T> *y;
  double *rowdot;
  struct Pre {
    C2<T> xi;
    T d0r, d0i, d1b;
  };
  __device__ Pre load(int i) const { return Pre{x[i], d[3 * i], d[3 * i + 1], d[3 * i + 2]}; }
  __device__ double finish(int i, T sr, T si, const Pre &p) const {
    const T yr = sr + p.d0r * p.xi.x + p.d1b * p.xi.y;
    const T yi = si + p.d1b * p.xi.x + p.d0i * p.xi.y;
    y[i] = C2<T>{yr, yi};
    rowdot[i] = (double)p.xi.x * (double)yr + (double)p.xi.y * (double)yi;
    return 0.0;
  }
};

template <typename T>
__global__ void rowdot_kernel(int64_t N, const C2<T> *__restrict__ a, const C2<T> *__restrict__ b,
                              double *__restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
    const C2<T> p = a[i], q = b[i];
    out[i] = (double)p.x * (double)q.x + (double)p.y * (double)q.y;
  }
}

// per-system scalar work once the system's sum is known
enum SysMode { kInit = 0, kLanczos = 1, kAdvance = 2 };

__device__ void sys_init(MinresScalars *s, double rz, double rtol, int maxit) {
  s->rz = rz;
  s->rtol = rtol;
  s->maxit = maxit;
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
  if (!(rz >= 0.0) || isinf(rz)) {
    s->flag = isnan(rz) || isinf(rz) ? NOSH_ERR_NAN : NOSH_ERR_BREAKDOWN;
    s->done = 2;
    s->beta1 = s->beta = s->phibar = 0.0;
    return;
  }
  s->beta1 = sqrt(rz);
  s->beta = s->beta1;
  s->phibar = s->beta1;
  if (rz == 0.0) s->done = 2;  // b_s == 0: x_s = 0
}

// grid: one CTA per chunk.  Chunk c covers vertices [cstart[c], cstart[c+1])
// of system csys[c]; system s owns chunks [schunk[s], schunk[s+1]).
template <int Mode>
__global__ void sys_reduce(const int64_t *__restrict__ cstart, const int32_t *__restrict__ csys,
                           const int32_t *__restrict__ schunk, const double *__restrict__ rowdot,
                           double *__restrict__ cpart, unsigned *__restrict__ counter, MinresScalars *sc,
                           const double *__restrict__ rtol, int maxit) {
  __shared__ double s32[32];
  __shared__ bool last;
  const int c = blockIdx.x;
  const int sy = csys[c];
  double v = 0.0;
  for (int64_t i = cstart[c] + threadIdx.x; i < cstart[c + 1]; i += blockDim.x) v += rowdot[i];
  v = block_sum(v, s32);
  const int c0 = schunk[sy], c1 = schunk[sy + 1];
  if (threadIdx.x == 0) {
    cpart[c] = v;
    __threadfence();
    const unsigned t = atomicAdd(counter + sy, 1u);
    last = (t == (unsigned)(c1 - c0 - 1));
  }
  __syncthreads();
  if (!last || threadIdx.x != 0) return;
  __threadfence();
  double tot = 0.0;
  for (int q = c0; q < c1; q++) tot += __ldcg(cpart + q);
  counter[sy] = 0u;
  MinresScalars *s = sc + sy;
  if (Mode == kInit) sys_init(s, tot, rtol[sy], maxit);
  else if (Mode == kLanczos) minres_lanczos_coefs(s, tot);
  else minres_advance(s, tot);
}

// r_old <- la0 u - la1 r_old - la2 r_cur (the new Lanczos vector, zero for
// a frozen system)
template <typename T>
__global__ void lanczos_sys(int64_t N, const int32_t *__restrict__ vsys, const MinresScalars *__restrict__ sc,
                            const C2<T> *__restrict__ u, C2<T> *__restrict__ r_old, const C2<T> *__restrict__ r_cur) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
    const MinresScalars *s = sc + vsys[i];
    if (s->done >= 2) {
      r_old[i] = C2<T>{0, 0};
      continue;
    }
    const T *la = lanczos_coef<T>(s);
    const C2<T> ui = u[i], ro = r_old[i], rc = r_cur[i];
    r_old[i] = C2<T>{la[0] * ui.x - la[1] * ro.x - la[2] * rc.x, la[0] * ui.y - la[1] * ro.y - la[2] * rc.y};
  }
}

// w = (z c0 - c1 w2 - c2 w) c3 over the w1 buffer, x += c4 w, for systems
// whose Givens step is pending
template <typename T>
__global__ void wx_sys(int64_t N, const int32_t *__restrict__ vsys, const MinresScalars *__restrict__ sc,
                       const T *__restrict__ z, T *__restrict__ wa, const T *__restrict__ wb,
                       const T *__restrict__ wc, T *__restrict__ x) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
    const MinresScalars *s = sc + vsys[i];
    if (!s->wx_pending) continue;
    const T *c = wx_coef<T>(s);
    minres_wx_elem<T>(c, 2 * i, z, wa, wb, wc, x);
    minres_wx_elem<T>(c, 2 * i + 1, z, wa, wb, wc, x);
  }
}

// One CTA after every Givens step: clears the pending w/x updates, counts
// the running systems into *active, and applies the batch's stopping test
// sum_s phibar_s^2 <= eta^2 sum_s beta1_s^2; when it holds every running
// system stops (done = 1: frozen at its next Lanczos step).
__global__ void batch_check(int S, MinresScalars *sc, const double *eta_p, int *active) {
  const double eta = *eta_p;
  __shared__ double s32[32];
  __shared__ bool stop;
  double num = 0.0, den = 0.0, run = 0.0;
  for (int q = threadIdx.x; q < S; q += blockDim.x) {
    MinresScalars *s = sc + q;
    s->wx_pending = 0;
    num += s->phibar * s->phibar;
    den += s->beta1 * s->beta1;
    run += s->done == 0 ? 1.0 : 0.0;
  }
  num = block_sum(num, s32);
  den = block_sum(den, s32);
  run = block_sum(run, s32);
  if (threadIdx.x == 0) stop = !(num > eta * eta * den);
  __syncthreads();
  if (stop)
    for (int q = threadIdx.x; q < S; q += blockDim.x)
      if (sc[q].done == 0) sc[q].done = 1;
  if (threadIdx.x == 0) *active = stop ? 0 : (int)run;
}

inline int egrid(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>(div_up(n, 256), kNumSMs * 8)); }

}  // namespace

template <typename T>
MinresSys<T>::MinresSys(NlsImpl &nls) : s(nls), N(nls.N), S(nls.nsys()) {
  for (DevBuf<T> *b : {&r[0], &r[1], &z[0], &z[1], &w[0], &w[1], &w[2], &u, &x}) b->alloc(2 * N);
  rowdot.alloc(N);
  sc.alloc(S);
  rtol.alloc(S);
  counter.alloc(S);
  counter.zero(s.stream);
  active.alloc(1);
  // vertex -> system, and reduction chunks that never straddle two systems
  std::vector<int32_t> vs(N);
  std::vector<int64_t> cs;
  std::vector<int32_t> csy, sch(S + 1, 0);
  for (int64_t q = 0; q < S; q++) {
    const int64_t a = s.sys_off[q], b = s.sys_off[q + 1];
    for (int64_t i = a; i < b; i++) vs[i] = (int32_t)q;
    sch[q] = (int32_t)csy.size();
    for (int64_t c = a; c < b; c += kChunk) {
      cs.push_back(c);
      csy.push_back((int32_t)q);
    }
  }
  sch[S] = (int32_t)csy.size();
  cs.push_back(N);
  nchunks = (int)csy.size();
  vsys.upload(vs, s.stream);
  cstart.upload(cs, s.stream);
  csys.upload(csy, s.stream);
  schunk.upload(sch, s.stream);
  cpart.alloc(nchunks);
  h_sc.resize(S);
  NOSH_CUDA(cudaMallocHost(&h_active, sizeof(int)));
  NOSH_CUDA(cudaMallocHost(&h_err, sizeof(int)));
  NOSH_CUDA(cudaMallocHost(&h_eta, sizeof(double)));
  eta.alloc(1);
  NOSH_CUDA(cudaFuncSetAttribute(row_block_apply<T, JacRowDotOp<T>>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 100 * 1024));
  s.sync();
}

template <typename T>
MinresSys<T>::~MinresSys() {
  if (chunk_exec) cudaGraphExecDestroy(chunk_exec);
  if (h_active) cudaFreeHost(h_active);
  if (h_err) cudaFreeHost(h_err);
  if (h_eta) cudaFreeHost(h_eta);
}

// Iteration j (0..5) of a chunk: buffer roles rotate with periods 2 (z, r)
// and 3 (w), so six iterations always start from the same assignment.
template <typename T>
void MinresSys<T>::iteration(int j, int maxit) {
  cudaStream_t st = s.stream;
  const int G = egrid(N);
  const int cap = sizeof(T) == 4 ? s.cap32 : s.cap64;
  const C2<T> *val = sizeof(T) == 4 ? (const C2<T> *)s.d_keo32.p : (const C2<T> *)s.d_keo64.p;
  const T *jd = sizeof(T) == 4 ? (const T *)s.d_jd32.p : (const T *)s.d_jd64.p;
  const bool warp = sizeof(T) == 4 ? s.warp32 : s.warp64;
  T *zc = z[j % 2].p, *zn = z[(j + 1) % 2].p;
  T *r_old = r[j % 2].p, *r_cur = r[(j + 1) % 2].p;
  JacRowDotOp<T> op{jd, (const C2<T> *)zc, (C2<T> *)u.p, rowdot.p};
  launch_spmv<T>(warp, (int)N, s.mesh->d_rp.p, s.mesh->d_ci.p, val, (const C2<T> *)zc, cap, op, s.red.partials.p,
                 s.red.counter.p, nullptr, st);
  ++s.launch_count;
  reduce(kLanczos, maxit);
  lanczos_sys<T><<<G, 256, 0, st>>>(N, vsys.p, sc.p, (const C2<T> *)u.p, (C2<T> *)r_old, (const C2<T> *)r_cur);
  ++s.launch_count;
  s.amg->apply<T>(r_old, zn);
  rowdot_kernel<T><<<G, 256, 0, st>>>(N, (const C2<T> *)r_old, (const C2<T> *)zn, rowdot.p);
  ++s.launch_count;
  reduce(kAdvance, maxit);
  // the Givens step's w/x update: v = z of this iteration / beta
  wx_sys<T><<<G, 256, 0, st>>>(N, vsys.p, sc.p, zc, w[j % 3].p, w[(j + 1) % 3].p, w[(j + 2) % 3].p, x.p);
  batch_check<<<1, 1024, 0, st>>>((int)S, sc.p, eta.p, active.p);
  s.launch_count += 2;
  NOSH_CUDA(cudaGetLastError());
}

template <typename T>
void MinresSys<T>::reduce(int mode, int maxit) {
  cudaStream_t st = s.stream;
  if (mode == kInit)
    sys_reduce<kInit><<<nchunks, 256, 0, st>>>(cstart.p, csys.p, schunk.p, rowdot.p, cpart.p, counter.p, sc.p,
                                               rtol.p, maxit);
  else if (mode == kLanczos)
    sys_reduce<kLanczos><<<nchunks, 256, 0, st>>>(cstart.p, csys.p, schunk.p, rowdot.p, cpart.p, counter.p, sc.p,
                                                  rtol.p, maxit);
  else
    sys_reduce<kAdvance><<<nchunks, 256, 0, st>>>(cstart.p, csys.p, schunk.p, rowdot.p, cpart.p, counter.p, sc.p,
                                                  rtol.p, maxit);
  ++s.launch_count;
}

template <typename T>
int MinresSys<T>::solve(const T *b, double eta, const std::vector<double> &rtol_host, int maxit,
                        std::vector<int> &its, int &status) {
  cudaStream_t st = s.stream;
  const int64_t n2 = 2 * N;
  const size_t bytes = n2 * sizeof(T);
  const int G = egrid(N);
  rtol.upload(rtol_host.data(), S, st);
  *h_eta = eta;
  NOSH_CUDA(cudaMemcpyAsync(this->eta.p, h_eta, sizeof(double), cudaMemcpyHostToDevice, st));
  // prologue: r_old = r_cur = b, x = w = 0, z = M b, <b, z>_s
  NOSH_CUDA(cudaMemcpyAsync(r[0].p, b, bytes, cudaMemcpyDeviceToDevice, st));
  NOSH_CUDA(cudaMemcpyAsync(r[1].p, b, bytes, cudaMemcpyDeviceToDevice, st));
  for (DevBuf<T> *q : {&x, &w[0], &w[1], &w[2]}) NOSH_CUDA(cudaMemsetAsync(q->p, 0, bytes, st));
  s.amg->apply<T>(r[1].p, z[0].p);
  rowdot_kernel<T><<<G, 256, 0, st>>>(N, (const C2<T> *)r[1].p, (const C2<T> *)z[0].p, rowdot.p);
  ++s.launch_count;
  reduce(kInit, maxit);
  NOSH_CUDA(cudaGetLastError());
  // the six iterations of a chunk are captured once as a CUDA graph (the
  // tolerance and iteration limit reach it through device memory), unless
  // kernel timing is on
  const bool graphs = !s.timers[NOSH_KERNEL_JACOBIAN].on;
  if (graphs && (!chunk_exec || chunk_maxit != maxit)) {
    if (chunk_exec) NOSH_CUDA(cudaGraphExecDestroy(chunk_exec));
    chunk_exec = nullptr;
    cudaGraph_t g;
    const int64_t before = s.launch_count;
    NOSH_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    for (int q = 0; q < 6; q++) iteration(q, maxit);
    NOSH_CUDA(cudaStreamEndCapture(st, &g));
    chunk_kernels = s.launch_count - before;
    s.launch_count = before;
    NOSH_CUDA(cudaGraphInstantiate(&chunk_exec, g, 0));
    NOSH_CUDA(cudaGraphDestroy(g));
    chunk_maxit = maxit;
  }
  int it = 0;
  for (;;) {
    // a chunk of iterations between two polls of the running count
    if (graphs) {
      NOSH_CUDA(cudaGraphLaunch(chunk_exec, st));
      s.launch_count += chunk_kernels;
    } else {
      for (int q = 0; q < 6; q++) iteration(q, maxit);
    }
    it += 6;
    NOSH_CUDA(cudaMemcpyAsync(h_active, active.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    s.sync();
    if (*h_active <= 0 || it >= maxit + 6) break;
  }
  NOSH_CUDA(cudaMemcpyAsync(h_sc.data(), sc.p, S * sizeof(MinresScalars), cudaMemcpyDeviceToHost, st));
  NOSH_CUDA(cudaMemcpyAsync(h_err, s.amg->error_flag_ptr(), sizeof(int), cudaMemcpyDeviceToHost, st));
  s.sync();
  if (*h_err != 0) {
    s.amg->clear_error();
    throw Error(NOSH_ERR_BREAKDOWN,
                "the regularised KEO or a level of its AMG hierarchy is not positive definite "
                "(a diagonal block or a coarsest pivot)");
  }
  its.assign(S, 0);
  status = NOSH_OK;
  int mx = 0;
  for (int64_t q = 0; q < S; q++) {
    its[q] = h_sc[q].itn;
    mx = std::max(mx, its[q]);
    const int f = h_sc[q].flag;
    if (f == NOSH_ERR_NAN || f == NOSH_ERR_BREAKDOWN) status = f;
    else if (f == NOSH_ERR_NOT_CONVERGED && status == NOSH_OK) status = f;
  }
  return mx;
}

template struct MinresSys<float>;
template struct MinresSys<double>;

}  // namespace nosh
