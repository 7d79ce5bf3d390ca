// Model-evaluator operators on the GPU: KEO / DkeoDP assembly, F(psi),
// dF/dp, Jacobian and regularised-KEO diagonals, fused applies, energy.
#include <cmath>
#include <cstring>

#include "amg.cuh"
#include <algorithm>

#include "nls.cuh"
#include "spmv.cuh"

namespace nosh {

using namespace dev;

namespace {

// ---------------------------------------------------------------- fields
// p_e = 1/2 (A(x0) + A(x1)) . (x0 - x1)
// (vector_field::explicit_values, src/vector_field_explicit_values.cpp:31-48)
// alpha_e = covolume/length * mean thickness
// (keo::build_alpha_cache_, src/parameter_matrix_keo.cpp:221-228)
__global__ void edge_fields_kernel(int64_t E, const int32_t *__restrict__ edges,
                                   const double *__restrict__ x, const double *__restrict__ A,
                                   const double *__restrict__ len, const double *__restrict__ covol,
                                   const double *__restrict__ t, double *p, double *alpha) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= E) return;
  const int64_t a = edges[2 * e], b = edges[2 * e + 1];
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 3; k++) s += 0.5 * (A[3 * a + k] + A[3 * b + k]) * (x[3 * a + k] - x[3 * b + k]);
  const double al = covol[e] / len[e] * 0.5 * (t[a] + t[b]);
  p[e] = s;
  alpha[e] = al;
}

// K_ii = sum of alpha over the edges of row i (mu-independent), in column
// order; cvt = cv * thickness.
__global__ void vertex_fields_kernel(int64_t N, const int32_t *__restrict__ rp,
                                     const int32_t *__restrict__ nz_edge,
                                     const double *__restrict__ alpha, const double *__restrict__ cv,
                                     const double *__restrict__ t, double *kdiag, float *kdiagf,
                                     double *cvt) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= N) return;
  double s = 0.0;
  for (int k = rp[i]; k < rp[i + 1]; k++) {
    const int32_t e = nz_edge[k];
    s += alpha[e >= 0 ? e : ~e];
  }
  kdiag[i] = s;
  kdiagf[i] = (float)s;
  cvt[i] = cv[i] * t[i];
}

// --------------------------------------------------------- KEO assembly
// keo::refill_ (src/parameter_matrix_keo.cpp:106-180): per edge v0->v1,
// a = mu p_e, complex coefficient -alpha e^{-ia} at (v0,v1) and its
// conjugate at (v1,v0), written through the edge -> nonzero scatter map.
// The diagonal (sum alpha) is mu-independent and kept separately.
// sin and cos of an FP64 angle.  Magnetic phases on a mesh edge are small
// (|mu A . e| <= 0.1 covers every mesh finer than about 10 cells per unit
// field length): there the Maclaurin series of sin to x^11 and cos to x^12
// (Horner form in x^2; truncation below 1e-21 relative at |x| = 0.1) costs a
// dozen FP64 FMAs, well below a general sincos with argument reduction, which the
// larger angles still use.  Most phases are far smaller (|x| <= 0.02 on the
// 64^3 cube at mu = 1): there sin to x^7 and cos to x^8 suffice (truncation
// below 1e-18 relative), and the assembly is bound by FP64 arithmetic on
// GB300.
__device__ __forceinline__ void edge_sincos(double x, double &s, double &c) {
  // Maclaurin coefficients (-1)^k / (2k+1)! and (-1)^k / (2k)!, folded at
  // compile time; Horner in x^2 with one FMA per term
  constexpr double s1 = -1.0 / 6, s2 = 1.0 / 120, s3 = -1.0 / 5040, s4 = 1.0 / 362880, s5 = -1.0 / 39916800;
  constexpr double c1 = -1.0 / 2, c2 = 1.0 / 24, c3 = -1.0 / 720, c4 = 1.0 / 40320, c5 = -1.0 / 3628800,
                   c6 = 1.0 / 479001600;
  if (fabs(x) <= 0.02) {
    const double x2 = x * x;
    s = fma(x * x2, fma(x2, fma(x2, s3, s2), s1), x);
    c = fma(x2, fma(x2, fma(x2, fma(x2, c4, c3), c2), c1), 1.0);
  } else if (fabs(x) <= 0.1) {
    const double x2 = x * x;
    s = fma(x * x2, fma(x2, fma(x2, fma(x2, fma(x2, s5, s4), s3), s2), s1), x);
    c = fma(x2, fma(x2, fma(x2, fma(x2, fma(x2, fma(x2, c6, c5), c4), c3), c2), c1), 1.0);
  } else {
    sincos(x, &s, &c);
  }
}

// KEO assembly, edge-parallel through the scatter map (no atomics): c_e =
// -alpha_e e^{-i mu p_e} at (v0, v1), conj(c_e) at (v1, v0).  mu_sys / esys
// (optional): the edge's system supplies its own mu.  The FP32 operator of
// the mixed path is written in the same pass, each component the FP64
// value rounded to nearest (|K32 - K| <= 2^-24 |K| per component, the
// premise of the residual update's bound): the pass is bound by FP64
// arithmetic, so the extra 16 bytes per edge cost no time, and a separate
// FP32 assembly pass (16 us at 64^3) is saved.
__global__ void keo_assemble(int64_t E, const double *__restrict__ alpha, const double *__restrict__ p, double mu,
                             const int32_t *__restrict__ pf, const int32_t *__restrict__ pb,
                             C2<double> *__restrict__ val, C2<float> *__restrict__ val32,
                             const double *__restrict__ mu_sys, const int32_t *__restrict__ esys) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= E) return;
  const double m = mu_sys ? mu_sys[esys[e]] : mu;
  double s, c;
  edge_sincos(m * p[e], s, c);
  const double al = alpha[e];
  const double re = -al * c, im = al * s;
  const int32_t f = pf[e], b = pb[e];
  val[f] = C2<double>{re, im};
  val[b] = C2<double>{re, -im};
  val32[f] = C2<float>{(float)re, (float)im};
  val32[b] = C2<float>{(float)re, -(float)im};
}

// DkeoDP::refill_ (src/parameter_matrix_dkeo_dp.cpp:96-151): block entries
// v0 = alpha dp sin a, v1 = -alpha dp cos a, no diagonal.  dp = p_e for the
// derivative parameter "mu", else 0 (get_d_edge_projection_dp,
// src/vector_field_explicit_values.cpp:80-90).
__global__ void dkeo_assemble64(int64_t E, const double *__restrict__ alpha,
                                const double *__restrict__ p, double mu, double dscale,
                                const int32_t *__restrict__ pf, const int32_t *__restrict__ pb,
                                C2<double> *__restrict__ val, const double *__restrict__ mu_sys,
                                const int32_t *__restrict__ esys) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= E) return;
  const double m = mu_sys ? mu_sys[esys[e]] : mu;
  double s, c;
  edge_sincos(m * p[e], s, c);
  const double w = alpha[e] * p[e] * dscale;
  // complex v0 - i v1 at (v0,v1): w sin a + i w cos a; conjugate at (v1,v0)
  val[pf[e]] = C2<double>{w * s, w * c};
  val[pb[e]] = C2<double>{w * s, -w * c};
}

// ------------------------------------------------------------ diagonals
// jacobian_operator::rebuild_diags_ (src/jacobian_operator.cpp:184-197),
// with K_ii folded in: [[d0r, d1b], [d1b, d0i]].
__global__ void jac_diag_kernel(int64_t N, const double *__restrict__ kdiag,
                                const double *__restrict__ cvt, const double *__restrict__ V,
                                double g, const C2<double> *__restrict__ x, double *d64,
                                float *d32) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= N) return;
  const C2<double> p = x[k];
  const double w = cvt[k];
  const double al = w * (V[k] + g * 2.0 * (p.x * p.x + p.y * p.y));
  const double rx2 = g * w * (p.x * p.x - p.y * p.y);
  const double a = kdiag[k] + al + rx2, b = kdiag[k] + al - rx2, c = g * w * (2.0 * p.x * p.y);
  d64[3 * k] = a;
  d64[3 * k + 1] = b;
  d64[3 * k + 2] = c;
  d32[3 * k] = (float)a;
  d32[3 * k + 1] = (float)b;
  d32[3 * k + 2] = (float)c;
}

// keo_regularized::rebuild (src/keo_regularized.cpp:233-258): + g cv t
// [[2|x|^2 + gamma, beta], [beta, 2|x|^2 - gamma]] when g > 0.
__global__ void reg_diag_kernel(int64_t N, const double *__restrict__ kdiag,
                                const double *__restrict__ cvt, double g,
                                const C2<double> *__restrict__ x, double *d64, float *d32) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= N) return;
  double a = kdiag[k], b = kdiag[k], c = 0.0;
  if (g > 0.0) {
    const C2<double> p = x[k];
    const double w = g * cvt[k];
    const double al = w * 2.0 * (p.x * p.x + p.y * p.y);
    const double be = w * (2.0 * p.x * p.y);
    const double ga = w * (p.x * p.x - p.y * p.y);
    a += al + ga;
    b += al - ga;
    c = be;
  }
  d64[3 * k] = a;
  d64[3 * k + 1] = b;
  d64[3 * k + 2] = c;
  d32[3 * k] = (float)a;
  d32[3 * k + 1] = (float)b;
  d32[3 * k + 2] = (float)c;
}

// Both FP32 diagonal blocks (Jacobian and regularised KEO) in one pass, for
// the mixed-precision Newton step's operators: the arithmetic of the two
// kernels above (so the FP32 blocks are bitwise theirs), the FP64 blocks not
// written.  (The same formulas in FP32 arithmetic saved a few more
// microseconds but moved the Krylov counts of the 64^3 continuation.)
__global__ void jac_reg_diag32_kernel(int64_t N, const double *__restrict__ kdiag, const double *__restrict__ cvt,
                                      const double *__restrict__ V, double g, const C2<double> *__restrict__ x,
                                      float *jd32, float *rd32) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= N) return;
  const C2<double> p = x[k];
  const double w = cvt[k], kd = kdiag[k];
  {
    const double al = w * (V[k] + g * 2.0 * (p.x * p.x + p.y * p.y));
    const double rx2 = g * w * (p.x * p.x - p.y * p.y);
    jd32[3 * k] = (float)(kd + al + rx2);
    jd32[3 * k + 1] = (float)(kd + al - rx2);
    jd32[3 * k + 2] = (float)(g * w * (2.0 * p.x * p.y));
  }
  double a = kd, b = kd, c = 0.0;
  if (g > 0.0) {
    const double wg = g * w;
    const double al = wg * 2.0 * (p.x * p.x + p.y * p.y);
    const double be = wg * (2.0 * p.x * p.y);
    const double ga = wg * (p.x * p.x - p.y * p.y);
    a += al + ga;
    b += al - ga;
    c = be;
  }
  rd32[3 * k] = (float)a;
  rd32[3 * k + 1] = (float)b;
  rd32[3 * k + 2] = (float)c;
}

// dF/dp diagonal terms (src/model_evaluator_nls.cpp:665-691): out +=
// cv t |x|^2 x for "g", cv t dV/dp x otherwise (dV/dp = 0 for the explicit
// potential used here).
__global__ void dfdp_diag_kernel(int64_t N, const double *__restrict__ cvt, int is_g,
                                 const C2<double> *__restrict__ x, C2<double> *out) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= N) return;
  if (!is_g) return;
  const C2<double> p = x[k];
  const double a = cvt[k] * (p.x * p.x + p.y * p.y);
  out[k].x += a * p.x;
  out[k].y += a * p.y;
}

// -sum cv |psi|^4 (gibbs_energy) and sum cv <phi, psi> (inner_product)
__global__ void energy_kernel(int64_t N, const double *__restrict__ cv,
                              const C2<double> *__restrict__ psi, double *partials,
                              unsigned *counter, double *out) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double v = 0.0;
  if (k < N) {
    const C2<double> p = psi[k];
    const double a = p.x * p.x + p.y * p.y;
    v = -cv[k] * a * a;
  }
  grid_reduce(v, partials, counter, out);
}

__global__ void inner_kernel(int64_t N, const double *__restrict__ cv,
                             const C2<double> *__restrict__ a, const C2<double> *__restrict__ b,
                             double *partials, unsigned *counter, double *out) {
  const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double v = 0.0;
  if (k < N) v = cv[k] * (a[k].x * b[k].x + a[k].y * b[k].y);
  grid_reduce(v, partials, counter, out);
}


__global__ void d2f_kernel(const double *__restrict__ a, float *__restrict__ b, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}
__global__ void f2d_kernel(const float *__restrict__ a, double *__restrict__ b, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) b[i] = (double)a[i];
}

// full-graph values: off-diagonal + diagonal, in complex_graph order
__global__ void export_kernel(int64_t N, const int32_t *__restrict__ rp,
                              const int32_t *__restrict__ ci, const C2<double> *__restrict__ od,
                              const double *__restrict__ diag, C2<double> *out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= N) return;
  int64_t o = rp[i] + i;
  bool placed = false;
  for (int k = rp[i]; k < rp[i + 1]; k++) {
    if (!placed && ci[k] > i) {
      out[o++] = C2<double>{diag ? diag[i] : 0.0, 0.0};
      placed = true;
    }
    out[o++] = od[k];
  }
  if (!placed) out[o] = C2<double>{diag ? diag[i] : 0.0, 0.0};
}

template <typename T>
int staging_cap(const MeshImpl &m) {
  // largest staged range of any row block, capped by the shared memory
  int64_t mx = 0;
  for (int64_t r0 = 0; r0 < m.N; r0 += kRows) {
    const int64_t r1 = std::min<int64_t>(m.N, r0 + kRows);
    mx = std::max<int64_t>(mx, m.rp[r1] - (m.rp[r0] & ~(int64_t)3));
  }
  mx = (mx + 3) & ~(int64_t)3;
  return (int)std::min<int64_t>(mx, stage_limit<T>());
}

template <typename T, class Op>
void launch_rows(const NlsImpl &s, const C2<T> *val, const C2<T> *x, const Op &op, int cap,
                 double *red_out) {
  launch_spmv<T, Op>(sizeof(T) == 4 ? s.warp32 : s.warp64, (int)s.N, s.mesh->d_rp.p, s.mesh->d_ci.p, val, x, cap,
                     op, s.red.partials.p, s.red.counter.p, red_out, s.stream);
  ++s.launch_count;
}

}  // namespace

__global__ void normalize_phases(int n, double *c) {
  const int k = threadIdx.x;
  if (k >= n) return;
  const double re = c[2 * k], im = c[2 * k + 1];
  const double m = sqrt(re * re + im * im);
  c[2 * k] = m > 0 ? re / m : 1.0;
  c[2 * k + 1] = m > 0 ? im / m : 0.0;
}

__global__ void history_dots(int64_t n, const double *x0, const double *x1, const double *x2, const double *x3,
                             const double *x4, int count, double *partials, unsigned *counter, double *out) {
  const C2<double> *xs[4] = {(const C2<double> *)x1, (const C2<double> *)x2, (const C2<double> *)x3,
                             (const C2<double> *)x4};
  const C2<double> *a0 = (const C2<double> *)x0;
  double re[4] = {0, 0, 0, 0}, im[4] = {0, 0, 0, 0};
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  // two elements per pass, all their loads issued before the first product
  for (; i + stride < n; i += 2 * stride) {
    const C2<double> y0 = a0[i], y1 = a0[i + stride];
    C2<double> u[4], v[4];
#pragma unroll
    for (int k = 0; k < 4; k++)
      if (k < count) {
        u[k] = xs[k][i];
        v[k] = xs[k][i + stride];
      }
#pragma unroll
    for (int k = 0; k < 4; k++) {
      if (k < count) {
        re[k] += u[k].x * y0.x + u[k].y * y0.y;
        im[k] += u[k].x * y0.y - u[k].y * y0.x;
        re[k] += v[k].x * y1.x + v[k].y * y1.y;
        im[k] += v[k].x * y1.y - v[k].y * y1.x;
      }
    }
  }
  for (; i < n; i += stride) {
    const C2<double> y = a0[i];
#pragma unroll
    for (int k = 0; k < 4; k++) {
      if (k < count) {
        const C2<double> x = xs[k][i];
        re[k] += x.x * y.x + x.y * y.y;
        im[k] += x.x * y.y - x.y * y.x;
      }
    }
  }
  const double v[8] = {re[0], im[0], re[1], im[1], re[2], im[2], re[3], im[3]};
  dev::grid_reduce_n<8>(v, 2 * count, partials, counter, out);
}

namespace dev {
template <typename T>
bool pick_warp_schedule(int N, const int32_t *rp, const int32_t *ci, const C2<T> *val, int cap, double *partials,
                        unsigned *counter, cudaStream_t st) {
  if (N <= 0) return false;
  DevBuf<C2<T>> xb, yb;
  DevBuf<T> db;
  DevBuf<double> rb;
  xb.alloc(N);
  yb.alloc(N);
  db.alloc(3 * (int64_t)N);
  rb.alloc(1);
  xb.zero(st);
  db.zero(st);
  // a representative epilogue: the diagonal block and a grid reduction, as
  // the Jacobian and the last smoothing step have
  BlockDiagOp<T, true> op{db.p, xb.p, yb.p};
  cudaEvent_t e0, e1;
  NOSH_CUDA(cudaEventCreate(&e0));
  NOSH_CUDA(cudaEventCreate(&e1));
  // best of three rounds of 5 launches each, alternating the schedules; the
  // warp schedule must win by 10 % (the staged one is the default)
  float best[2] = {1e30f, 1e30f};
  for (int round = 0; round < 3; round++)
    for (int w = 0; w < 2; w++) {
      for (int r = 0; r < 2; r++) launch_spmv<T>(w == 1, N, rp, ci, val, xb.p, cap, op, partials, counter, rb.p, st);
      NOSH_CUDA(cudaEventRecord(e0, st));
      for (int r = 0; r < 5; r++) launch_spmv<T>(w == 1, N, rp, ci, val, xb.p, cap, op, partials, counter, rb.p, st);
      NOSH_CUDA(cudaEventRecord(e1, st));
      NOSH_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      NOSH_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      best[w] = std::min(best[w], ms);
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return best[1] < 0.9f * best[0];
}
template bool pick_warp_schedule<float>(int, const int32_t *, const int32_t *, const C2<float> *, int, double *,
                                        unsigned *, cudaStream_t);
template bool pick_warp_schedule<double>(int, const int32_t *, const int32_t *, const C2<double> *, int, double *,
                                         unsigned *, cudaStream_t);

int warp_grid(const void *kernel, int64_t n_rows) {
  static int sms = 0;
  if (sms == 0) {
    int d = 0;
    NOSH_CUDA(cudaGetDevice(&d));
    NOSH_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, d));
  }
  int per_sm = 0;
  NOSH_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kWarpThreads, 0));
  const int64_t blocks = (n_rows + kWarpThreads - 1) / kWarpThreads;
  const int64_t cap = (int64_t)std::max(per_sm, 1) * sms;
  return (int)std::max<int64_t>(1, std::min(blocks, cap));
}

int row_grid(const void *kernel, int threads, size_t smem, int64_t n_rows) {
  static int sms = 0;
  if (sms == 0) {
    int d = 0;
    NOSH_CUDA(cudaGetDevice(&d));
    NOSH_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, d));
  }
  int per_sm = 0;
  NOSH_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem));
  const int64_t blocks = (n_rows + kRows - 1) / kRows;
  const int64_t cap = (int64_t)std::max(per_sm, 1) * sms;
  return (int)std::max<int64_t>(1, std::min(blocks, cap));
}
}  // namespace dev

// F(a) and F(b) (FP64, compute_f_) in one pass over the KEO graph, their
// squared norms into out[0], out[1]: thread per row, the nonzeros read once
// for both states, gathers in batches of four.  Per row the same summation
// order as the row-block kernel's ResidualOp.  sa / sb (optional): the
// off-diagonal sums of K a and K b.
__global__ void __launch_bounds__(128) residual_pair_kernel(
    int N, const int32_t *__restrict__ rp, const int32_t *__restrict__ ci, const C2<double> *__restrict__ val,
    const double *__restrict__ kdiag, const double *__restrict__ cvt, const double *__restrict__ V, double g,
    const C2<double> *__restrict__ xa, const C2<double> *__restrict__ xb, C2<double> *__restrict__ fa,
    C2<double> *__restrict__ fb, C2<double> *__restrict__ sa, C2<double> *__restrict__ sb, double *partials,
    unsigned *counter, double *out) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  double na = 0.0, nb = 0.0;
  if (row < N) {
    double ar = 0.0, ai = 0.0, br = 0.0, bi = 0.0;
    const int b = __ldg(rp + row), e = __ldg(rp + row + 1);
    for (int k0 = b; k0 < e; k0 += 4) {
      C2<double> v[4], p[4], q[4];
#pragma unroll
      for (int u = 0; u < 4; u++) {
        if (k0 + u < e) {
          const int c = __ldg(ci + k0 + u);
          v[u] = ldg(val + k0 + u);
          p[u] = ldg(xa + c);
          q[u] = ldg(xb + c);
        }
      }
#pragma unroll
      for (int u = 0; u < 4; u++) {
        if (k0 + u < e) {
          ar += v[u].x * p[u].x - v[u].y * p[u].y;
          ai += v[u].x * p[u].y + v[u].y * p[u].x;
          br += v[u].x * q[u].x - v[u].y * q[u].y;
          bi += v[u].x * q[u].y + v[u].y * q[u].x;
        }
      }
    }
    if (sa) sa[row] = C2<double>{ar, ai};
    if (sb) sb[row] = C2<double>{br, bi};
    const double kd = kdiag[row], ct = cvt[row], vv = V[row];
    const C2<double> pa = xa[row], pb = xb[row];
    const double ca = kd + ct * (vv + g * (pa.x * pa.x + pa.y * pa.y));
    const double cb = kd + ct * (vv + g * (pb.x * pb.x + pb.y * pb.y));
    const double far = ar + ca * pa.x, fai = ai + ca * pa.y, fbr = br + cb * pb.x, fbi = bi + cb * pb.y;
    fa[row] = C2<double>{far, fai};
    fb[row] = C2<double>{fbr, fbi};
    na = far * far + fai * fai;
    nb = fbr * fbr + fbi * fbi;
  }
  const double v[2] = {na, nb};
  grid_reduce_n<2>(v, 2, partials, counter, out);
}

// Device-side validation of an off-diagonal CSR graph (index-check mode):
// every row's range must be non-decreasing within [0, nnz], every column id
// in [0, N), different from the row and increasing along the row.  The
// first offending position is recorded as (kind << 56 | position) with an
// atomicMin, so the report is the same on every run; nothing is trapped and
// no out-of-range entry is dereferenced.
__global__ void graph_check_kernel(int64_t N, int64_t nnz, const int32_t *__restrict__ rp,
                                   const int32_t *__restrict__ ci, unsigned long long *err) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = rp[i], e = rp[i + 1];
    if (i == 0 && b != 0) atomicMin(err, (1ull << 56) | 0ull);
    if (i == N - 1 && e != nnz) atomicMin(err, (1ull << 56) | (unsigned long long)N);
    if (b > e || b < 0 || e > nnz) {
      atomicMin(err, (1ull << 56) | (unsigned long long)i);
      continue;
    }
    int64_t prev = -1;
    for (int64_t k = b; k < e; k++) {
      const int64_t c = ci[k];
      if (c < 0 || c >= N || c == i || c <= prev) {
        atomicMin(err, (2ull << 56) | (unsigned long long)k);
        break;
      }
      prev = c;
    }
  }
}

void check_graph(int64_t N, int64_t nnz, const int32_t *rp, const int32_t *ci, unsigned long long *err_dev,
                 cudaStream_t st) {
  NOSH_CUDA(cudaMemsetAsync(err_dev, 0xff, sizeof(unsigned long long), st));
  graph_check_kernel<<<(int)std::max<int64_t>(1, std::min<int64_t>(div_up(N, 256), 8 * kNumSMs)), 256, 0, st>>>(
      N, nnz, rp, ci, err_dev);
  NOSH_CUDA(cudaGetLastError());
}

void report_graph_error(unsigned long long w) {
  if (w == ~0ull) return;
  const unsigned long long kind = w >> 56, pos = w & ((1ull << 56) - 1);
  if (kind == 1)
    throw Error(NOSH_ERR_INVALID, "index check: row pointer out of order or out of range at row " +
                                      std::to_string(pos));
  throw Error(NOSH_ERR_INVALID, "index check: column id out of range, on the diagonal or not increasing at "
                                "entry " + std::to_string(pos));
}

// Achievable-bandwidth probe: a streaming read of n16 16-byte words
// (L2-allocating loads, one in flight per thread per iteration, eight
// 256-thread CTAs per SM) XOR-folded per CTA, one atomic per CTA: per-warp
// atomics on the single result word serialised at the L2 and cost ~10 us
// per launch.
__global__ void __launch_bounds__(256) stream_read_kernel(int64_t n16, const uint4 *__restrict__ a,
                                                          unsigned *out) {
  __shared__ unsigned s_acc[8];
  unsigned acc = 0u;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n16; i += stride) {
    const uint4 v = __ldcg(a + i);
    acc ^= v.x ^ v.y ^ v.z ^ v.w;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc ^= __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) s_acc[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned t = 0u;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t ^= s_acc[w];
    atomicXor(out, t);
  }
}

void stream_read(const void *buf, int64_t bytes, unsigned *out, cudaStream_t st) {
  stream_read_kernel<<<8 * kNumSMs, 256, 0, st>>>(bytes / 16, reinterpret_cast<const uint4 *>(buf), out);
  NOSH_CUDA(cudaGetLastError());
}

void launch_f64_to_f32(const double *a, float *b, int64_t n, cudaStream_t s) {
  if (n) d2f_kernel<<<div_up(n, 256), 256, 0, s>>>(a, b, n);
}
void launch_f32_to_f64(const float *a, double *b, int64_t n, cudaStream_t s) {
  if (n) f2d_kernel<<<div_up(n, 256), 256, 0, s>>>(a, b, n);
}

// ------------------------------------------------------------------------
NlsImpl::NlsImpl(MeshImpl *m, const double *mvp, double mu, const double *V, double g,
                 const double *t, const char *deriv)
    : mesh(m), N(m->N), E(m->E), deriv_param(deriv ? deriv : "mu"), g0(g), mu0(mu) {
  NOSH_CHECK(deriv_param == "mu" || deriv_param == "g", NOSH_ERR_INVALID,
             "deriv_parameter must be \"mu\" or \"g\"");
  // the solver's stream at the highest priority: work overlapped with it
  // on other streams (the learned predictor's inference) yields SM slots to
  // it as they free up
  {
    int lo = 0, hi = 0;
    NOSH_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    NOSH_CUDA(cudaStreamCreateWithPriority(&stream, cudaStreamNonBlocking, hi));
  }
  cudaStream_t s = stream;
  // aggregation defaults by mesh kind (sweeps of the 64^3 tetrahedral
  // continuation and the batched triangular squares): tetrahedra aggregate
  // every connection, triangles only strong ones
  if (m->nvc == 3) {
    amg_theta = 0.05;
    amg_cheb_ratio = 30.0;
  }
  h_V.assign(V, V + N);
  h_t.assign(t, t + N);
  d_A.upload(mvp, 3 * N, s);
  d_V.upload(h_V, s);
  d_t.upload(h_t, s);
  d_p.alloc(E);
  d_alpha.alloc(E);
  d_kdiag.alloc(N);
  d_kdiagf.alloc(N);
  d_cvt.alloc(N);
  edge_fields_kernel<<<div_up(E, 256), 256, 0, s>>>(E, m->d_edges.p, m->d_x.p, d_A.p, m->d_len.p,
                                                     m->d_covol.p, d_t.p, d_p.p, d_alpha.p);
  ++launch_count;
  vertex_fields_kernel<<<div_up(N, 256), 256, 0, s>>>(N, m->d_rp.p, m->d_nz_edge.p, d_alpha.p,
                                                       m->d_cv.p, d_t.p, d_kdiag.p, d_kdiagf.p,
                                                       d_cvt.p);
  ++launch_count;
  NOSH_CUDA(cudaGetLastError());
  const size_t nz = 2 * E + kPad;
  d_keo64.alloc(nz);
  d_keo32.alloc(nz);
  d_dkeo64.alloc(nz);
  d_keo64.zero(s);
  d_keo32.zero(s);
  d_dkeo64.zero(s);
  d_jd64.alloc(3 * N);
  d_rd64.alloc(3 * N);
  d_jd32.alloc(3 * N);
  d_rd32.alloc(3 * N);
  d_jd64.zero(s);
  d_rd64.zero(s);
  d_jd32.zero(s);
  d_rd32.zero(s);
  d_in.alloc(2 * N);
  d_out.alloc(2 * N);
  d_tmp.alloc(2 * N);
  d_inf.alloc(2 * N);
  d_outf.alloc(2 * N);
  red.init(div_up(N, kRows) + div_up(N, 256) + 1024, 64, s);
  NOSH_CUDA(cudaMallocHost(&h_stage_err, sizeof(unsigned)));
  *h_stage_err = 0u;
  cap32 = staging_cap<float>(*m);
  cap64 = staging_cap<double>(*m);
  tune_schedules();
  for (double c : m->h_cv) cv_sum += c;
  sync();
}

void NlsImpl::set_systems(const int64_t *offsets, int64_t num, const double *mu) {
  NOSH_CHECK(num >= 1 && offsets[0] == 0 && offsets[num] == N, NOSH_ERR_INVALID,
             "system offsets must run from 0 to the number of vertices");
  for (int64_t q = 0; q < num; q++)
    NOSH_CHECK(offsets[q + 1] > offsets[q], NOSH_ERR_INVALID, "every system needs at least one vertex");
  // edge -> system, and no edge between two systems
  std::vector<int32_t> es(E);
  const std::vector<int32_t> &ed = mesh->edges;  // 2E, sorted pairs
  for (int64_t e = 0; e < E; e++) {
    const int64_t a = ed[2 * e], b = ed[2 * e + 1];
    const int64_t sa = std::upper_bound(offsets, offsets + num + 1, a) - offsets - 1;
    const int64_t sb = std::upper_bound(offsets, offsets + num + 1, b) - offsets - 1;
    NOSH_CHECK(sa == sb, NOSH_ERR_INVALID, "an edge joins two systems");
    es[e] = (int32_t)sa;
  }
  sys_off.assign(offsets, offsets + num + 1);
  d_sys_off.upload(sys_off, stream);
  d_esys.upload(es, stream);
  d_mu_sys.upload(mu, num, stream);
  d_sys_norm.alloc(num);
  h_sys_norm.assign(num, 0.0);
  keo_mu = std::nan("");
  dkeo_mu = std::nan("");
  sync();
}

namespace {
// ||F_s||^2 of each system: one CTA per system (its rows are contiguous)
__global__ void system_norms_kernel(const int64_t *__restrict__ off, const C2<double> *__restrict__ f,
                                    double *__restrict__ out) {
  __shared__ double s32[32];
  const int64_t r0 = off[blockIdx.x], r1 = off[blockIdx.x + 1];
  double a = 0.0;
  for (int64_t i = r0 + threadIdx.x; i < r1; i += blockDim.x) {
    const C2<double> v = f[i];
    a += v.x * v.x + v.y * v.y;
  }
  a = dev::block_sum(a, s32);
  if (threadIdx.x == 0) out[blockIdx.x] = sqrt(a);
}
__global__ void mask_systems_kernel(const int64_t *__restrict__ off, const double *__restrict__ nrm, double tol,
                                    C2<double> *__restrict__ f) {
  if (!(nrm[blockIdx.x] <= tol)) return;
  for (int64_t i = off[blockIdx.x] + threadIdx.x; i < off[blockIdx.x + 1]; i += blockDim.x)
    f[i] = C2<double>{0.0, 0.0};
}
}  // namespace

double NlsImpl::system_norms(const double *f) {
  const int64_t ns = nsys();
  system_norms_kernel<<<(unsigned)ns, 256, 0, stream>>>(d_sys_off.p, (const C2<double> *)f, d_sys_norm.p);
  ++launch_count;
  NOSH_CUDA(cudaGetLastError());
  d_sys_norm.download(h_sys_norm.data(), ns, stream);
  sync();
  double mx = 0.0;
  for (double v : h_sys_norm) mx = std::max(mx, v);
  return mx;
}

void NlsImpl::mask_converged(double *f, double tol) {
  mask_systems_kernel<<<(unsigned)nsys(), 256, 0, stream>>>(d_sys_off.p, d_sys_norm.p, tol, (C2<double> *)f);
  ++launch_count;
  NOSH_CUDA(cudaGetLastError());
}

void NlsImpl::tune_schedules() {
  sync();
  if (spmv_schedule == 1) {
    warp32 = warp64 = false;
  } else if (spmv_schedule == 2) {
    warp32 = warp64 = true;
  } else {
    warp32 = pick_warp_schedule<float>((int)N, mesh->d_rp.p, mesh->d_ci.p, d_keo32.p, cap32, red.partials.p,
                                       red.counter.p, stream);
    warp64 = pick_warp_schedule<double>((int)N, mesh->d_rp.p, mesh->d_ci.p, d_keo64.p, cap64, red.partials.p,
                                        red.counter.p, stream);
  }
}

NlsImpl::~NlsImpl() {
  solver_state.reset();
  amg.reset();
  if (stream) cudaStreamDestroy(stream);
  if (h_stage_err) cudaFreeHost(h_stage_err);
}

void NlsImpl::sync() {
  if (!h_stage_err || !red.counter.p) {
    NOSH_CUDA(cudaStreamSynchronize(stream));
    return;
  }
  NOSH_CUDA(cudaMemcpyAsync(h_stage_err, red.counter.p + kStageErrorSlot, sizeof(unsigned), cudaMemcpyDeviceToHost,
                            stream));
  NOSH_CUDA(cudaStreamSynchronize(stream));
  if (*h_stage_err) stage_failure();
}

void NlsImpl::stage_failure() {
  // the CTAs that left early never reached their grid reductions: reset the
  // arrival counters they left behind along with the flag (the wait-bound
  // override in kStageWaitSlot stays)
  NOSH_CUDA(cudaMemsetAsync(red.counter.p, 0, kStageWaitSlot * sizeof(unsigned), stream));
  NOSH_CUDA(cudaMemsetAsync(red.counter.p + kStageErrorSlot, 0, sizeof(unsigned), stream));
  NOSH_CUDA(cudaStreamSynchronize(stream));
  if (h_stage_err) *h_stage_err = 0;
  throw Error(NOSH_ERR_CUDA,
              "an SpMV staging copy did not complete within its wait bound: the results of this call are "
              "invalid (the handle stays usable)");
}

void NlsImpl::check_indices() {
  if (d_check.n == 0) d_check.alloc(1);
  check_graph(N, 2 * E, mesh->d_rp.p, mesh->d_ci.p, d_check.p, stream);
  unsigned long long w = 0;
  d_check.download(&w, 1, stream);
  sync();
  report_graph_error(w);
}

void NlsImpl::set_stage_wait_limit(int64_t polls) {
  NOSH_CHECK(polls < (int64_t)0xffffffffLL, NOSH_ERR_INVALID, "stage wait limit out of range");
  const unsigned v = polls < 0 ? 0u : (unsigned)(polls + 1);
  NOSH_CUDA(cudaMemcpyAsync(red.counter.p + kStageWaitSlot, &v, sizeof(unsigned), cudaMemcpyHostToDevice, stream));
  NOSH_CUDA(cudaStreamSynchronize(stream));
}

void NlsImpl::keo_refill(double mu) {
  const double *ms = sys_off.empty() ? nullptr : d_mu_sys.p;
  keo_assemble<<<div_up(E, 256), 256, 0, stream>>>(E, d_alpha.p, d_p.p, mu, mesh->d_pos_fwd.p, mesh->d_pos_bwd.p,
                                                    d_keo64.p, d_keo32.p, ms, d_esys.p);
  ++launch_count;
  NOSH_CUDA(cudaGetLastError());
  keo_mu = mu;
}

void NlsImpl::dkeo_refill(double mu) {
  dkeo_assemble64<<<div_up(E, 256), 256, 0, stream>>>(
      E, d_alpha.p, d_p.p, mu, deriv_param == "mu" ? 1.0 : 0.0, mesh->d_pos_fwd.p,
      mesh->d_pos_bwd.p, d_dkeo64.p, sys_off.empty() ? nullptr : d_mu_sys.p, d_esys.p);
  ++launch_count;
  NOSH_CUDA(cudaGetLastError());
  dkeo_mu = mu;
}

void NlsImpl::keo_apply64(const double *x, double *y) {
  KeoOp<double> op{d_kdiag.p, (const C2<double> *)x, (C2<double> *)y};
  launch_rows<double>(*this, d_keo64.p, (const C2<double> *)x, op, cap64, nullptr);
}

void NlsImpl::dkeo_apply64(const double *x, double *y) {
  PlainOp<double> op{(C2<double> *)y};
  launch_rows<double>(*this, d_dkeo64.p, (const C2<double> *)x, op, cap64,
                      nullptr);
}

void NlsImpl::compute_f64(const double *x, double g, double mu, double *f, int norm_slot, double *soff) {
  if (!(keo_mu == mu)) keo_refill(mu);
  const int cap = cap64;
  if (norm_slot >= 0) {
    ResidualOp<true> op{d_kdiag.p, d_cvt.p, d_V.p, g, (const C2<double> *)x, (C2<double> *)f, (C2<double> *)soff};
    launch_rows<double>(*this, d_keo64.p, (const C2<double> *)x, op, cap, red.out.p + norm_slot);
  } else {
    ResidualOp<false> op{d_kdiag.p, d_cvt.p, d_V.p, g, (const C2<double> *)x, (C2<double> *)f,
                         (C2<double> *)soff};
    launch_rows<double>(*this, d_keo64.p, (const C2<double> *)x, op, cap, nullptr);
  }
}

void NlsImpl::residual_update(const double *x, const float *dx, double g, double mu, double *f, double *soff) {
  if (!(keo_mu == mu)) keo_refill(mu);
  ResidualUpdateOp op{d_kdiag.p, d_cvt.p, d_V.p, g, (const C2<double> *)x, (C2<double> *)f, (C2<double> *)soff};
  launch_rows<float>(*this, d_keo32.p, (const C2<float> *)dx, op, cap32, red.out.p);
}

namespace {
// max over rows of sum_k |v_k| (FP64 sums of the FP32 values' moduli),
// as the bits of a non-negative double (ordered like the values)
__global__ void abs_rowmax_kernel(int64_t n, const int32_t *__restrict__ rp, const C2<float> *__restrict__ val,
                                  unsigned long long *out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int32_t k = rp[i]; k < rp[i + 1]; k++) s += sqrt((double)val[k].x * val[k].x + (double)val[k].y * val[k].y);
  atomicMax(out, (unsigned long long)__double_as_longlong(s));
}
}  // namespace

double NlsImpl::keo_abs_rowmax() {
  if (abs_rowmax_ >= 0.0) return abs_rowmax_;
  if (!(keo_mu == keo_mu)) keo_refill(mu0);
  DevBuf<unsigned long long> w(1);
  w.zero(stream);
  abs_rowmax_kernel<<<div_up(N, 256), 256, 0, stream>>>(N, mesh->d_rp.p, d_keo32.p, w.p);
  ++launch_count;
  NOSH_CUDA(cudaGetLastError());
  unsigned long long h = 0;
  w.download(&h, 1, stream);
  sync();
  // the FP32 values' moduli: |alpha| to 2^-24
  double v = 0.0;
  std::memcpy(&v, &h, sizeof(v));
  abs_rowmax_ = v * (1.0 + std::ldexp(1.0, -22));
  return abs_rowmax_;
}

int NlsImpl::max_row_nnz() {
  if (max_row_nnz_ < 0) {
    int m = 0;
    for (int64_t i = 0; i < N; i++) m = std::max(m, (int)(mesh->rp[i + 1] - mesh->rp[i]));
    max_row_nnz_ = m;
  }
  return max_row_nnz_;
}

void NlsImpl::residual_pair(const double *xa, const double *xb, double g, double mu, double *fa, double *fb,
                            double norms[2], double *sa, double *sb, bool wait) {
  if (!(keo_mu == mu)) keo_refill(mu);
  residual_pair_kernel<<<div_up(N, 128), 128, 0, stream>>>(
      (int)N, mesh->d_rp.p, mesh->d_ci.p, d_keo64.p, d_kdiag.p, d_cvt.p, d_V.p, g, (const C2<double> *)xa,
      (const C2<double> *)xb, (C2<double> *)fa, (C2<double> *)fb, (C2<double> *)sa, (C2<double> *)sb,
      red.partials.p, red.counter.p, red.out.p);
  ++launch_count;
  NOSH_CUDA(cudaGetLastError());
  if (wait) residual_pair_norms(norms);
}

void NlsImpl::residual_pair_norms(double norms[2]) {
  red.out.download(norms, 2, stream);
  sync();
  norms[0] = std::sqrt(norms[0]);
  norms[1] = std::sqrt(norms[1]);
}

void NlsImpl::dfdp64(const double *x, double g, double mu, int param, double *out) {
  (void)g;
  if (!(dkeo_mu == mu)) dkeo_refill(mu);
  dkeo_apply64(x, out);
  dfdp_diag_kernel<<<div_up(N, 256), 256, 0, stream>>>(N, d_cvt.p, param == 0 ? 1 : 0,
                                                        (const C2<double> *)x, (C2<double> *)out);
  ++launch_count;
  NOSH_CUDA(cudaGetLastError());
}

void NlsImpl::jac_rebuild(const double *x, double g, double mu) {
  if (!(keo_mu == mu)) keo_refill(mu);
  jac_diag_kernel<<<div_up(N, 256), 256, 0, stream>>>(N, d_kdiag.p, d_cvt.p, d_V.p, g,
                                                       (const C2<double> *)x, d_jd64.p, d_jd32.p);
  ++launch_count;
  NOSH_CUDA(cudaGetLastError());
  jac_ready = true;
}

void NlsImpl::operators32_rebuild(const double *x, double g, double mu) {
  if (!(keo_mu == mu)) keo_refill(mu);
  jac_reg_diag32_kernel<<<div_up(N, 256), 256, 0, stream>>>(N, d_kdiag.p, d_cvt.p, d_V.p, g,
                                                             (const C2<double> *)x, d_jd32.p, d_rd32.p);
  ++launch_count;
  NOSH_CUDA(cudaGetLastError());
  // the FP64 blocks no longer belong to the same state: the operator entry
  // points want their own rebuild
  jac_ready = reg_ready = false;
}

void NlsImpl::reg_rebuild(const double *x, double g, double mu) {
  if (!(keo_mu == mu)) keo_refill(mu);
  reg_diag_kernel<<<div_up(N, 256), 256, 0, stream>>>(N, d_kdiag.p, d_cvt.p, g,
                                                       (const C2<double> *)x, d_rd64.p, d_rd32.p);
  ++launch_count;
  NOSH_CUDA(cudaGetLastError());
  reg_g = g;
  reg_ready = true;
}

template <>
void NlsImpl::jac_apply<double>(const double *x, double *y, double *dot_out) {
  const int cap = cap64;
  if (dot_out) {
    BlockDiagOp<double, true> op{d_jd64.p, (const C2<double> *)x, (C2<double> *)y};
    launch_rows<double>(*this, d_keo64.p, (const C2<double> *)x, op, cap, dot_out);
  } else {
    BlockDiagOp<double, false> op{d_jd64.p, (const C2<double> *)x, (C2<double> *)y};
    launch_rows<double>(*this, d_keo64.p, (const C2<double> *)x, op, cap, nullptr);
  }
}

template <>
void NlsImpl::jac_apply<float>(const float *x, float *y, double *dot_out) {
  const int cap = cap32;
  if (dot_out) {
    BlockDiagOp<float, true> op{d_jd32.p, (const C2<float> *)x, (C2<float> *)y};
    launch_rows<float>(*this, d_keo32.p, (const C2<float> *)x, op, cap, dot_out);
  } else {
    BlockDiagOp<float, false> op{d_jd32.p, (const C2<float> *)x, (C2<float> *)y};
    launch_rows<float>(*this, d_keo32.p, (const C2<float> *)x, op, cap, nullptr);
  }
}

template <>
void NlsImpl::reg_apply<double>(const double *x, double *y) {
  BlockDiagOp<double, false> op{d_rd64.p, (const C2<double> *)x, (C2<double> *)y};
  launch_rows<double>(*this, d_keo64.p, (const C2<double> *)x, op, cap64,
                      nullptr);
}

template <>
void NlsImpl::reg_apply<float>(const float *x, float *y) {
  BlockDiagOp<float, false> op{d_rd32.p, (const C2<float> *)x, (C2<float> *)y};
  launch_rows<float>(*this, d_keo32.p, (const C2<float> *)x, op, cap32,
                     nullptr);
}

double NlsImpl::energy(const double *psi) {
  energy_kernel<<<div_up(N, 256), 256, 0, stream>>>(N, mesh->d_cv.p, (const C2<double> *)psi,
                                                     red.partials.p, red.counter.p, red.out.p);
  ++launch_count;
  NOSH_CUDA(cudaGetLastError());
  double e = 0.0;
  red.out.download(&e, 1, stream);
  sync();
  return e / cv_sum;
}

double NlsImpl::inner_product(const double *phi, const double *psi) {
  inner_kernel<<<div_up(N, 256), 256, 0, stream>>>(N, mesh->d_cv.p, (const C2<double> *)phi,
                                                    (const C2<double> *)psi, red.partials.p,
                                                    red.counter.p, red.out.p);
  ++launch_count;
  NOSH_CUDA(cudaGetLastError());
  double e = 0.0;
  red.out.download(&e, 1, stream);
  sync();
  return e / cv_sum;
}

void NlsImpl::export_values(const C2<double> *offdiag, const double *diag, double *out) {
  export_kernel<<<div_up(N, 256), 256, 0, stream>>>(N, mesh->d_rp.p, mesh->d_ci.p, offdiag, diag,
                                                     (C2<double> *)out);
  ++launch_count;
  NOSH_CUDA(cudaGetLastError());
}

}  // namespace nosh
