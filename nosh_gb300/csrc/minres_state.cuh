// MINRES recurrence state (device memory) and its device-side update.
#pragma once

#include "common.cuh"

namespace nosh {

struct MinresScalars {
  double beta1, beta, oldb, alfa, dbar, epsln, oldeps, phibar, phi, cs, sn, gamma, delta;
  double zu, rz;  // reduction results: <z, J z>, <r, M r>
  double rtol;
  int itn, maxit;
  int done;        // 0 running, 1 converged in the last update, 2 frozen
  int flag;        // NOSH_OK / NOSH_ERR_NOT_CONVERGED / _NAN / _BREAKDOWN
  int wx_pending;  // the w/x update of the last Lanczos step is still due
  // per-element coefficients, computed once per step by the single thread
  // that owns the recurrence (FP64 division is slow on GB300: element
  // kernels only load these):
  //   lanczos: r_new = la[0] u - la[1] r_old - la[2] r_cur
  //   w/x:     w = (z wx[0] - wx[1] w2 - wx[2] w) wx[3];  x += wx[4] w
  double la64[3], wx64[5];
  float la32[3], wx32[5];
};

template <typename T>
__device__ __forceinline__ const T *lanczos_coef(const MinresScalars *s);
template <>
__device__ __forceinline__ const float *lanczos_coef<float>(const MinresScalars *s) {
  return s->la32;
}
template <>
__device__ __forceinline__ const double *lanczos_coef<double>(const MinresScalars *s) {
  return s->la64;
}
template <typename T>
__device__ __forceinline__ const T *wx_coef(const MinresScalars *s);
template <>
__device__ __forceinline__ const float *wx_coef<float>(const MinresScalars *s) {
  return s->wx32;
}
template <>
__device__ __forceinline__ const double *wx_coef<double>(const MinresScalars *s) {
  return s->wx64;
}

// Lanczos coefficients once <z, J z> (zu) is known.  Single thread.  After
// convergence (done == 1) the launch has applied the last deferred w/x
// update, and the recurrence is frozen (done = 2): the remaining launches of
// the chunk return at once.  The state is read into registers in one go and
// written back once: field by field, its dependent global loads and stores
// were the longest chain of the launch's tail.
__device__ __forceinline__ void minres_lanczos_coefs(MinresScalars *sp, double zu) {
  MinresScalars s = *sp;
  if (s.done) {
    sp->done = 2;
    sp->wx_pending = 0;
    return;
  }
  s.zu = zu;
  const double beta = s.beta, alfa = zu / (beta * beta);
  const double c[3] = {1.0 / beta, s.itn > 0 ? beta / s.oldb : 0.0, alfa / beta};
  for (int k = 0; k < 3; k++) {
    s.la64[k] = c[k];
    s.la32[k] = (float)c[k];
  }
  *sp = s;
}

// One step of the Paige-Saunders Givens recurrence after <r_new, M r_new>
// (rz) is known; scipy / Paige-Saunders variable names.  Single thread; the
// state in registers as above.
__device__ __forceinline__ void minres_advance(MinresScalars *sp, double rz) {
  MinresScalars s = *sp;
  s.rz = rz;
  if (s.done) {
    s.done = 2;
    s.wx_pending = 0;
    *sp = s;
    return;
  }
  const double beta = s.beta;
  const double alfa = s.zu / (beta * beta);
  s.alfa = alfa;
  s.oldb = beta;
  if (!(rz >= 0.0) || isinf(rz) || isnan(alfa)) {
    s.flag = (isnan(rz) || isinf(rz) || isnan(alfa)) ? NOSH_ERR_NAN : NOSH_ERR_BREAKDOWN;
    s.done = 2;
    s.wx_pending = 0;
    *sp = s;
    return;
  }
  const double nb = sqrt(rz);
  s.beta = nb;
  s.oldeps = s.epsln;
  const double delta = s.cs * s.dbar + s.sn * alfa;
  const double gbar = s.sn * s.dbar - s.cs * alfa;
  s.epsln = s.sn * nb;
  s.dbar = -s.cs * nb;
  double gamma = hypot(gbar, nb);
  if (gamma == 0.0) gamma = 2.2e-16;
  s.cs = gbar / gamma;
  s.sn = nb / gamma;
  s.phi = s.cs * s.phibar;
  s.phibar = s.sn * s.phibar;
  s.gamma = gamma;
  s.delta = delta;
  s.itn += 1;
  s.wx_pending = 1;
  const double w[5] = {1.0 / s.oldb, s.oldeps, delta, 1.0 / gamma, s.phi};
  for (int k = 0; k < 5; k++) {
    s.wx64[k] = w[k];
    s.wx32[k] = (float)w[k];
  }
  if (s.phibar <= s.rtol * s.beta1 || nb == 0.0) {
    s.done = 1;
  } else if (s.itn >= s.maxit) {
    s.done = 1;
    s.flag = NOSH_ERR_NOT_CONVERGED;
  }
  *sp = s;
}

// The deferred w/x update of one Lanczos step for element i:
// w_new = (z/oldb - oldeps w2 - delta w) / gamma (over the w1 buffer),
// x += phi w_new.
template <typename T>
__device__ __forceinline__ void minres_wx_elem(const T *c, int64_t i, const T *z, T *wa, const T *wb,
                                               const T *wc, T *x) {
  const T w = (z[i] * c[0] - c[1] * wb[i] - c[2] * wc[i]) * c[3];
  wa[i] = w;
  x[i] += c[4] * w;
}

}  // namespace nosh
