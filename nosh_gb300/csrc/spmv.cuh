// Row-block SpMV over the off-diagonal KEO graph with a fused per-vertex
// epilogue (diagonal 2x2 block, residual nonlinearity, reductions).
//
// One CTA = kRows consecutive rows = kRows threads.  The CTA's nonzeros
// [rp[r0], rp[r1]) are contiguous; they are staged into shared memory with
// 128-bit coalesced loads (int4 for column ids, 16-byte chunks of the complex
// values), then every thread reduces its own row out of shared memory and
// gathers x through the read-only path.  A CTA whose nonzeros exceed the
// staging capacity reads them directly.
#pragma once

#include "common.cuh"

namespace nosh {
namespace dev {

constexpr int kRows = 128;

template <typename T>
struct Acc;  // accumulator type per value type
template <> struct Acc<float> { using type = float; };
template <> struct Acc<double> { using type = double; };

// Grid-wide deterministic sum of one double per thread: block partials, then
// the last CTA to arrive adds them in fixed order and stores *out.
__device__ __forceinline__ void grid_reduce(double v, double *partials,
                                            unsigned *counter, double *out) {
  __shared__ double s32[32];
  __shared__ bool last;
  const double b = block_sum(v, s32);
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = b;
    __threadfence();
    const unsigned t = atomicAdd(counter, 1u);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (last) {
    __threadfence();
    double s = 0.0;
    for (unsigned j = threadIdx.x; j < gridDim.x; j += blockDim.x) s += __ldcg(partials + j);
    s = block_sum(s, s32);
    if (threadIdx.x == 0) {
      *out = s;
      *counter = 0u;
    }
  }
}

// Op must provide:
//   static constexpr bool kReduce;
//   __device__ double finish(int row, C2<acc> sum) -- writes y[row], returns
//                                                     the thread's partial
template <typename T, class Op>
__global__ void __launch_bounds__(kRows)
    row_block_apply(int N, const int32_t *__restrict__ rp, const int32_t *__restrict__ ci,
                    const C2<T> *__restrict__ val, const C2<T> *__restrict__ x, int cap,
                    Op op, double *partials, unsigned *counter, double *red_out) {
  using A = typename Acc<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int r0 = blockIdx.x * kRows;
  const int r1 = min(N, r0 + kRows);
  const int k0 = __ldg(rp + r0), k1 = __ldg(rp + r1);
  const int ks = k0 & ~3;  // 16-byte aligned start for both arrays
  const int n = k1 - ks;
  const bool staged = n <= cap;
  int32_t *s_col = reinterpret_cast<int32_t *>(smem_raw);
  C2<T> *s_val = reinterpret_cast<C2<T> *>(smem_raw + (size_t)cap * sizeof(int32_t));
  if (staged) {
    const int n4 = (n + 3) >> 2;
    const int4 *c4 = reinterpret_cast<const int4 *>(ci + ks);
    for (int j = threadIdx.x; j < n4; j += kRows) reinterpret_cast<int4 *>(s_col)[j] = __ldg(c4 + j);
    const int nv = (int)((n * sizeof(C2<T>) + 15) / 16);
    const uint4 *v4 = reinterpret_cast<const uint4 *>(val + ks);
    for (int j = threadIdx.x; j < nv; j += kRows) reinterpret_cast<uint4 *>(s_val)[j] = __ldg(v4 + j);
  }
  __syncthreads();
  const int row = r0 + threadIdx.x;
  double part = 0.0;
  if (row < N) {
    A sr = 0, si = 0;
    const int b = __ldg(rp + row), e = __ldg(rp + row + 1);
    if (staged) {
      for (int k = b - ks; k < e - ks; k++) {
        const C2<T> v = s_val[k];
        const C2<T> xv = ldg(x + s_col[k]);
        sr += v.x * xv.x - v.y * xv.y;
        si += v.x * xv.y + v.y * xv.x;
      }
    } else {
      for (int k = b; k < e; k++) {
        const C2<T> v = ldg(val + k);
        const C2<T> xv = ldg(x + __ldg(ci + k));
        sr += v.x * xv.x - v.y * xv.y;
        si += v.x * xv.y + v.y * xv.x;
      }
    }
    part = op.finish(row, sr, si);
  }
  if (Op::kReduce) grid_reduce(part, partials, counter, red_out);
}

// ---- epilogues --------------------------------------------------------
// y = K x : diagonal K_ii = sum of incident alpha (real)
template <typename T>
struct KeoOp {
  static constexpr bool kReduce = false;
  const T *kdiag;
  const C2<T> *x;
  C2<T> *y;
  __device__ double finish(int i, T sr, T si) const {
    const C2<T> xi = x[i];
    const T d = kdiag[i];
    y[i] = C2<T>{sr + d * xi.x, si + d * xi.y};
    return 0.0;
  }
};

// y = sum (no diagonal): dK/dp
template <typename T>
struct PlainOp {
  static constexpr bool kReduce = false;
  C2<T> *y;
  __device__ double finish(int i, T sr, T si) const {
    y[i] = C2<T>{sr, si};
    return 0.0;
  }
};

// y = K_offdiag x + [[d0r, d1b], [d1b, d0i]] x_i (Jacobian or regularised
// KEO; the diagonal blocks include K_ii); optionally sum_i <x_i, y_i>.
template <typename T, bool kDot>
struct BlockDiagOp {
  static constexpr bool kReduce = kDot;
  const T *d;  // 3 per vertex
  const C2<T> *x;
  C2<T> *y;
  __device__ double finish(int i, T sr, T si) const {
    const C2<T> xi = x[i];
    const T d0r = d[3 * i], d0i = d[3 * i + 1], d1b = d[3 * i + 2];
    const T yr = sr + d0r * xi.x + d1b * xi.y;
    const T yi = si + d1b * xi.x + d0i * xi.y;
    y[i] = C2<T>{yr, yi};
    return kDot ? (double)xi.x * (double)yr + (double)xi.y * (double)yi : 0.0;
  }
};

// F = K psi + cv t (V + g|psi|^2) psi (FP64), optionally ||F||^2
template <bool kNorm>
struct ResidualOp {
  static constexpr bool kReduce = kNorm;
  const double *kdiag, *cvt, *V;
  double g;
  const C2<double> *x;
  C2<double> *y;
  __device__ double finish(int i, double sr, double si) const {
    const C2<double> p = x[i];
    const double a = kdiag[i] + cvt[i] * (V[i] + g * (p.x * p.x + p.y * p.y));
    const double fr = sr + a * p.x, fi = si + a * p.y;
    y[i] = C2<double>{fr, fi};
    return kNorm ? fr * fr + fi * fi : 0.0;
  }
};

}  // namespace dev
}  // namespace nosh
