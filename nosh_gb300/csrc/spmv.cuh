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

#include <utility>

#include <type_traits>

#include "common.cuh"

namespace nosh {
namespace dev {

constexpr int kRows = 128;

template <typename T>
struct Acc;  // accumulator type per value type
template <> struct Acc<float> { using type = float; };
template <> struct Acc<double> { using type = double; };

// Grid-wide deterministic sum of one double per thread: block partials, then
// the last CTA to arrive adds them in fixed order and stores *out.  Returns
// true in exactly one thread (thread 0 of that last CTA), with the sum in
// *total, so callers can continue with scalar work on the result.
__device__ __forceinline__ bool grid_reduce(double v, double *partials, unsigned *counter,
                                            double *out, double *total = nullptr) {
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
  bool finisher = false;
  if (last) {
    __threadfence();
    // four independent accumulators so the partial loads overlap (fixed
    // order per thread: deterministic)
    const unsigned G = gridDim.x, st = blockDim.x;
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
    unsigned j = threadIdx.x;
    for (; j + 3 * st < G; j += 4 * st) {
      a0 += __ldcg(partials + j);
      a1 += __ldcg(partials + j + st);
      a2 += __ldcg(partials + j + 2 * st);
      a3 += __ldcg(partials + j + 3 * st);
    }
    for (; j < G; j += st) a0 += __ldcg(partials + j);
    double s = block_sum((a0 + a1) + (a2 + a3), s32);
    if (threadIdx.x == 0) {
      *out = s;
      *counter = 0u;
      if (total) *total = s;
      finisher = true;
    }
  }
  return finisher;
}

// Op must provide:
//   static constexpr bool kReduce;
//   __device__ double finish(int row, acc sr, acc si) -- writes y[row],
//                                                       returns the thread's
//                                                       partial
// and, when kReduce, may provide kHook + hook(total): scalar work done by one
// thread once the grid sum is known.
template <class Op, class = void>
struct HasHook {
  static constexpr bool value = false;
};
template <class Op>
struct HasHook<Op, decltype((void)Op::kHook, void())> {
  static constexpr bool value = Op::kHook;
};
template <class Op>
__device__ __forceinline__ typename std::enable_if<HasHook<Op>::value>::type run_hook(const Op &op,
                                                                                     double t) {
  op.hook(t);
}
template <class Op>
__device__ __forceinline__ typename std::enable_if<!HasHook<Op>::value>::type run_hook(const Op &,
                                                                                      double) {}
// An Op may also carry `const int *halt`: when it points at a value >= 2
// the whole launch returns at once (MINRES iterations of a captured chunk
// that follow convergence).
template <class Op, class = void>
struct HasHalt {
  static constexpr bool value = false;
};
template <class Op>
struct HasHalt<Op, decltype((void)std::declval<Op>().halt, void())> {
  static constexpr bool value = true;
};
template <class Op>
__device__ __forceinline__ bool halted(const Op &op) {
  if constexpr (HasHalt<Op>::value) {
    return op.halt != nullptr && *op.halt >= 2;
  } else {
    return false;
  }
}
template <typename T, class Op>
__global__ void __launch_bounds__(kRows)
    row_block_apply(int N, const int32_t *__restrict__ rp, const int32_t *__restrict__ ci,
                    const C2<T> *__restrict__ val, const C2<T> *__restrict__ x, int cap,
                    Op op, double *partials, unsigned *counter, double *red_out) {
  using A = typename Acc<T>::type;
  if (halted(op)) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  int32_t *s_col = reinterpret_cast<int32_t *>(smem_raw);
  C2<T> *s_val = reinterpret_cast<C2<T> *>(smem_raw + (size_t)cap * sizeof(int32_t));
  const int nblocks = (N + kRows - 1) / kRows;
  A part = 0;
  // persistent: the grid is sized to the resident capacity and each CTA
  // walks row blocks with a grid stride (whole waves, fewer partial sums)
  for (int rb = blockIdx.x; rb < nblocks; rb += gridDim.x) {
    const int r0 = rb * kRows;
    const int r1 = min(N, r0 + kRows);
    const int k0 = __ldg(rp + r0), k1 = __ldg(rp + r1);
    const int ks = k0 & ~3;  // 16-byte aligned start for both arrays
    const int n = k1 - ks;
    const bool staged = n <= cap;
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
      part += (A)op.finish(row, sr, si);
    }
    __syncthreads();  // the staging buffer is reused by the next row block
  }
  if (Op::kReduce) {
    double total = 0.0;
    if (grid_reduce((double)part, partials, counter, red_out, &total)) run_hook(op, total);
  }
}

// Grid for a persistent row kernel: the resident capacity of the device for
// this kernel and shared-memory size, capped by the number of row blocks.
int row_grid(const void *kernel, size_t smem, int64_t n_rows);

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
