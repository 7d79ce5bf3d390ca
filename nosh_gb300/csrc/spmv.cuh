// Row-block SpMV over the off-diagonal KEO graph with a fused per-vertex
// epilogue (diagonal 2x2 block, residual nonlinearity, reductions).
//
// One CTA = kRows consecutive rows (row_threads<T>() threads per row),
// persistent over row blocks.  A row block's nonzeros [rp[r0], rp[r1]) are
// contiguous: one thread stages them into shared memory with two bulk
// asynchronous copies (TMA, cp.async.bulk: column ids and complex values)
// completing on an mbarrier, double-buffered so that the copy of the CTA's
// next row block overlaps the current one's arithmetic.  The threads of a
// row then reduce its nonzeros out of shared memory and gather x through
// the read-only path.  A row block whose nonzeros exceed the staging
// capacity reads them directly.
#pragma once

#include <utility>

#include <type_traits>

#include "common.cuh"

namespace nosh {
namespace dev {

// Arrival at a grid reduction: counter += 1 with acquire-release semantics
// at GPU scope, returning the old value.  The release publishes the CTA's
// partial written before it; the acquire, in the CTA that arrives last,
// orders the partials read after it (behind the CTA barrier that follows)
// after every other CTA's write.  It takes the place of a full fence on
// either side of a relaxed atomic.
__device__ __forceinline__ unsigned arrive_acq_rel(unsigned *counter) {
  unsigned old;
  asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;\n" : "=r"(old) : "l"(counter) : "memory");
  return old;
}

constexpr int kRows = 128;
// Threads per row of the staged schedule (adjacent lanes, each taking every
// row_threads-th nonzero).  One: two lanes per FP32 row (twice the warps
// per SM for the gathers' latency, four CTAs per SM instead of five)
// measured 4 % slower on the 64^3 smoother launch and 9 % on the 160^3 one.
template <typename T>
__host__ __device__ constexpr int row_threads() {
  return 1;
}
template <typename T>
__host__ __device__ constexpr int block_threads() {
  return kRows * row_threads<T>();
}

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
    const unsigned t = arrive_acq_rel(counter);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  bool finisher = false;
  if (last) {
    dep_trigger();
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

// The same for m <= K values at once (v[0..m-1], partials in columns
// partials + k gridDim.x, one arrival counter): one pass of block sums and
// one arrival instead of m successive grid_reduce calls, each with its own
// barriers, fence and atomic.  The sums are bitwise those of m grid_reduce
// calls (the same block and final summation orders).  Writes out[0..m-1]
// in the last CTA; returns true in exactly one thread.
template <int K>
__device__ __forceinline__ bool grid_reduce_n(const double (&v)[K], int m, double *partials, unsigned *counter,
                                              double *out) {
  __shared__ double sw[32 * K];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  double r[K];
#pragma unroll
  for (int k = 0; k < K; k++) r[k] = k < m ? warp_sum(v[k]) : 0.0;
  __syncthreads();
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < K; k++)
      if (k < m) sw[w * K + k] = r[k];
  }
  __syncthreads();
  if (w == 0) {
#pragma unroll
    for (int k = 0; k < K; k++) {
      if (k < m) {
        double t = lane < nw ? sw[lane * K + k] : 0.0;
        t = warp_sum(t);
        if (lane == 0) partials[(size_t)k * gridDim.x + blockIdx.x] = t;
      }
    }
  }
  if (threadIdx.x == 0) {
    const unsigned t = arrive_acq_rel(counter);
    last = (t == gridDim.x - 1);
  }
  __syncthreads();
  bool finisher = false;
  if (last) {
    dep_trigger();
    const unsigned G = gridDim.x, st = blockDim.x;
    double acc[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
      acc[k] = 0.0;
      if (k < m) {
        const double *pk = partials + (size_t)k * G;
        double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
        unsigned j = threadIdx.x;
        for (; j + 3 * st < G; j += 4 * st) {
          a0 += __ldcg(pk + j);
          a1 += __ldcg(pk + j + st);
          a2 += __ldcg(pk + j + 2 * st);
          a3 += __ldcg(pk + j + 3 * st);
        }
        for (; j < G; j += st) a0 += __ldcg(pk + j);
        acc[k] = warp_sum((a0 + a1) + (a2 + a3));
      }
    }
    __syncthreads();
    if (lane == 0) {
#pragma unroll
      for (int k = 0; k < K; k++)
        if (k < m) sw[w * K + k] = acc[k];
    }
    __syncthreads();
    if (w == 0) {
#pragma unroll
      for (int k = 0; k < K; k++) {
        if (k < m) {
          double t = lane < nw ? sw[lane * K + k] : 0.0;
          t = warp_sum(t);
          if (lane == 0) out[k] = t;
        }
      }
    }
    if (threadIdx.x == 0) {
      *counter = 0u;
      finisher = true;
    }
  }
  return finisher;
}

// The type a launch accumulates the epilogues' partials in: the SpMV's
// accumulator type unless the Op asks for FP64 (`using Part = double`).
template <class Op, class A, class = void>
struct PartOf {
  using type = A;
};
template <class Op, class A>
struct PartOf<Op, A, decltype((void)sizeof(typename Op::Part), void())> {
  using type = typename Op::Part;
};

// Op must provide:
//   static constexpr bool kReduce;
//   struct Pre;                                  -- the row's epilogue operands
//   __device__ Pre load(int row)                 -- issued before the row's
//                                                   nonzeros arrive, so the
//                                                   epilogue loads overlap the
//                                                   staging and the gathers
//   __device__ double finish(int row, acc sr, acc si, const Pre &)
//                                                -- writes y[row], returns the
//                                                   thread's partial
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
// The same test before dep_sync(), read from L2: the flag only rises within
// a solve and is reset several launches before the solve's first iteration,
// so a true answer is final, while a false one may be stale (the kernel this
// launch follows may have raised it without its write being visible yet).
template <class Op>
__device__ __forceinline__ bool halted_early(const Op &op) {
  if constexpr (HasHalt<Op>::value) {
    return op.halt != nullptr && __ldcg(op.halt) >= 2;
  } else {
    return false;
  }
}
// ---- bulk-copy staging (TMA + mbarrier) ------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_addr(bar)));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}
// global -> shared bulk copy; dst, src 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
// Default bound of a staging wait, in polls of mbarrier.try_wait.
constexpr uint32_t kStageWaitPolls = 1u << 20;
// Bounded wait for the phase with the given parity; false after `limit`
// polls (at once for a limit of 0).
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, uint32_t limit = kStageWaitPolls) {
  const uint32_t a = smem_addr(bar);
  for (uint32_t it = 0; it < limit; it++) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Shared memory of one staging buffer (column ids, then complex values) for
// a capacity of cap nonzeros (a multiple of 4); the kernel uses two.
template <typename T>
__host__ __device__ constexpr size_t stage_bytes(int cap) {
  return (size_t)cap * (sizeof(int32_t) + sizeof(C2<T>));
}
// Largest staging capacity: two buffers within 96 KB.
template <typename T>
__host__ __device__ constexpr int stage_limit() {
  return (int)((48 * 1024) / (sizeof(int32_t) + sizeof(C2<T>))) & ~3;
}
// Slot of the per-stream reduction counters that records a staging copy
// that never completed (checked by the host at its next synchronisation).
constexpr int kStageErrorSlot = 15;
// Slot holding a diagnostic override of the staging-wait bound: 0 = the
// default kStageWaitPolls, v > 0 = v - 1 polls.  Read only by launches that
// stage (cap > 0).
constexpr int kStageWaitSlot = 14;

template <typename T, class Op>
__global__ void __launch_bounds__(block_threads<T>(), sizeof(T) == 4 ? 5 : 1)
    row_block_apply(int N, const int32_t *__restrict__ rp, const int32_t *__restrict__ ci,
                    const C2<T> *__restrict__ val, const C2<T> *__restrict__ x, int cap,
                    Op op, double *partials, unsigned *counter, double *red_out) {
  using A = typename Acc<T>::type;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bar[2];
  const size_t buf = stage_bytes<T>(cap);
  const int nblocks = (N + kRows - 1) / kRows;
  if (threadIdx.x == 0) {
    mbar_init(&bar[0]);
    mbar_init(&bar[1]);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
  }
  __syncthreads();
  // row block -> its aligned nonzero range; staged when it fits
  auto range = [&](int rb, int &ks, int &n) {
    const int r0 = rb * kRows, r1 = min(N, r0 + kRows);
    const int k0 = __ldg(rp + r0), k1 = __ldg(rp + r1);
    ks = k0 & ~3;  // 16-byte aligned start for both arrays
    n = k1 - ks;
  };
  auto issue = [&](int rb, int stage) {
    int ks, n;
    range(rb, ks, n);
    if (n > 0 && n <= cap) {
      unsigned char *base = smem_raw + stage * buf;
      const uint32_t cb = (uint32_t)(((n + 3) >> 2) * 16);                   // column ids
      const uint32_t vb = (uint32_t)(((size_t)n * sizeof(C2<T>) + 15) / 16 * 16);  // values
      mbar_expect_tx(&bar[stage], cb + vb);
      bulk_g2s(base, ci + ks, cb, &bar[stage]);
      bulk_g2s(base + (size_t)cap * sizeof(int32_t), val + ks, vb, &bar[stage]);
    }
  };
  // The first row block's copy is issued before dep_sync(): the matrix (row
  // pointers, column ids, values) is never written by the kernel that a
  // launch with overlap follows, so the copy is in flight while the launch
  // waits for that kernel's completion.
  // row blocks blockIdx.x, + gridDim.x, ... (strided: consecutive row blocks,
  // which share x gathers, run at the same time on different SMs; contiguous
  // chunks per CTA measured 5 % slower at 64^3)
  const int rb0 = blockIdx.x, rb_end = nblocks;
  auto nxt = [&](int rb) { return rb + (int)gridDim.x; };
  const bool skip = halted_early(op);
  if (!skip && threadIdx.x == 0 && rb0 < rb_end) issue(rb0, 0);
  dep_sync();
  if (halted(op)) {
    // let the copy issued above land before the CTA leaves
    if (!skip && threadIdx.x == 0 && rb0 < rb_end) {
      int ks, n;
      range(rb0, ks, n);
      if (n > 0 && n <= cap && !mbar_wait(&bar[0], 0u)) atomicOr(counter + kStageErrorSlot, 1u);
    }
    return;
  }
  typename PartOf<Op, A>::type part = 0;
  uint32_t parity[2] = {0u, 0u};
  bool ok = true;
  // copies issued and not yet waited for: the current and the next row block
  bool cur_staged = false, next_staged = false;
  uint32_t limit = kStageWaitPolls;
  if (cap > 0) {
    const unsigned o = __ldcg(counter + kStageWaitSlot);
    if (o != 0u) limit = o - 1u;
  }
  int stage = 0;
  for (int rb = rb0; rb < rb_end; rb = nxt(rb), stage ^= 1) {
    // the other buffer was released by the barrier that ended the previous
    // iteration: start the next row block's copy into it
    if (threadIdx.x == 0 && nxt(rb) < rb_end) issue(nxt(rb), stage ^ 1);
    int ks, n;
    range(rb, ks, n);
    constexpr int R = row_threads<T>();
    const int row = rb * kRows + (int)threadIdx.x / R, lane_r = (int)threadIdx.x % R;
    typename Op::Pre pre{};
    if (row < N && lane_r == 0) pre = op.load(row);
    const bool staged = n > 0 && n <= cap;
    cur_staged = staged;
    next_staged = false;
    if (nxt(rb) < rb_end) {
      int ks2, n2;
      range(nxt(rb), ks2, n2);
      next_staged = n2 > 0 && n2 <= cap;
    }
    const bool arrived = staged ? mbar_wait(&bar[stage], parity[stage], limit) : true;
    if (__syncthreads_or(!arrived)) {  // the CTA leaves together
      ok = false;
      break;
    }
    if (staged) parity[stage] ^= 1u;
    const int32_t *s_col = reinterpret_cast<const int32_t *>(smem_raw + stage * buf);
    const C2<T> *s_val = reinterpret_cast<const C2<T> *>(smem_raw + stage * buf + (size_t)cap * sizeof(int32_t));
    A sr = 0, si = 0;
    if (row < N) {
      const int b = __ldg(rp + row), e = __ldg(rp + row + 1);
      if (staged) {
        // batches of kBatch nonzeros per lane (the row's lanes take every
        // R-th one): all gathers of a batch are issued before the first is
        // used (rows of the mesh graph fit one batch); the values are read
        // from shared memory when used, so only the gathered x of a batch
        // occupies registers
        constexpr int kBatch = (sizeof(T) == 4 ? 16 : 8) / R;
        for (int k0 = b - ks + lane_r; k0 < e - ks; k0 += kBatch * R) {
          const int cnt = (e - ks - k0 + R - 1) / R;
          C2<T> xv[kBatch];
#pragma unroll
          for (int u = 0; u < kBatch; u++)
            if (u < cnt) xv[u] = ldg(x + s_col[k0 + u * R]);
#pragma unroll
          for (int u = 0; u < kBatch; u++) {
            if (u < cnt) {
              const C2<T> v = s_val[k0 + u * R];
              sr += v.x * xv[u].x - v.y * xv[u].y;
              si += v.x * xv[u].y + v.y * xv[u].x;
            }
          }
        }
      } else {
        for (int k = b + lane_r; k < e; k += R) {
          const C2<T> v = ldg(val + k);
          const C2<T> xv = ldg(x + __ldg(ci + k));
          sr += v.x * xv.x - v.y * xv.y;
          si += v.x * xv.y + v.y * xv.x;
        }
      }
    }
    // the row's lanes are adjacent: fold their partial sums into lane 0
#pragma unroll
    for (int o = R / 2; o > 0; o >>= 1) {
      sr += __shfl_xor_sync(0xffffffffu, sr, o);
      si += __shfl_xor_sync(0xffffffffu, si, o);
    }
    if (row < N && lane_r == 0) part += (typename PartOf<Op, A>::type)op.finish(row, sr, si, pre);
    __syncthreads();  // this buffer is refilled two row blocks later
  }
  if (!ok) {
    // a wait gave up: record it, give the copies still in flight (this row
    // block's and the next one's) a last wait at the default bound, so no
    // copy lands in shared memory after the CTA has left, and leave (the
    // results of this launch are invalid)
    if (threadIdx.x == 0) atomicOr(counter + kStageErrorSlot, 1u);
    if (cur_staged) mbar_wait(&bar[stage], parity[stage]);
    if (next_staged) mbar_wait(&bar[stage ^ 1], parity[stage ^ 1]);
    return;
  }
  if (Op::kReduce) {
    double total = 0.0;
    if (grid_reduce((double)part, partials, counter, red_out, &total)) run_hook(op, total);
  }
}

// Warp-cooperative schedule of the same SpMV + epilogue (no staging): a
// warp owns 32 consecutive rows and walks them in 16 pairs, a half-warp per
// row, each lane loading one nonzero (coalesced: a row's nonzeros are
// contiguous) and gathering its x; half-warp shuffles reduce the row and
// hand the sum to the row's own lane, so the epilogue runs on all 32 lanes
// with coalesced accesses.  Few registers and no shared memory: high
// occupancy for latency hiding.  kWarpThreads threads per CTA, persistent.
constexpr int kWarpThreads = 256;
template <typename T, class Op>
__global__ void __launch_bounds__(kWarpThreads)
    row_warp_apply(int N, const int32_t *__restrict__ rp, const int32_t *__restrict__ ci,
                   const C2<T> *__restrict__ val, const C2<T> *__restrict__ x, Op op, double *partials,
                   unsigned *counter, double *red_out) {
  using A = typename Acc<T>::type;
  dep_sync();
  if (halted(op)) return;
  const int lane = threadIdx.x & 31, hl = lane & 15, half = lane >> 4;
  const int nwb = (N + 31) / 32;
  const int wpb = kWarpThreads / 32;
  typename PartOf<Op, A>::type part = 0;
  for (int wb = blockIdx.x * wpb + (threadIdx.x >> 5); wb < nwb; wb += gridDim.x * wpb) {
    const int r0 = wb * 32;
    const int row = r0 + lane;
    typename Op::Pre pre{};
    if (row < N) pre = op.load(row);
    // row pointers of the 32 rows and the block end
    const int beg = __ldg(rp + min(row, N));
    const int bend = __ldg(rp + min(r0 + 32, N));
    A msr = 0, msi = 0;
    // two batches of 8 row pairs: the column ids and values of a batch are
    // loaded together, then all its x gathers, so a batch costs two memory
    // round trips; rows longer than 16 nonzeros finish in a tail loop
#pragma unroll
    for (int p0 = 0; p0 < 16; p0 += 8) {
      int k[8], e[8];
      int32_t c[8];
      C2<T> v[8], xv[8];
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const int rr = 2 * (p0 + q) + half;
        const int b = __shfl_sync(0xffffffffu, beg, rr);
        const int e1 = __shfl_sync(0xffffffffu, beg, (rr + 1) & 31);
        e[q] = rr < 31 ? e1 : bend;
        k[q] = b + hl;
      }
#pragma unroll
      for (int q = 0; q < 8; q++) {
        c[q] = 0;
        v[q] = C2<T>{0, 0};
        if (k[q] < e[q]) {
          c[q] = __ldg(ci + k[q]);
          v[q] = ldg(val + k[q]);
        }
      }
#pragma unroll
      for (int q = 0; q < 8; q++) xv[q] = k[q] < e[q] ? ldg(x + c[q]) : C2<T>{0, 0};
#pragma unroll
      for (int q = 0; q < 8; q++) {
        A sr = v[q].x * xv[q].x - v[q].y * xv[q].y;
        A si = v[q].x * xv[q].y + v[q].y * xv[q].x;
        for (int kk = k[q] + 16; kk < e[q]; kk += 16) {
          const C2<T> vv = ldg(val + kk);
          const C2<T> xx = ldg(x + __ldg(ci + kk));
          sr += vv.x * xx.x - vv.y * xx.y;
          si += vv.x * xx.y + vv.y * xx.x;
        }
#pragma unroll
        for (int off = 8; off > 0; off >>= 1) {
          sr += __shfl_xor_sync(0xffffffffu, sr, off);
          si += __shfl_xor_sync(0xffffffffu, si, off);
        }
        // lanes 2p and 2p+1 take the sums of halves 0 and 1
        const A tr = __shfl_sync(0xffffffffu, sr, (lane & 1) << 4);
        const A ti = __shfl_sync(0xffffffffu, si, (lane & 1) << 4);
        if ((lane >> 1) == p0 + q) {
          msr = tr;
          msi = ti;
        }
      }
    }
    if (row < N) part += (typename PartOf<Op, A>::type)op.finish(row, msr, msi, pre);
  }
  if (Op::kReduce) {
    double total = 0.0;
    if (grid_reduce((double)part, partials, counter, red_out, &total)) run_hook(op, total);
  }
}

// Resident CTAs of row_warp_apply on the device, capped by the work.
int warp_grid(const void *kernel, int64_t n_rows);

// Grid for a persistent row kernel of `threads` threads per CTA: the
// resident capacity of the device for this kernel and shared-memory size,
// capped by the number of row blocks.
int row_grid(const void *kernel, int threads, size_t smem, int64_t n_rows);

// Launch the SpMV + epilogue over an off-diagonal CSR with one of the two
// schedules (warp: row_warp_apply, else the staged row_block_apply with
// staging capacity cap).
//
// With `overlap` the launch may start while the previous kernel of the stream
// finishes (launch_dep); the staged schedule then copies its first row block
// before waiting for it, so the previous kernel must not write this matrix.
template <typename T, class Op>
void launch_spmv(bool warp, int N, const int32_t *rp, const int32_t *ci, const C2<T> *val, const C2<T> *x,
                 int cap, const Op &op, double *partials, unsigned *counter, double *red_out, cudaStream_t st,
                 bool overlap = false) {
  if (warp) {
    const int grid = warp_grid((const void *)row_warp_apply<T, Op>, N);
    launch_dep(overlap, row_warp_apply<T, Op>, dim3(grid), dim3(kWarpThreads), 0, st, N, rp, ci, val, x, op,
               partials, counter, red_out);
  } else {
    static bool attr_set = false;  // per instantiation; first call precedes any capture
    if (!attr_set) {
      NOSH_CUDA(cudaFuncSetAttribute(row_block_apply<T, Op>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     100 * 1024));
      attr_set = true;
    }
    const size_t smem = 2 * stage_bytes<T>(cap);
    launch_dep(overlap, row_block_apply<T, Op>,
               dim3(row_grid((const void *)row_block_apply<T, Op>, block_threads<T>(), smem, N)),
               dim3(block_threads<T>()), smem, st, N, rp, ci, val, x, cap, op, partials, counter, red_out);
  }
  NOSH_CUDA(cudaGetLastError());
}

// The faster schedule for one matrix: both are timed once (CUDA events,
// after a warm-up) on y = A x + D x with <x, y> reduced, when the matrix
// structure is set up.
template <typename T>
bool pick_warp_schedule(int N, const int32_t *rp, const int32_t *ci, const C2<T> *val, int cap, double *partials,
                        unsigned *counter, cudaStream_t st);

// ---- epilogues --------------------------------------------------------
// y = K x : diagonal K_ii = sum of incident alpha (real)
template <typename T>
struct KeoOp {
  static constexpr bool kReduce = false;
  const T *kdiag;
  const C2<T> *x;
  C2<T> *y;
  struct Pre {
    C2<T> xi;
    T d;
  };
  __device__ Pre load(int i) const { return Pre{x[i], kdiag[i]}; }
  __device__ double finish(int i, T sr, T si, const Pre &p) const {
    y[i] = C2<T>{sr + p.d * p.xi.x, si + p.d * p.xi.y};
    return 0.0;
  }
};

// y = sum (no diagonal): dK/dp
template <typename T>
struct PlainOp {
  static constexpr bool kReduce = false;
  C2<T> *y;
  struct Pre {};
  __device__ Pre load(int) const { return Pre{}; }
  __device__ double finish(int i, T sr, T si, const Pre &) const {
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
  struct Pre {
    C2<T> xi;
    T d0r, d0i, d1b;
  };
  __device__ Pre load(int i) const { return Pre{x[i], d[3 * i], d[3 * i + 1], d[3 * i + 2]}; }
  __device__ double finish(int i, T sr, T si, const Pre &p) const {
    const T yr = sr + p.d0r * p.xi.x + p.d1b * p.xi.y;
    const T yi = si + p.d1b * p.xi.x + p.d0i * p.xi.y;
    y[i] = C2<T>{yr, yi};
    return kDot ? (double)p.xi.x * (double)yr + (double)p.xi.y * (double)yi : 0.0;
  }
};

// F = K psi + cv t (V + g|psi|^2) psi (FP64), optionally ||F||^2; with soff,
// also the off-diagonal sums (K psi)_i - K_ii psi_i (the base of a later
// ResidualUpdateOp)
template <bool kNorm>
struct ResidualOp {
  static constexpr bool kReduce = kNorm;
  const double *kdiag, *cvt, *V;
  double g;
  const C2<double> *x;
  C2<double> *y;
  C2<double> *soff = nullptr;
  struct Pre {
    C2<double> p;
    double kd, ct, v;
  };
  __device__ Pre load(int i) const { return Pre{x[i], kdiag[i], cvt[i], V[i]}; }
  __device__ double finish(int i, double sr, double si, const Pre &q) const {
    if (soff) soff[i] = C2<double>{sr, si};
    const double a = q.kd + q.ct * (q.v + g * (q.p.x * q.p.x + q.p.y * q.p.y));
    const double fr = sr + a * q.p.x, fi = si + a * q.p.y;
    y[i] = C2<double>{fr, fi};
    return kNorm ? fr * fr + fi * fi : 0.0;
  }
};

// F of psi + dx from the off-diagonal sums of K psi (soff, FP64) and the
// FP32 SpMV of the update: soff += K dx (in place), F = soff + cv t (V +
// g|psi+dx|^2)(psi+dx) with the updated state `x` (FP64), ||F||^2 summed in
// FP64.  K is linear and the nonlinearity is per vertex, so this is F itself;
// the FP32 part is the product of the small update only, whose rounding
// (~1e-7 of |K dx|) lies far below the FP64 rounding of the O(1) sums.
struct ResidualUpdateOp {
  static constexpr bool kReduce = true;
  using Part = double;
  const double *kdiag, *cvt, *V;
  double g;
  const C2<double> *x;
  C2<double> *y;
  C2<double> *soff;
  struct Pre {
    C2<double> p, s;
    double kd, ct, v;
  };
  __device__ Pre load(int i) const { return Pre{x[i], soff[i], kdiag[i], cvt[i], V[i]}; }
  __device__ double finish(int i, float sr, float si, const Pre &q) const {
    const double s_r = q.s.x + (double)sr, s_i = q.s.y + (double)si;
    soff[i] = C2<double>{s_r, s_i};
    const double a = q.kd + q.ct * (q.v + g * (q.p.x * q.p.x + q.p.y * q.p.y));
    const double fr = s_r + a * q.p.x, fi = s_i + a * q.p.y;
    y[i] = C2<double>{fr, fi};
    return fr * fr + fi * fi;
  }
};

}  // namespace dev
}  // namespace nosh
