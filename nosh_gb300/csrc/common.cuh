// Shared helpers of the nosh_gb300 CUDA library (sm_103a only).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <thread>
#include <utility>
#include <vector>

#include "nosh_gb300.h"

namespace nosh {

// ---------------------------------------------------------------- errors
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

#define NOSH_CUDA(call)                                                      \
  do {                                                                       \
    cudaError_t e_ = (call);                                                 \
    if (e_ != cudaSuccess)                                                   \
      throw ::nosh::Error(NOSH_ERR_CUDA, std::string(#call) + ": " +         \
                                             cudaGetErrorString(e_));        \
  } while (0)

#define NOSH_CHECK(cond, code, msg)                                          \
  do {                                                                       \
    if (!(cond)) throw ::nosh::Error((code), (msg));                         \
  } while (0)

// ---------------------------------------------------------- device memory
template <typename T>
struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  explicit DevBuf(size_t count) { alloc(count); }
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  DevBuf(DevBuf &&o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
  DevBuf &operator=(DevBuf &&o) noexcept {
    if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
    return *this;
  }
  ~DevBuf() { release(); }
  void alloc(size_t count) {
    release();
    if (count == 0) return;
    cudaError_t e = cudaMalloc(&p, count * sizeof(T));
    if (e != cudaSuccess) {
      p = nullptr;
      throw Error(e == cudaErrorMemoryAllocation ? NOSH_ERR_NO_MEMORY
                                                 : NOSH_ERR_CUDA,
                  std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    n = count;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  void upload(const T *h, size_t count, cudaStream_t s) {
    if (count > n) alloc(count);
    if (count)
      NOSH_CUDA(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
  }
  void upload(const std::vector<T> &h, cudaStream_t s) { upload(h.data(), h.size(), s); }
  void download(T *h, size_t count, cudaStream_t s) const {
    if (count)
      NOSH_CUDA(cudaMemcpyAsync(h, p, count * sizeof(T), cudaMemcpyDeviceToHost, s));
  }
  void download_at(T *h, size_t count, size_t offset, cudaStream_t s) const {
    if (count)
      NOSH_CUDA(cudaMemcpyAsync(h, p + offset, count * sizeof(T), cudaMemcpyDeviceToHost, s));
  }
  void zero(cudaStream_t s) {
    if (n) NOSH_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), s));
  }
};

// True when p points to device (or managed) memory of the CUDA context.
bool is_device_pointer(const void *p);

// ------------------------------------------------------- host parallelism
// Static-partition parallel loop over [0, n) on the host cores (integer mesh
// work during set-up).
template <class F>
void parallel_for(int64_t n, F &&f, int64_t grain = 1 << 14) {
  unsigned hw = std::thread::hardware_concurrency();
  int64_t nt = hw ? hw : 1;
  if (nt > 64) nt = 64;
  if (n < grain * 2 || nt == 1) {
    for (int64_t i = 0; i < n; i++) f(i);
    return;
  }
  if (nt > n / grain) nt = n / grain;
  std::vector<std::thread> th;
  th.reserve(nt);
  for (int64_t t = 0; t < nt; t++) {
    int64_t b = n * t / nt, e = n * (t + 1) / nt;
    th.emplace_back([b, e, &f] {
      for (int64_t i = b; i < e; i++) f(i);
    });
  }
  for (auto &x : th) x.join();
}

// ------------------------------------------------------------ launch math
constexpr int kPad = 8;        // tail padding of nonzero arrays (elements)
constexpr int kNumSMs = 152;  // GB300: 2 dies x 76 SMs (queried at run time)
// Grid of a 256-thread FP64 reduction over n elements: about four elements
// per thread, at most two CTAs per SM.  GB300 issues FP64 at a small
// fraction of its FP32 rate, and with one element per thread the per-thread
// shuffle tree of each reduction costs more FP64 adds than the element work.
inline int reduce_grid(int64_t n) {
  const int64_t g = (n + 1023) / 1024;
  return (int)(g < 1 ? 1 : (g > 2 * kNumSMs ? 2 * kNumSMs : g));
}

// In place: each of the first n complex values c[2k], c[2k+1] (a dot
// product <x_k, x_0>) becomes the unit phase factor c / |c| (1 when c = 0)
// that aligns x_k with x_0.  One launch of 32 threads: the FP64 square root
// and divisions run once per factor, not once per vector element.
__global__ void normalize_phases(int n, double *c);
// out[2k], out[2k+1] = <x_k, x_0> (complex, sum conj(x_k) x_0) for the
// count <= 4 vectors x_1..x_count, reading x_0 once; deterministic grid
// reductions into counter slots 0 .. 2 count - 1.
__global__ void history_dots(int64_t n, const double *x0, const double *x1, const double *x2, const double *x3,
                             const double *x4, int count, double *partials, unsigned *counter, double *out);
inline int div_up(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

// Launch a kernel, with programmatic stream serialisation when `overlap` is
// set: the kernel's CTAs may then be scheduled as soon as the previous
// kernel's CTAs have exited, before that kernel's completion is signalled,
// and run up to their dev::dep_sync(), which returns once it has completed
// and its writes are visible.  Only kernels that call dep_sync() before
// touching memory the previous kernel writes may be launched with overlap.
template <typename... P, typename... Args>
void launch_dep(bool overlap, void (*kernel)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                Args &&...args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = overlap ? 1 : 0;
  NOSH_CUDA(cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...));
}

// The same for a grid of one thread-block cluster of `ctas` CTAs.
template <typename... P, typename... Args>
void launch_cluster_dep(bool overlap, int ctas, void (*kernel)(P...), dim3 block, size_t smem, cudaStream_t st,
                        Args &&...args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(ctas);
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[2];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = ctas;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[1].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = overlap ? 2 : 1;
  NOSH_CUDA(cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...));
}

}  // namespace nosh

// ----------------------------------------------------- device-side helpers
namespace nosh {
namespace dev {

template <typename T> struct C2;  // complex pair (interleaved storage)
template <> struct alignas(8) C2<float> { float x, y; };
template <> struct alignas(16) C2<double> { double x, y; };

// Programmatic dependent launch (griddepcontrol, sm_90 and later).
// dep_sync: block until the kernel this one was launched after (with
// overlap, see launch_dep) has completed and flushed its writes; returns at
// once for a plain launch.  Kernels do not trigger their successors
// explicitly (griddepcontrol.launch_dependents), so a successor launches as
// the last CTA exits, except for the one CTA that finishes a grid reduction
// (dep_trigger).  Measured on GB300 over chains of 100 graph-captured
// kernels (16 K to 8 M elements): the implicit trigger saved 0.16-0.25 us
// per launch against plain edges, while a trigger at the start of every CTA
// cost up to 3.8 us per launch (the successor's waiting CTAs hold the SMs)
// and one after the work in every CTA up to 1.4 us.
__device__ __forceinline__ void dep_sync() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
// Let the next kernel of the stream start launching now (used by the CTA
// that finishes a grid reduction: every other CTA has left by then, and its
// own tail of serial work overlaps the successor's launch; the successor
// still waits in dep_sync for this kernel's completion).
__device__ __forceinline__ void dep_trigger() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }

// read-only-path loads of complex pairs
__device__ __forceinline__ C2<float> ldg(const C2<float> *p) {
  const float2 v = __ldg(reinterpret_cast<const float2 *>(p));
  return C2<float>{v.x, v.y};
}
__device__ __forceinline__ C2<double> ldg(const C2<double> *p) {
  const double2 v = __ldg(reinterpret_cast<const double2 *>(p));
  return C2<double>{v.x, v.y};
}

template <typename T>
__device__ __forceinline__ C2<T> cmul(C2<T> a, C2<T> b) {
  return C2<T>{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}

// Warp-level sum of a double.
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-level sum (blockDim.x multiple of 32, <= 1024); valid in thread 0.
__device__ __forceinline__ double block_sum(double v, double *smem32) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) smem32[w] = v;
  __syncthreads();
  double r = 0.0;
  if (w == 0) {
    r = (lane < (int)(blockDim.x >> 5)) ? smem32[lane] : 0.0;
    r = warp_sum(r);
  }
  return r;
}

}  // namespace dev
}  // namespace nosh
