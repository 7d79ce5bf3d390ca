// Residual + norm entry point that allocates no device memory.
//
// Same fused kernel as nosh_nls_compute_f_norm (row-block SpMV of the KEO
// with the F epilogue and a grid reduction of ||F||^2), but everything comes
// from the caller and the reduction's scratch (per-CTA partial sums and the
// arrival counter) lives in one file-scope __device__ array instead of a
// buffer owned by an nls handle.
#include <mutex>

#include "spmv.cuh"

namespace nosh {
void set_last_error(const std::string &msg);  // capi.cu

namespace {

using namespace dev;

// Scratch: element 0 holds the arrival counter (read as unsigned), elements
// 1..kNoallocMaxBlocks the per-CTA partial sums.  One launch uses one CTA per
// kRows rows, so the largest mesh is kNoallocMaxBlocks * kRows vertices.
constexpr int64_t kNoallocMaxBlocks = 65536;
constexpr int64_t kNoallocMaxVertices = kNoallocMaxBlocks * kRows;  // 8,388,608
static __device__ __align__(256) double g_noalloc_scratch[1 + kNoallocMaxBlocks];

constexpr int kMaxDevices = 64;
std::mutex g_mtx;
double *g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device.  The array's
// name is only a host-side stand-in in host code, so the address is looked up
// once per device (with that device current) and cached.
double *scratch_on_current_device() {
  int dev = 0;
  NOSH_CUDA(cudaGetDevice(&dev));
  NOSH_CHECK(dev >= 0 && dev < kMaxDevices, NOSH_ERR_INVALID, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_mtx);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr)
      throw Error(NOSH_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
    g_scratch_ptr[dev] = static_cast<double *>(p);
  }
  return g_scratch_ptr[dev];
}

// The residual epilogue whose finishing thread also takes the square root:
// grid_reduce stores ||F||^2 into *norm, then the hook overwrites it with
// ||F||, so the call is one launch.
struct ResidualNormOp : ResidualOp<true> {
  static constexpr bool kHook = true;
  double *norm;
  __device__ void hook(double total) const { *norm = sqrt(total); }
};

// Device memory of `device` (or managed memory, reachable from every
// device), aligned to `align` bytes.
bool device_resident(const void *p, size_t align, int device) {
  if (p == nullptr || reinterpret_cast<uintptr_t>(p) % align != 0) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (a.type == cudaMemoryTypeManaged) return true;
  return a.type == cudaMemoryTypeDevice && a.device == device;
}

}  // namespace
}  // namespace nosh

extern "C" int nosh_residual_norm_noalloc(int64_t num_vertices, const int32_t *row_ptr,
                                          const int32_t *cols, const double *keo_offdiag,
                                          const double *keo_diag, const double *cv_thickness,
                                          const double *scalar_potential, double g,
                                          const double *psi, double *f, double *norm,
                                          void *stream) {
  using namespace nosh;
  try {
    NOSH_CHECK(num_vertices >= 1, NOSH_ERR_INVALID, "num_vertices must be >= 1");
    NOSH_CHECK(num_vertices <= kNoallocMaxVertices, NOSH_ERR_INVALID,
               "nosh_residual_norm_noalloc: " + std::to_string(num_vertices) +
                   " vertices exceed the fixed scratch limit of " +
                   std::to_string(kNoallocMaxVertices) + "; use nosh_nls_compute_f_norm");
    int device = 0;
    NOSH_CUDA(cudaGetDevice(&device));
    NOSH_CHECK(device_resident(row_ptr, 4, device) && device_resident(cols, 4, device) &&
                   device_resident(keo_diag, 8, device) && device_resident(cv_thickness, 8, device) &&
                   device_resident(scalar_potential, 8, device) && device_resident(norm, 8, device),
               NOSH_ERR_INVALID,
               "nosh_residual_norm_noalloc: every array must be device memory of the current device (" +
                   std::to_string(device) + ")");
    NOSH_CHECK(device_resident(keo_offdiag, 16, device) && device_resident(psi, 16, device) &&
                   device_resident(f, 16, device),
               NOSH_ERR_INVALID,
               "nosh_residual_norm_noalloc: complex arrays (keo_offdiag, psi, f) must be "
               "16-byte aligned device memory of the current device (" + std::to_string(device) + ")");
    double *scratch = scratch_on_current_device();
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // the arrival counter must start at zero; the partials are overwritten
    NOSH_CUDA(cudaMemsetAsync(scratch, 0, sizeof(double), s));
    ResidualNormOp op;
    op.kdiag = keo_diag;
    op.cvt = cv_thickness;
    op.V = scalar_potential;
    op.g = g;
    op.x = reinterpret_cast<const dev::C2<double> *>(psi);
    op.y = reinterpret_cast<dev::C2<double> *>(f);
    op.norm = norm;
    const int grid = div_up(num_vertices, dev::kRows);
    // cap = 0: nonzeros are read directly (no shared-memory staging), so the
    // launch needs no host-side knowledge of the row pointers
    dev::row_block_apply<double, ResidualNormOp><<<grid, dev::block_threads<double>(), 0, s>>>(
        (int)num_vertices, row_ptr, cols, reinterpret_cast<const dev::C2<double> *>(keo_offdiag),
        reinterpret_cast<const dev::C2<double> *>(psi), 0, op, scratch + 1,
        reinterpret_cast<unsigned *>(scratch), norm);
    NOSH_CUDA(cudaGetLastError());
    set_last_error("");
    return NOSH_OK;
  } catch (const Error &e) {
    set_last_error(e.what());
    return e.code;
  }
}
