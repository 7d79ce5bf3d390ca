// Model-evaluator handle: fields, KEO / DkeoDP values, Jacobian and
// preconditioner state, all resident in HBM.
#pragma once

#include <memory>
#include <string>

#include "mesh.cuh"

namespace nosh {

using dev::C2;

// Scratch for deterministic grid reductions ("last block finishes"):
// per-block partial sums, an arrival counter and the finished scalars.
struct Reducer {
  DevBuf<double> partials;   // >= number of blocks of any reducing launch
  DevBuf<unsigned> counter;  // zero between launches
  DevBuf<double> out;        // result slots
  void init(int max_blocks, int nslots, cudaStream_t s) {
    partials.alloc(max_blocks * 4 + 64);
    counter.alloc(16);
    counter.zero(s);
    out.alloc(nslots);
    out.zero(s);
  }
};

struct Amg;  // aggregation AMG hierarchy (amg.cu)

// Event pairs around the launches of one kernel class (roofline timing).
// Outside stream capture the events are recorded on the stream.  Inside a
// capture they become event-record nodes of the graph (recorded again at
// every replay); the graph's owner takes them with take() and adds the
// replays it wants counted with harvest() once they have completed.
struct KernelTimer {
  bool on = false;
  std::vector<cudaEvent_t> ev;  // start, stop, start, stop, ...
  size_t used = 0;
  int64_t launches = 0;
  double bytes = 0.0;
  double graph_ms = 0.0;  // harvested graph pairs
  struct Pair {
    cudaEvent_t a = nullptr, b = nullptr;
    double bytes = 0.0;
    int n = 1;  // launches between the two events
  };
  std::vector<Pair> captured;  // pairs captured since the last take()
  Pair cap;
  bool cap_open = false;
  static bool capturing(cudaStream_t s) {
    cudaStreamCaptureStatus c = cudaStreamCaptureStatusNone;
    return cudaStreamIsCapturing(s, &c) == cudaSuccess && c != cudaStreamCaptureStatusNone;
  }
  bool open_pair = false;
  void begin(cudaStream_t s) {
    if (!on) return;
    if (capturing(s)) {
      NOSH_CUDA(cudaEventCreate(&cap.a));
      NOSH_CUDA(cudaEventCreate(&cap.b));
      NOSH_CUDA(cudaEventRecordWithFlags(cap.a, s, cudaEventRecordExternal));
      cap_open = true;
      return;
    }
    open_pair = true;
    if (used + 2 > ev.size()) {
      for (int k = 0; k < 2; k++) {
        cudaEvent_t e;
        NOSH_CUDA(cudaEventCreate(&e));
        ev.push_back(e);
      }
    }
    NOSH_CUDA(cudaEventRecord(ev[used], s));
  }
  // n: the launches of the class issued since begin (consecutive, with no
  // other kernel between them); b: their algorithmic bytes
  void end(cudaStream_t s, double b, int n = 1) {
    if (!on) return;
    if (cap_open) {
      cap_open = false;
      NOSH_CUDA(cudaEventRecordWithFlags(cap.b, s, cudaEventRecordExternal));
      cap.bytes = b;
      cap.n = n;
      captured.push_back(cap);
      return;
    }
    if (!open_pair) return;
    open_pair = false;
    NOSH_CUDA(cudaEventRecord(ev[used + 1], s));
    used += 2;
    launches += n;
    bytes += b;
  }
  std::vector<Pair> take() {
    std::vector<Pair> v;
    v.swap(captured);
    return v;
  }
  // one completed replay of a captured pair (bytes >= 0: this replay's
  // algorithmic bytes, when they differ from the captured launch's)
  void harvest(const Pair &p, double b = -1.0) {
    float t = 0.f;
    NOSH_CUDA(cudaEventElapsedTime(&t, p.a, p.b));
    graph_ms += t;
    launches += p.n;
    bytes += b >= 0.0 ? b : p.bytes;
  }
  static void release(std::vector<Pair> &v) {
    for (Pair &p : v) {
      cudaEventDestroy(p.a);
      cudaEventDestroy(p.b);
    }
    v.clear();
  }
  void read(int64_t &n, double &ms, double &b) {
    ms = graph_ms;
    graph_ms = 0.0;
    for (size_t k = 0; k < used; k += 2) {
      NOSH_CUDA(cudaEventSynchronize(ev[k + 1]));
      float t = 0.f;
      NOSH_CUDA(cudaEventElapsedTime(&t, ev[k], ev[k + 1]));
      ms += t;
    }
    n = launches;
    b = bytes;
    used = 0;
    launches = 0;
    bytes = 0.0;
  }
  ~KernelTimer() {
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
    release(captured);
  }
};

struct NlsImpl {
  MeshImpl *mesh;
  int64_t N, E;
  cudaStream_t stream = nullptr;
  int precision = NOSH_PREC_MIXED;
  std::string deriv_param;
  double g0, mu0;

  // fields (FP64) and derived per-edge / per-vertex data
  DevBuf<double> d_A, d_V, d_t, d_cvt;  // 3N, N, N, N (cv * thickness)
  std::vector<double> h_V, h_t;
  DevBuf<double> d_p, d_alpha, d_kdiag;  // E, E, N
  DevBuf<float> d_kdiagf;
  double cv_sum = 0.0;

  // off-diagonal KEO values in adjacency-CSR order (2E + kPad)
  DevBuf<C2<double>> d_keo64, d_dkeo64;
  DevBuf<C2<float>> d_keo32;
  double keo_mu = std::nan(""), dkeo_mu = std::nan("");

  // diagonal 2x2 blocks (Re-Re, Im-Im, Re-Im), K_ii included:
  // Jacobian (rebuild_diags_) and regularised KEO
  DevBuf<double> d_jd64, d_rd64;  // 3N each
  DevBuf<float> d_jd32, d_rd32;
  bool jac_ready = false, reg_ready = false;
  double reg_g = 0.0;

  // staging for host / misaligned vectors
  DevBuf<double> d_in, d_out, d_tmp;  // 2N each
  DevBuf<float> d_inf, d_outf;

  Reducer red;
  int cap32 = 0, cap64 = 0;  // staged nonzeros per row block (FP32 / FP64)
  // SpMV schedule of the fine-level operators (spmv.cuh): 0 autotuned, 1
  // staged row blocks, 2 warp-cooperative; warp32/64 hold the choice
  int spmv_schedule = 0;
  bool warp32 = false, warp64 = false;
  void tune_schedules();

  // independent systems (batched solves): vertices [sys_off[s], sys_off[s+1])
  // form system s, which uses its own mu (d_mu_sys) in the KEO; empty for
  // one system.  Edges never join two systems.
  std::vector<int64_t> sys_off;
  DevBuf<int64_t> d_sys_off;
  DevBuf<int32_t> d_esys;          // E: system of each edge
  DevBuf<double> d_mu_sys, d_sys_norm;  // per system
  std::vector<double> h_sys_norm;
  int64_t nsys() const { return sys_off.empty() ? 1 : (int64_t)sys_off.size() - 1; }
  void set_systems(const int64_t *offsets, int64_t num, const double *mu);
  // per-system ||F_s|| of f (2N) into h_sys_norm; returns the largest
  double system_norms(const double *f);
  // zero the rows of f that belong to systems with ||F_s|| <= tol
  void mask_converged(double *f, double tol);

  std::unique_ptr<Amg> amg;
  // preconditioner options (amg.cuh AmgOptions), applied when the hierarchy
  // is next built
  int amg_max_levels = 10, amg_coarse_size = 64, amg_smooth_degree = 2, amg_reuse_period = 8;
  // the fraction of the Newton target a step's forcing term aims at when the
  // target bounds it (eta >= forcing_aim * target / ||F||)
  double forcing_aim = 0.5;
  // launches of the MINRES iteration and the V-cycle overlap their
  // predecessors (programmatic dependent launch); off for A/B timing
  bool overlap_launches = true;
  double amg_theta = 0.0, amg_cheb_ratio = 15.0;
  KernelTimer timers[2];  // NOSH_KERNEL_JACOBIAN, NOSH_KERNEL_SMOOTHER
  mutable int64_t launch_count = 0;  // kernels launched by this handle
  // algorithmic bytes of one fine-level SpMV launch: matrix + indices once,
  // plus `vec_bytes_per_vertex` of vector traffic per vertex
  double spmv_bytes(int value_bytes, int vec_bytes_per_vertex) const {
    return 4.0 * (N + 1) + (4.0 + value_bytes) * 2.0 * E + (double)vec_bytes_per_vertex * N;
  }
  std::shared_ptr<void> solver_state;  // Newton / MINRES work space (solver.cu)

  NlsImpl(MeshImpl *m, const double *mvp, double mu, const double *V, double g,
          const double *t, const char *deriv);
  ~NlsImpl();

  // operators (device pointers to interleaved complex vectors)
  void keo_refill(double mu);
  void dkeo_refill(double mu);
  void keo_apply64(const double *x, double *y);
  void dkeo_apply64(const double *x, double *y);
  // y = F(x); optional ||F||^2 into red.out[slot]; with soff, also the
  // off-diagonal sums of K x (2N doubles), the base of residual_update
  void compute_f64(const double *x, double g, double mu, double *f, int norm_slot, double *soff = nullptr);
  // F and ||F||^2 (into red.out[0]; not waited for) of x = x_old + dx, dx
  // an FP32 update already added to x, from soff = the off-diagonal sums of
  // K x_old (updated in place to those of K x): an FP32 SpMV of dx with an
  // FP64 epilogue (ResidualUpdateOp)
  void residual_update(const double *x, const float *dx, double g, double mu, double *f, double *soff);
  // bounds for residual_update's rounding (computed once): the largest row
  // sum of |K| (mu-independent: |K_ij| = |alpha_ij|) and the longest row
  double keo_abs_rowmax();
  int max_row_nnz();
  double abs_rowmax_ = -1.0;
  int max_row_nnz_ = -1;
  void dfdp64(const double *x, double g, double mu, int param, double *out);
  // F(xa) into fa and F(xb) into fb in one pass, norms[0..1] = their norms
  // (synchronises); with sa / sb, also the off-diagonal sums of K xa / K xb
  void residual_pair(const double *xa, const double *xb, double g, double mu, double *fa, double *fb,
                     double norms[2], double *sa = nullptr, double *sb = nullptr, bool wait = true);
  // the norms of a residual_pair(..., wait = false): waits, then norms[0..1]
  void residual_pair_norms(double norms[2]);
  void jac_rebuild(const double *x, double g, double mu);
  // the FP32 diagonal blocks of J and of the regularised KEO only, for a
  // mixed-precision solve
  void operators32_rebuild(const double *x, double g, double mu);
  void reg_rebuild(const double *x, double g, double mu);
  template <typename T>
  void jac_apply(const T *x, T *y, double *dot_out = nullptr);
  template <typename T>
  void reg_apply(const T *x, T *y);
  double energy(const double *psi);
  double inner_product(const double *phi, const double *psi);
  // full-graph values (with diagonal) in complex_graph order, complex
  void export_values(const C2<double> *offdiag, const double *diag, double *out);

  // Waits for the handle's stream.  A staged SpMV that gave up waiting for
  // its copies (kStageErrorSlot set) makes it throw NOSH_ERR_CUDA after
  // clearing the flag and the reduction counters, so the handle stays usable.
  void sync();
  [[noreturn]] void stage_failure();
  unsigned *h_stage_err = nullptr;  // pinned, one word
  // diagnostics: bound of the staging waits (polls; < 0 restores the default)
  void set_stage_wait_limit(int64_t polls);
  // index-check mode: the KEO graph is validated on the device before every
  // Newton solve, continuation step and operator apply of the C ABI
  bool index_checks = false;
  DevBuf<unsigned long long> d_check;
  void check_indices();
};

// index-check mode: validates an off-diagonal CSR graph on the device into
// *err_dev (all ones: valid; else the first offence, see ops.cu), and turns
// a host copy of that word into NOSH_ERR_INVALID with the position
void check_graph(int64_t N, int64_t nnz, const int32_t *rp, const int32_t *ci, unsigned long long *err_dev,
                 cudaStream_t st);
void report_graph_error(unsigned long long w);

// streaming read of `bytes` (a multiple of 16) at 16-byte aligned device
// memory, XOR-reduced into *out (the achievable-bandwidth probe)
void stream_read(const void *buf, int64_t bytes, unsigned *out, cudaStream_t st);

// launch helpers shared with the solver
void launch_f64_to_f32(const double *a, float *b, int64_t n, cudaStream_t s);
void launch_f32_to_f64(const float *a, double *b, int64_t n, cudaStream_t s);

}  // namespace nosh
