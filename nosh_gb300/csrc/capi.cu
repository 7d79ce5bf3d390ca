// extern "C" entry points (include/nosh_gb300.h).  Argument checking,
// host/device pointer staging and error translation; the work itself is in
// mesh.cu, ops.cu, amg.cu and solver.cu.
#include <cmath>
#include <cstring>
#include <string>

#include "amg.cuh"
#include "nls.cuh"
#include "continuation.cuh"
#include "mpnn.cuh"
#include "solver.cuh"

struct nosh_mesh_s {
  nosh::MeshImpl *impl;
};
struct nosh_nls_s {
  nosh::NlsImpl *impl;
};
struct nosh_continuation_s {
  nosh::ContinuationImpl *impl;
};
struct nosh_mpnn_s {
  nosh::Mpnn *impl;
};

namespace {

thread_local std::string g_last_error;

template <class F>
int guarded(F &&f) {
  try {
    g_last_error.clear();
    f();
    return NOSH_OK;
  } catch (const nosh::Error &e) {
    g_last_error = e.what();
    return e.code;
  } catch (const std::bad_alloc &) {
    g_last_error = "out of host memory";
    return NOSH_ERR_NO_MEMORY;
  } catch (const std::exception &e) {
    g_last_error = e.what();
    return NOSH_ERR_INVALID;
  }
}

void require(bool c, const char *msg) {
  if (!c) throw nosh::Error(NOSH_ERR_INVALID, msg);
}

void require_gpu() {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    throw nosh::Error(NOSH_ERR_CUDA, "no usable CUDA device");
  }
}

nosh::NlsImpl &N(nosh_nls h) {
  require(h && h->impl, "null nls handle");
  return *h->impl;
}
// N() for the entry points that run kernels over the KEO graph: in
// index-check mode the graph is validated on the device first
nosh::NlsImpl &NC(nosh_nls h) {
  nosh::NlsImpl &s = N(h);
  if (s.index_checks) s.check_indices();
  return s;
}
nosh::MeshImpl &M(nosh_mesh h) {
  require(h && h->impl, "null mesh handle");
  return *h->impl;
}

// Parameter vector [g, mu] from host or device memory.
void read_params(const double *p, double &g, double &mu) {
  require(p != nullptr, "null parameter vector");
  double h[2];
  if (nosh::is_device_pointer(p)) {
    NOSH_CUDA(cudaMemcpy(h, p, sizeof(h), cudaMemcpyDeviceToHost));
  } else {
    h[0] = p[0];
    h[1] = p[1];
  }
  require(!std::isnan(h[0]) && !std::isnan(h[1]), "parameter is NaN");
  g = h[0];
  mu = h[1];
}

bool usable_in_place(const void *p) {
  return nosh::is_device_pointer(p) && (reinterpret_cast<uintptr_t>(p) % 16) == 0;
}

// Device view of a caller's input vector of n doubles.
const double *stage_in(nosh::NlsImpl &s, const double *user, nosh::DevBuf<double> &buf, size_t n) {
  require(user != nullptr, "null vector argument");
  if (usable_in_place(user)) return user;
  if (buf.n < n) buf.alloc(n);
  NOSH_CUDA(cudaMemcpyAsync(buf.p, user, n * sizeof(double), cudaMemcpyDefault, s.stream));
  return buf.p;
}

// Device destination for a caller's output vector; finish() copies back.
struct OutVec {
  double *user, *dev;
  size_t n;
  OutVec(nosh::NlsImpl &s, double *u, nosh::DevBuf<double> &buf, size_t count)
      : user(u), dev(nullptr), n(count) {
    require(u != nullptr, "null output vector");
    if (usable_in_place(u)) {
      dev = u;
    } else {
      if (buf.n < n) buf.alloc(n);
      dev = buf.p;
    }
  }
  void finish(nosh::NlsImpl &s) {
    if (dev != user)
      NOSH_CUDA(cudaMemcpyAsync(user, dev, n * sizeof(double), cudaMemcpyDefault, s.stream));
    s.sync();
  }
};

void check_apply_args(int mode, double alpha, double beta, int nvec) {
  // jacobian_operator::apply accepts only NO_TRANS, alpha == 1, beta == 0
  // (src/jacobian_operator.cpp:48-59)
  if (mode != NOSH_NO_TRANS)
    throw nosh::Error(NOSH_ERR_UNSUPPORTED, "Only untransposed applies supported.");
  if (alpha != 1.0) throw nosh::Error(NOSH_ERR_UNSUPPORTED, "Only alpha==1.0 supported.");
  if (beta != 0.0) throw nosh::Error(NOSH_ERR_UNSUPPORTED, "Only beta==0.0 supported.");
  require(nvec >= 1, "num_vectors must be >= 1");
}

}  // namespace

namespace nosh {
// lets other translation units report through nosh_last_error()
void set_last_error(const std::string &msg) { g_last_error = msg; }

bool is_device_pointer(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}
}  // namespace nosh

extern "C" {

const char *nosh_last_error(void) { return g_last_error.c_str(); }

int nosh_version(void) { return 100; }

int nosh_device_count(int *count) {
  return guarded([&] {
    require(count != nullptr, "null count");
    *count = 0;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) {
      cudaGetLastError();
      throw nosh::Error(NOSH_ERR_CUDA, cudaGetErrorString(e));
    }
    *count = n;
  });
}

// ---------------------------------------------------------------- mesh
int nosh_mesh_create(const double *coords, int64_t num_vertices, const int32_t *cells,
                     int64_t num_cells, int verts_per_cell, nosh_mesh *out) {
  return guarded([&] {
    require(out != nullptr && coords != nullptr && cells != nullptr, "null argument");
    *out = nullptr;
    // a malformed mesh is reported as such with or without a GPU
    nosh::MeshImpl::validate(num_vertices, cells, num_cells, verts_per_cell);
    require_gpu();
    auto *h = new nosh_mesh_s{nullptr};
    try {
      h->impl = new nosh::MeshImpl(coords, num_vertices, cells, num_cells, verts_per_cell);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}

int nosh_mesh_destroy(nosh_mesh mesh) {
  return guarded([&] {
    if (!mesh) return;
    delete mesh->impl;
    delete mesh;
  });
}

int nosh_mesh_sizes(nosh_mesh mesh, int64_t *nv, int64_t *ne, int64_t *nc, int64_t *nnz) {
  return guarded([&] {
    auto &m = M(mesh);
    if (nv) *nv = m.N;
    if (ne) *ne = m.E;
    if (nc) *nc = m.T;
    if (nnz) *nnz = m.N + 2 * m.E;
  });
}

int nosh_mesh_edges(nosh_mesh mesh, int32_t *edges) {
  return guarded([&] {
    auto &m = M(mesh);
    require(edges != nullptr, "null output");
    std::memcpy(edges, m.edges.data(), m.edges.size() * sizeof(int32_t));
  });
}

int nosh_mesh_edge_gids_complex(nosh_mesh mesh, int32_t *idx) {
  return guarded([&] {
    auto &m = M(mesh);
    require(idx != nullptr, "null output");
    for (int64_t e = 0; e < m.E; e++) {
      const int32_t g0 = m.edges[2 * e] + 1, g1 = m.edges[2 * e + 1] + 1;  // 1-based GIDs
      idx[4 * e + 0] = 2 * g0;
      idx[4 * e + 1] = 2 * g0 + 1;
      idx[4 * e + 2] = 2 * g1;
      idx[4 * e + 3] = 2 * g1 + 1;
    }
  });
}

int nosh_mesh_edge_data(nosh_mesh mesh, double *length, double *covolume) {
  return guarded([&] {
    auto &m = M(mesh);
    if (length) std::memcpy(length, m.h_len.data(), m.E * sizeof(double));
    if (covolume) std::memcpy(covolume, m.h_covol.data(), m.E * sizeof(double));
  });
}

int nosh_mesh_control_volumes(nosh_mesh mesh, double *cv) {
  return guarded([&] {
    auto &m = M(mesh);
    require(cv != nullptr, "null output");
    std::memcpy(cv, m.h_cv.data(), m.N * sizeof(double));
  });
}

int nosh_mesh_complex_graph(nosh_mesh mesh, int32_t *row_ptr, int32_t *cols) {
  return guarded([&] {
    auto &m = M(mesh);
    require(row_ptr != nullptr && cols != nullptr, "null output");
    m.complex_graph(row_ptr, cols);
  });
}

// ------------------------------------------------------------------ nls
int nosh_nls_create(nosh_mesh mesh, const double *mvp, double mu, const double *V, double g,
                    const double *t, const char *deriv, nosh_nls *out) {
  return guarded([&] {
    require(out != nullptr && mvp != nullptr && V != nullptr && t != nullptr, "null argument");
    *out = nullptr;
    auto &m = M(mesh);
    auto *h = new nosh_nls_s{nullptr};
    try {
      h->impl = new nosh::NlsImpl(&m, mvp, mu, V, g, t, deriv);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}

int nosh_nls_destroy(nosh_nls nls) {
  return guarded([&] {
    if (!nls) return;
    delete nls->impl;
    delete nls;
  });
}

int nosh_nls_num_params(nosh_nls nls, int *num) {
  return guarded([&] {
    N(nls);
    require(num != nullptr, "null output");
    *num = 2;
  });
}

int nosh_nls_param_name(nosh_nls nls, int index, char *buf, size_t len) {
  return guarded([&] {
    N(nls);
    require(buf != nullptr && len >= 3, "buffer too small");
    require(index == 0 || index == 1, "parameter index out of range");
    std::strcpy(buf, index == 0 ? "g" : "mu");
  });
}

int nosh_nls_set_precision(nosh_nls nls, int precision) {
  return guarded([&] {
    require(precision == NOSH_PREC_FP64 || precision == NOSH_PREC_MIXED, "unknown precision");
    N(nls).precision = precision;
  });
}

int nosh_nls_get_precision(nosh_nls nls, int *precision) {
  return guarded([&] {
    require(precision != nullptr, "null argument");
    *precision = N(nls).precision;
  });
}

int nosh_nls_set_amg_options(nosh_nls nls, int max_levels, int coarse_size, int smooth_degree,
                             int reuse_period, double strength_threshold, double cheb_ratio) {
  return guarded([&] {
    auto &s = N(nls);
    require(max_levels >= 1 && max_levels <= 16 && coarse_size >= 1 && coarse_size <= 512 &&
                smooth_degree >= 1 && smooth_degree <= 8 && reuse_period >= 1 && strength_threshold >= 0 &&
                strength_threshold < 1 && cheb_ratio > 1,
            "AMG options out of range");
    s.amg_max_levels = max_levels;
    s.amg_coarse_size = coarse_size;
    s.amg_smooth_degree = smooth_degree;
    s.amg_reuse_period = reuse_period;
    s.amg_theta = strength_threshold;
    s.amg_cheb_ratio = cheb_ratio;
    nosh::reset_preconditioner(s);
  });
}

int nosh_nls_set_systems(nosh_nls nls, int64_t num_systems, const int64_t *vertex_offsets, const double *mu) {
  return guarded([&] {
    auto &s = N(nls);
    require(num_systems >= 1 && vertex_offsets && mu, "null argument");
    s.set_systems(vertex_offsets, num_systems, mu);
    nosh::reset_preconditioner(s);
  });
}

int nosh_nls_system_iterations(nosh_nls nls, int *newton_iters, int *krylov_iters) {
  return guarded([&] {
    auto &s = N(nls);
    require(!s.sys_off.empty(), "no systems set");
    nosh::NewtonState &ns = nosh::state_of(s);
    const int64_t S = s.nsys();
    for (int64_t q = 0; q < S; q++) {
      if (newton_iters) newton_iters[q] = q < (int64_t)ns.sys_newton.size() ? ns.sys_newton[q] : 0;
      if (krylov_iters) krylov_iters[q] = q < (int64_t)ns.sys_krylov.size() ? ns.sys_krylov[q] : 0;
    }
  });
}

int nosh_nls_system_norms(nosh_nls nls, double *norms) {
  return guarded([&] {
    auto &s = N(nls);
    require(norms != nullptr, "null argument");
    require(!s.sys_off.empty(), "no systems set");
    std::copy(s.h_sys_norm.begin(), s.h_sys_norm.end(), norms);
  });
}

int nosh_nls_amg_levels(nosh_nls nls, int *num_levels, int64_t *sizes, int max_sizes, int *tail_level) {
  return guarded([&] {
    auto &s = N(nls);
    require(num_levels != nullptr, "null argument");
    if (!s.amg) {
      *num_levels = 0;
      if (tail_level) *tail_level = -1;
      return;
    }
    *num_levels = s.amg->num_levels();
    for (int l = 0; l < std::min(*num_levels, max_sizes) && sizes; l++) sizes[l] = s.amg->level_size(l);
    if (tail_level) *tail_level = s.amg->tail_level();
  });
}

int nosh_nls_set_spmv_schedule(nosh_nls nls, int schedule) {
  return guarded([&] {
    auto &s = N(nls);
    require(schedule >= 0 && schedule <= 2, "unknown SpMV schedule");
    s.spmv_schedule = schedule;
    s.tune_schedules();
    nosh::reset_preconditioner(s);
  });
}

int nosh_diag_stream_read(const void *buf, int64_t bytes, void *out_word, void *stream) {
  return guarded([&] {
    require(buf != nullptr && out_word != nullptr, "null argument");
    require(bytes >= 16 && bytes % 16 == 0, "bytes must be a positive multiple of 16");
    require(reinterpret_cast<uintptr_t>(buf) % 16 == 0 && reinterpret_cast<uintptr_t>(out_word) % 4 == 0,
            "misaligned buffer");
    require(nosh::is_device_pointer(buf) && nosh::is_device_pointer(out_word), "device memory expected");
    nosh::stream_read(buf, bytes, static_cast<unsigned *>(out_word), static_cast<cudaStream_t>(stream));
  });
}

int nosh_nls_set_index_checks(nosh_nls nls, int enable) {
  return guarded([&] {
    auto &s = N(nls);
    s.index_checks = enable != 0;
    if (s.index_checks) s.check_indices();
  });
}

int nosh_graph_check(int64_t num_vertices, int64_t nnz, const int32_t *row_ptr, const int32_t *cols,
                     void *stream) {
  return guarded([&] {
    require(num_vertices >= 1 && nnz >= 0, "bad sizes");
    require(nosh::is_device_pointer(row_ptr) && (nnz == 0 || nosh::is_device_pointer(cols)),
            "row_ptr and cols must be device memory");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    nosh::DevBuf<unsigned long long> err(1);
    nosh::check_graph(num_vertices, nnz, row_ptr, cols, err.p, st);
    unsigned long long w = 0;
    NOSH_CUDA(cudaMemcpyAsync(&w, err.p, sizeof(w), cudaMemcpyDeviceToHost, st));
    NOSH_CUDA(cudaStreamSynchronize(st));
    nosh::report_graph_error(w);
  });
}

int nosh_nls_set_forcing_aim(nosh_nls nls, double aim) {
  return guarded([&] {
    require(aim > 0.0 && aim <= 1.0, "the forcing aim must lie in (0, 1]");
    N(nls).forcing_aim = aim;
  });
}

int nosh_nls_set_launch_overlap(nosh_nls nls, int enable) {
  return guarded([&] {
    auto &s = N(nls);
    require(enable == 0 || enable == 1, "enable must be 0 or 1");
    s.overlap_launches = enable == 1;
    nosh::reset_preconditioner(s);
  });
}

int nosh_nls_set_stage_wait_limit(nosh_nls nls, int64_t polls) {
  return guarded([&] { N(nls).set_stage_wait_limit(polls); });
}

int nosh_nls_stream(nosh_nls nls, void **stream) {
  return guarded([&] {
    require(stream != nullptr, "null output");
    *stream = (void *)N(nls).stream;
  });
}

int nosh_nls_compute_f_norm(nosh_nls nls, const double *x, const double *p, double *f,
                            double *norm) {
  return guarded([&] {
    auto &s = NC(nls);
    double g, mu;
    read_params(p, g, mu);
    const double *dx = stage_in(s, x, s.d_in, 2 * s.N);
    OutVec of(s, f, s.d_out, 2 * s.N);
    s.compute_f64(dx, g, mu, of.dev, norm ? 0 : -1);
    double n2 = 0.0;
    if (norm) s.red.out.download(&n2, 1, s.stream);
    of.finish(s);
    if (norm) *norm = std::sqrt(n2);
  });
}

int nosh_nls_compute_f(nosh_nls nls, const double *x, const double *p, double *f) {
  return nosh_nls_compute_f_norm(nls, x, p, f, nullptr);
}

int nosh_nls_compute_dfdp(nosh_nls nls, const double *x, const double *p, double *dfdp) {
  return guarded([&] {
    auto &s = NC(nls);
    double g, mu;
    read_params(p, g, mu);
    const double *dx = stage_in(s, x, s.d_in, 2 * s.N);
    require(dfdp != nullptr, "null output");
    for (int k = 0; k < 2; k++) {
      OutVec o(s, dfdp + k * 2 * s.N, s.d_out, 2 * s.N);
      s.dfdp64(dx, g, mu, k, o.dev);
      o.finish(s);
    }
  });
}

int nosh_nls_gibbs_energy(nosh_nls nls, const double *psi, double *out) {
  return guarded([&] {
    auto &s = N(nls);
    require(out != nullptr, "null output");
    *out = s.energy(stage_in(s, psi, s.d_in, 2 * s.N));
  });
}

int nosh_nls_inner_product(nosh_nls nls, const double *phi, const double *psi, double *out) {
  return guarded([&] {
    auto &s = N(nls);
    require(out != nullptr, "null output");
    const double *a = stage_in(s, phi, s.d_in, 2 * s.N);
    const double *b = stage_in(s, psi, s.d_tmp, 2 * s.N);
    *out = s.inner_product(a, b);
  });
}

// --------------------------------------------------- parameter matrices
int nosh_keo_set_parameters(nosh_nls nls, const double *p) {
  return guarded([&] {
    auto &s = N(nls);
    double g, mu;
    read_params(p, g, mu);
    s.keo_refill(mu);
    s.sync();
  });
}

int nosh_keo_values(nosh_nls nls, double *vals) {
  return guarded([&] {
    auto &s = N(nls);
    require(!std::isnan(s.keo_mu), "KEO not filled: call nosh_keo_set_parameters first");
    const size_t n = 2 * (s.N + 2 * s.E);
    nosh::DevBuf<double> tmp(n);
    s.export_values(s.d_keo64.p, s.d_kdiag.p, tmp.p);
    tmp.download(vals, n, s.stream);
    s.sync();
  });
}

int nosh_keo_apply(nosh_nls nls, const double *x, double *y) {
  return guarded([&] {
    auto &s = NC(nls);
    require(!std::isnan(s.keo_mu), "KEO not filled: call nosh_keo_set_parameters first");
    const double *dx = stage_in(s, x, s.d_in, 2 * s.N);
    OutVec o(s, y, s.d_out, 2 * s.N);
    s.keo_apply64(dx, o.dev);
    o.finish(s);
  });
}

int nosh_dkeo_set_parameters(nosh_nls nls, const double *p) {
  return guarded([&] {
    auto &s = N(nls);
    double g, mu;
    read_params(p, g, mu);
    s.dkeo_refill(mu);
    s.sync();
  });
}

int nosh_dkeo_values(nosh_nls nls, double *vals) {
  return guarded([&] {
    auto &s = N(nls);
    require(!std::isnan(s.dkeo_mu), "DkeoDP not filled: call nosh_dkeo_set_parameters first");
    const size_t n = 2 * (s.N + 2 * s.E);
    nosh::DevBuf<double> tmp(n);
    s.export_values(s.d_dkeo64.p, nullptr, tmp.p);
    tmp.download(vals, n, s.stream);
    s.sync();
  });
}

int nosh_dkeo_apply(nosh_nls nls, const double *x, double *y) {
  return guarded([&] {
    auto &s = NC(nls);
    require(!std::isnan(s.dkeo_mu), "DkeoDP not filled: call nosh_dkeo_set_parameters first");
    const double *dx = stage_in(s, x, s.d_in, 2 * s.N);
    OutVec o(s, y, s.d_out, 2 * s.N);
    s.dkeo_apply64(dx, o.dev);
    o.finish(s);
  });
}

// --------------------------------------------------- jacobian operator
int nosh_jacobian_rebuild(nosh_nls nls, const double *p, const double *x) {
  return guarded([&] {
    auto &s = N(nls);
    double g, mu;
    read_params(p, g, mu);
    s.jac_rebuild(stage_in(s, x, s.d_in, 2 * s.N), g, mu);
    s.sync();
  });
}

int nosh_jacobian_apply(nosh_nls nls, const double *X, double *Y, int nvec, int mode,
                        double alpha, double beta) {
  return guarded([&] {
    auto &s = NC(nls);
    check_apply_args(mode, alpha, beta, nvec);
    require(s.jac_ready, "Jacobian not built: call nosh_jacobian_rebuild first");
    for (int k = 0; k < nvec; k++) {
      const double *dx = stage_in(s, X + (size_t)k * 2 * s.N, s.d_in, 2 * s.N);
      OutVec o(s, Y + (size_t)k * 2 * s.N, s.d_out, 2 * s.N);
      if (s.precision == NOSH_PREC_FP64) {
        s.jac_apply<double>(dx, o.dev);
      } else {
        nosh::launch_f64_to_f32(dx, s.d_inf.p, 2 * s.N, s.stream);
        s.jac_apply<float>(s.d_inf.p, s.d_outf.p);
        nosh::launch_f32_to_f64(s.d_outf.p, o.dev, 2 * s.N, s.stream);
      }
      o.finish(s);
    }
  });
}

// -------------------------------------------------------- preconditioner
int nosh_keo_regularized_rebuild(nosh_nls nls, const double *p, const double *x) {
  return guarded([&] {
    auto &s = N(nls);
    double g, mu;
    read_params(p, g, mu);
    s.reg_rebuild(stage_in(s, x, s.d_in, 2 * s.N), g, mu);
    nosh::Amg &amg = nosh::ensure_preconditioner(s);
    if (s.precision == NOSH_PREC_FP64) amg.refresh<double>();
    else amg.refresh<float>();
    s.sync();
  });
}

int nosh_keo_regularized_apply(nosh_nls nls, const double *X, double *Y, int nvec, int mode,
                               double alpha, double beta) {
  return guarded([&] {
    auto &s = NC(nls);
    check_apply_args(mode, alpha, beta, nvec);
    require(s.reg_ready && s.amg, "preconditioner not built: call nosh_keo_regularized_rebuild");
    for (int k = 0; k < nvec; k++) {
      const double *dx = stage_in(s, X + (size_t)k * 2 * s.N, s.d_in, 2 * s.N);
      OutVec o(s, Y + (size_t)k * 2 * s.N, s.d_out, 2 * s.N);
      if (s.precision == NOSH_PREC_FP64) {
        s.amg->apply<double>(dx, o.dev);
      } else {
        nosh::launch_f64_to_f32(dx, s.d_inf.p, 2 * s.N, s.stream);
        s.amg->apply<float>(s.d_inf.p, s.d_outf.p);
        nosh::launch_f32_to_f64(s.d_outf.p, o.dev, 2 * s.N, s.stream);
      }
      o.finish(s);
    }
  });
}

int nosh_eig_lowest(nosh_nls nls, const double *psi, const double *p, int k, double tol, int maxit, int guard,
                    int deflate_gauge, uint64_t seed, double *eigenvalues, double *eigenvectors, int *iterations) {
  return guarded([&] {
    auto &s = NC(nls);
    double g, mu;
    read_params(p, g, mu);
    require(eigenvalues != nullptr, "null eigenvalue output");
    require(k >= 1 && tol > 0 && maxit >= 1, "bad eigensolver options");
    const double *dpsi = stage_in(s, psi, s.d_tmp, 2 * s.N);
    const int its = nosh::lowest_eigenpairs(s, dpsi, g, mu, k, tol, maxit, guard, deflate_gauge != 0, seed,
                                            eigenvalues, eigenvectors);
    if (iterations) *iterations = its;
  });
}

int nosh_keo_regularized_smoother_apply(nosh_nls nls, const double *x, double *y) {
  return guarded([&] {
    auto &s = NC(nls);
    require(s.reg_ready && s.amg, "preconditioner not built: call nosh_keo_regularized_rebuild");
    const double *dx = stage_in(s, x, s.d_in, 2 * s.N);
    OutVec o(s, y, s.d_out, 2 * s.N);
    if (s.precision == NOSH_PREC_FP64) {
      s.amg->presmooth<double>(dx, o.dev);
    } else {
      nosh::launch_f64_to_f32(dx, s.d_inf.p, 2 * s.N, s.stream);
      s.amg->presmooth<float>(s.d_inf.p, s.d_outf.p);
      nosh::launch_f32_to_f64(s.d_outf.p, o.dev, 2 * s.N, s.stream);
    }
    o.finish(s);
  });
}

int nosh_keo_regularized_operator_apply(nosh_nls nls, const double *x, double *y) {
  return guarded([&] {
    auto &s = NC(nls);
    require(s.reg_ready, "preconditioner not built: call nosh_keo_regularized_rebuild");
    const double *dx = stage_in(s, x, s.d_in, 2 * s.N);
    OutVec o(s, y, s.d_out, 2 * s.N);
    s.reg_apply<double>(dx, o.dev);
    o.finish(s);
  });
}

// --------------------------------------------------------------- solvers
void nosh_newton_default_options(nosh_newton_options *opt) {
  if (!opt) return;
  opt->tol = 1e-10;
  opt->max_newton = 20;
  opt->forcing = 0.0;
  opt->max_krylov = 1000;
  opt->precision = NOSH_PREC_MIXED;
  opt->verbose = 0;
  opt->refine = 0.0;
  opt->phase_fix = 0;
}

int nosh_newton_solve(nosh_nls nls, double *x, const double *p, const nosh_newton_options *opt,
                      nosh_newton_stats *stats) {
  nosh_newton_stats st{};
  int rc = guarded([&] {
    auto &s = NC(nls);
    double g, mu;
    read_params(p, g, mu);
    nosh_newton_options o;
    nosh_newton_default_options(&o);
    if (opt) o = *opt;
    require(o.tol > 0 && o.max_newton >= 0 && o.max_krylov > 0 && o.refine >= 0 && o.refine <= o.tol,
            "bad solver options");
    require(x != nullptr, "null state");
    nosh::newton_solve(s, x, g, mu, o, st);
  });
  if (rc == NOSH_OK) rc = st.status;
  if (stats) *stats = st;
  return rc;
}

int nosh_continuation_step(nosh_nls nls, double *x, double *x_prev, const double *p_new,
                           double mu_cur, double mu_prev, int predictor,
                           const nosh_newton_options *opt, nosh_newton_stats *stats) {
  nosh_newton_stats st{};
  int rc = guarded([&] {
    auto &s = NC(nls);
    double g, mu;
    read_params(p_new, g, mu);
    require(predictor >= NOSH_PREDICT_NONE && predictor <= NOSH_PREDICT_TANGENT, "unknown predictor");
    require(x != nullptr, "null state");
    require(predictor != NOSH_PREDICT_SECANT || x_prev != nullptr, "secant predictor needs x_prev");
    nosh_newton_options o;
    nosh_newton_default_options(&o);
    if (opt) o = *opt;
    require(o.tol > 0 && o.max_newton >= 0 && o.max_krylov > 0 && o.refine >= 0 && o.refine <= o.tol,
            "bad solver options");
    nosh::continuation_step(s, x, x_prev, g, mu, mu_cur, mu_prev, predictor, o, st);
  });
  if (rc == NOSH_OK) rc = st.status;
  if (stats) *stats = st;
  return rc;
}

int nosh_continuation_create(nosh_nls nls, const double *x0, double mu0, nosh_continuation *out) {
  return guarded([&] {
    auto &s = N(nls);
    require(out != nullptr && x0 != nullptr, "null argument");
    require(s.sys_off.empty(), "continuation needs a single-system handle");
    *out = nullptr;
    auto *h = new nosh_continuation_s{nullptr};
    try {
      h->impl = new nosh::ContinuationImpl(s, x0, mu0);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}

int nosh_continuation_destroy(nosh_continuation c) {
  return guarded([&] {
    if (!c) return;
    delete c->impl;
    delete c;
  });
}

int nosh_continuation_advance(nosh_continuation c, double mu_new, int predictor,
                              const nosh_newton_options *opt, nosh_newton_stats *stats) {
  nosh_newton_stats st{};
  int rc = guarded([&] {
    require(c && c->impl, "null continuation handle");
    nosh_newton_options o;
    nosh_newton_default_options(&o);
    if (opt) o = *opt;
    require(o.tol > 0 && o.max_newton >= 0 && o.max_krylov > 0 && o.refine >= 0 && o.refine <= o.tol,
            "bad solver options");
    if (c->impl->s.index_checks) c->impl->s.check_indices();
    c->impl->advance(mu_new, predictor, o, st);
  });
  if (rc == NOSH_OK) rc = st.status;
  if (stats) *stats = st;
  return rc;
}

int nosh_continuation_advance_arclength(nosh_continuation c, double ds, int predictor, double theta,
                                        const nosh_newton_options *opt, nosh_newton_stats *stats) {
  nosh_newton_stats st{};
  int rc = guarded([&] {
    require(c && c->impl, "null continuation handle");
    nosh_newton_options o;
    nosh_newton_default_options(&o);
    if (opt) o = *opt;
    require(o.tol > 0 && o.max_newton >= 0 && o.max_krylov > 0 && o.refine >= 0 && o.refine <= o.tol,
            "bad solver options");
    if (c->impl->s.index_checks) c->impl->s.check_indices();
    c->impl->advance_arclength(ds, predictor, theta, o, st);
  });
  if (rc == NOSH_OK) rc = st.status;
  if (stats) *stats = st;
  return rc;
}

int nosh_continuation_tangent(nosh_continuation c, double *tau_mu, double *theta) {
  return guarded([&] {
    require(c && c->impl, "null continuation handle");
    if (tau_mu) *tau_mu = c->impl->tau_mu;
    if (theta) *theta = c->impl->theta;
  });
}

int nosh_continuation_state(nosh_continuation c, double *x, double *mu) {
  return guarded([&] {
    require(c && c->impl, "null continuation handle");
    auto &C = *c->impl;
    if (x) {
      NOSH_CUDA(cudaMemcpyAsync(x, C.slot(0), 2 * C.s.N * sizeof(double), cudaMemcpyDefault, C.s.stream));
      C.s.sync();
    }
    if (mu) *mu = C.mu_of(0);
  });
}

int nosh_continuation_learning(nosh_continuation c, int train_steps, int iters_per_step, double learning_rate) {
  return guarded([&] {
    require(c && c->impl, "null continuation handle");
    require(train_steps >= 0 && iters_per_step >= 0 && learning_rate >= 0, "bad learning settings");
    c->impl->enable_learning(train_steps, iters_per_step, learning_rate);
  });
}

int nosh_continuation_inference_period(nosh_continuation c, int period) {
  return guarded([&] {
    require(c && c->impl, "null continuation handle");
    require(period >= 1, "the inference period must be >= 1");
    c->impl->infer_period = period;
    c->impl->infer_count = 0;
  });
}

int nosh_continuation_predictor_residuals(nosh_continuation c, double mu_new, double *residuals) {
  return guarded([&] {
    require(c && c->impl, "null continuation handle");
    require(residuals != nullptr, "null output");
    c->impl->predictor_residuals(mu_new, residuals);
  });
}

int nosh_continuation_last_prediction(nosh_continuation c, int *used, double *f_learned, double *f_secant,
                                      double *train_loss, double *coef) {
  return guarded([&] {
    require(c && c->impl, "null continuation handle");
    auto &C = *c->impl;
    if (used) *used = C.last_used;
    if (f_learned) *f_learned = C.f_learned;
    if (f_secant) *f_secant = C.f_secant;
    if (train_loss) *train_loss = C.train_loss;
    if (coef) *coef = C.coef;
  });
}

int nosh_mpnn_create(nosh_nls nls, nosh_mpnn *out) {
  return guarded([&] {
    auto &s = N(nls);
    require(out != nullptr, "null argument");
    *out = nullptr;
    auto *h = new nosh_mpnn_s{nullptr};
    try {
      h->impl = new nosh::Mpnn(s);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}

int nosh_mpnn_destroy(nosh_mpnn net) {
  return guarded([&] {
    if (!net) return;
    delete net->impl;
    delete net;
  });
}

int nosh_mpnn_num_params(nosh_mpnn net, int64_t *n) {
  return guarded([&] {
    require(net && net->impl && n, "null argument");
    *n = net->impl->num_params();
  });
}

int nosh_mpnn_params(nosh_mpnn net, float *get, const float *set) {
  return guarded([&] {
    require(net && net->impl, "null mpnn handle");
    if (get) net->impl->get_params(get);
    if (set) net->impl->set_params(set);
  });
}

int nosh_mpnn_edge_features(nosh_mpnn net, float *ef) {
  return guarded([&] {
    require(net && net->impl && ef, "null argument");
    net->impl->get_edge_features(ef);
  });
}

int nosh_mpnn_forward(nosh_mpnn net, const float *X, double *w) {
  return guarded([&] {
    require(net && net->impl && X && w, "null argument");
    net->impl->forward_features(X, w);
  });
}

int nosh_mpnn_loss_grad(nosh_mpnn net, const float *X, const double *gram, double *loss, float *grad) {
  return guarded([&] {
    require(net && net->impl && X && gram && grad, "null argument");
    const double l = net->impl->loss_and_grad(X, gram, grad);
    if (loss) *loss = l;
  });
}

int nosh_nls_profile_enable(nosh_nls nls, int enable) {
  return guarded([&] {
    auto &s = N(nls);
    for (auto &t : s.timers) t.on = enable != 0;
  });
}

int nosh_nls_profile_read(nosh_nls nls, int kernel, int64_t *launches, double *total_ms,
                          double *bytes) {
  return guarded([&] {
    auto &s = N(nls);
    require(kernel >= NOSH_KERNEL_JACOBIAN && kernel <= NOSH_KERNEL_ALL, "unknown kernel class");
    int64_t n = 0;
    double ms = 0.0, b = 0.0;
    if (kernel == NOSH_KERNEL_ALL) {
      n = s.launch_count;
      s.launch_count = 0;
    } else {
      s.timers[kernel].read(n, ms, b);
    }
    if (launches) *launches = n;
    if (total_ms) *total_ms = ms;
    if (bytes) *bytes = b;
  });
}

}  // extern "C"
