// nosh_gb300.hpp -- C++ API over the C ABI, with the class and method names
// of nschloe/nosh's hot path so that code written against the reference's
// classes ports by changing types, not calls.
//
//   nosh::mesh                          (src/mesh.hpp)
//   nosh::vector_field::explicit_values (src/vector_field_explicit_values.hpp)
//   nosh::scalar_field::constant        (src/scalar_field_constant.hpp)
//   nosh::parameter_matrix::keo/DkeoDP  (src/parameter_matrix_{keo,dkeo_dp}.hpp)
//   nosh::jacobian_operator             (src/jacobian_operator.hpp)
//   nosh::keo_regularized               (src/keo_regularized.hpp)
//   nosh::model_evaluator::nls          (src/model_evaluator_nls.hpp)
//   nosh::continuation                  (the LOCA stepper of executables/
//                                        nosh-cont and src/observer.cpp)
//   nosh::io                            (mesh / state files, .vtu for .h5m)
//   nosh::eig                           (stability eigenvalues, nosh-eig)
//
// Trilinos types are replaced by std::vector<double> (interleaved complex
// vectors of length 2N, multivectors as a vector of columns) and parameter
// maps by std::map<std::string, double>, as the reference's own set_parameters
// takes.  Errors surface as nosh::error exceptions carrying the C ABI status
// (the reference throws std::logic_error via TEUCHOS_TEST_FOR_EXCEPT_MSG).
#ifndef NOSH_GB300_HPP
#define NOSH_GB300_HPP

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "nosh_gb300.h"

namespace nosh {

struct error : std::runtime_error {
  int code;
  error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

inline void check(int rc) {
  if (rc != NOSH_OK) throw error(rc, nosh_last_error());
}

using vec = std::vector<double>;
using edge = std::tuple<int, int>;

// ------------------------------------------------------------------ mesh
class mesh {
 public:
  struct edge_data {
    double length;
    double covolume;
  };

  // coords: 3 per vertex; cells: verts_per_cell (3 or 4) vertex ids per cell
  mesh(const std::vector<double> &coords, const std::vector<int32_t> &cells, int verts_per_cell) {
    const int64_t N = (int64_t)coords.size() / 3, T = (int64_t)cells.size() / verts_per_cell;
    check(nosh_mesh_create(coords.data(), N, cells.data(), T, verts_per_cell, &h_));
    check(nosh_mesh_sizes(h_, &n_, &e_, &t_, &nnz_));
  }
  ~mesh() { nosh_mesh_destroy(h_); }
  mesh(const mesh &) = delete;
  mesh &operator=(const mesh &) = delete;

  nosh_mesh handle() const { return h_; }
  int64_t num_vertices() const { return n_; }
  int64_t num_edges() const { return e_; }

  std::vector<edge> my_edges() const {
    std::vector<int32_t> e(2 * e_);
    check(nosh_mesh_edges(h_, e.data()));
    std::vector<edge> out(e_);
    for (int64_t k = 0; k < e_; k++) out[k] = edge(e[2 * k], e[2 * k + 1]);
    return out;
  }
  std::vector<std::array<int, 4>> edge_gids_complex() const {
    std::vector<std::array<int, 4>> out(e_);
    check(nosh_mesh_edge_gids_complex(h_, reinterpret_cast<int32_t *>(out.data())));
    return out;
  }
  std::vector<edge_data> get_edge_data() const {
    vec len(e_), cov(e_);
    check(nosh_mesh_edge_data(h_, len.data(), cov.data()));
    std::vector<edge_data> out(e_);
    for (int64_t k = 0; k < e_; k++) out[k] = {len[k], cov[k]};
    return out;
  }
  vec control_volumes() const {
    vec cv(n_);
    check(nosh_mesh_control_volumes(h_, cv.data()));
    return cv;
  }
  // complex graph: row pointers and sorted columns (diagonal included)
  std::pair<std::vector<int32_t>, std::vector<int32_t>> build_complex_graph() const {
    std::vector<int32_t> rp(n_ + 1), ci(nnz_);
    check(nosh_mesh_complex_graph(h_, rp.data(), ci.data()));
    return {rp, ci};
  }

 private:
  nosh_mesh h_ = nullptr;
  int64_t n_ = 0, e_ = 0, t_ = 0, nnz_ = 0;
};

// ---------------------------------------------------------------- fields
namespace vector_field {
// A sampled per vertex (3 per vertex); edge projections scaled by "mu"
class explicit_values {
 public:
  explicit_values(const mesh &m, vec A, double mu) : A_(std::move(A)), mu_(mu) {
    if ((int64_t)A_.size() != 3 * m.num_vertices()) throw error(NOSH_ERR_INVALID, "A must hold 3 values per vertex");
  }
  std::map<std::string, double> get_scalar_parameters() const { return {{"mu", mu_}}; }
  const vec &values() const { return A_; }

 private:
  vec A_;
  double mu_;
};
}  // namespace vector_field

namespace scalar_field {
class base {
 public:
  virtual ~base() = default;
  virtual vec get_v(const std::map<std::string, double> &params) const = 0;
};
// c (+ the named parameter, when given), src/scalar_field_constant.cpp:45-58
class constant : public base {
 public:
  constant(const mesh &m, double c, const std::string &param_name = "", double param_init = 0.0)
      : n_(m.num_vertices()), c_(c), name_(param_name), init_(param_init) {}
  vec get_v(const std::map<std::string, double> &params) const override {
    double v = c_;
    if (!name_.empty()) {
      auto it = params.find(name_);
      v += it != params.end() ? it->second : init_;
    }
    return vec(n_, v);
  }

 private:
  int64_t n_;
  double c_;
  std::string name_;
  double init_;
};
class explicit_values : public base {
 public:
  explicit explicit_values(vec v) : v_(std::move(v)) {}
  vec get_v(const std::map<std::string, double> &) const override { return v_; }

 private:
  vec v_;
};
}  // namespace scalar_field

namespace model_evaluator {
class nls;
}

inline vec params_vector(const std::map<std::string, double> &p, const std::map<std::string, double> &nominal) {
  std::map<std::string, double> all = nominal;
  for (const auto &kv : p) all[kv.first] = kv.second;
  return {all.at("g"), all.at("mu")};
}

// ---------------------------------------------------- parameter matrices
namespace parameter_matrix {
class keo {
 public:
  keo(nosh_nls h, const std::map<std::string, double> *nominal, bool dkeo) : h_(h), nom_(nominal), d_(dkeo) {}
  // parameter_object::set_parameters -> refill_
  void set_parameters(const std::map<std::string, double> &params,
                      const std::map<std::string, std::shared_ptr<const vec>> & = {}) {
    const vec p = params_vector(params, *nom_);
    check(d_ ? nosh_dkeo_set_parameters(h_, p.data()) : nosh_keo_set_parameters(h_, p.data()));
  }
  // Y = K X (Tpetra::CrsMatrix::apply)
  void apply(const vec &x, vec &y) const {
    y.resize(x.size());
    check(d_ ? nosh_dkeo_apply(h_, x.data(), y.data()) : nosh_keo_apply(h_, x.data(), y.data()));
  }
  // complex values in build_complex_graph order (2 doubles per block)
  vec values(size_t nnz_blocks) const {
    vec v(2 * nnz_blocks);
    check(d_ ? nosh_dkeo_values(h_, v.data()) : nosh_keo_values(h_, v.data()));
    return v;
  }

 private:
  nosh_nls h_;
  const std::map<std::string, double> *nom_;
  bool d_;
};
using DkeoDP = keo;
}  // namespace parameter_matrix

// ------------------------------------------------------------ operators
class jacobian_operator {
 public:
  jacobian_operator(nosh_nls h, const std::map<std::string, double> *nominal) : h_(h), nom_(nominal) {}
  void rebuild(const std::map<std::string, double> &params, const vec &current_x) {
    const vec p = params_vector(params, *nom_);
    check(nosh_jacobian_rebuild(h_, p.data(), current_x.data()));
  }
  // Only NO_TRANS, alpha = 1, beta = 0 (src/jacobian_operator.cpp:48-59)
  void apply(const std::vector<vec> &X, std::vector<vec> &Y, int mode = NOSH_NO_TRANS, double alpha = 1.0,
             double beta = 0.0) const {
    Y.resize(X.size());
    for (size_t k = 0; k < X.size(); k++) {
      Y[k].resize(X[k].size());
      check(nosh_jacobian_apply(h_, X[k].data(), Y[k].data(), 1, mode, alpha, beta));
    }
  }

 private:
  nosh_nls h_;
  const std::map<std::string, double> *nom_;
};

class keo_regularized {
 public:
  keo_regularized(nosh_nls h, const std::map<std::string, double> *nominal) : h_(h), nom_(nominal) {}
  void rebuild(const std::map<std::string, double> &params, const vec &x) {
    const vec p = params_vector(params, *nom_);
    check(nosh_keo_regularized_rebuild(h_, p.data(), x.data()));
  }
  // one V-cycle (num_cycles_ == 1, src/keo_regularized.cpp:106-108)
  void apply(const std::vector<vec> &X, std::vector<vec> &Y, int mode = NOSH_NO_TRANS, double alpha = 1.0,
             double beta = 0.0) const {
    Y.resize(X.size());
    for (size_t k = 0; k < X.size(); k++) {
      Y[k].resize(X[k].size());
      check(nosh_keo_regularized_apply(h_, X[k].data(), Y[k].data(), 1, mode, alpha, beta));
    }
  }

 private:
  nosh_nls h_;
  const std::map<std::string, double> *nom_;
};

// ------------------------------------------------------- model evaluator
namespace model_evaluator {
class nls {
 public:
  nls(const std::shared_ptr<const mesh> &m, const std::shared_ptr<vector_field::explicit_values> &mvp,
      const std::shared_ptr<const scalar_field::base> &scalar_potential, double g,
      const std::shared_ptr<const scalar_field::base> &thickness, const std::shared_ptr<const vec> &initial_x,
      const std::string &deriv_parameter)
      : mesh_(m), x0_(initial_x) {
    nominal_ = mvp->get_scalar_parameters();
    nominal_["g"] = g;
    const vec V = scalar_potential->get_v(nominal_), t = thickness->get_v(nominal_);
    check(nosh_nls_create(m->handle(), mvp->values().data(), nominal_.at("mu"), V.data(), g, t.data(),
                          deriv_parameter.c_str(), &h_));
    keo_.reset(new parameter_matrix::keo(h_, &nominal_, false));
    dkeo_.reset(new parameter_matrix::DkeoDP(h_, &nominal_, true));
  }
  ~nls() { nosh_nls_destroy(h_); }
  nls(const nls &) = delete;
  nls &operator=(const nls &) = delete;

  nosh_nls handle() const { return h_; }
  void set_precision(int p) { check(nosh_nls_set_precision(h_, p)); }
  // device-side validation of every graph index before each launch
  void set_index_checks(bool on) { check(nosh_nls_set_index_checks(h_, on ? 1 : 0)); }
  // the fraction of the tolerance a Newton step's forcing term aims at
  void set_forcing_aim(double aim) { check(nosh_nls_set_forcing_aim(h_, aim)); }
  // programmatic dependent launch of the MINRES / V-cycle kernels (on by
  // default; results are bitwise the same either way)
  void set_launch_overlap(bool on) { check(nosh_nls_set_launch_overlap(h_, on ? 1 : 0)); }
  // SpMV schedule of every level: NOSH_SPMV_AUTO (timed once per matrix),
  // _STAGED or _WARP
  void set_spmv_schedule(int schedule) { check(nosh_nls_set_spmv_schedule(h_, schedule)); }
  // the preconditioner's options (MueLu parameter list of
  // src/keo_regularized.cpp:296-315); the next rebuild builds a new hierarchy
  void set_amg_options(int max_levels, int coarse_size, int smooth_degree, int reuse_period,
                       double strength_threshold, double cheb_ratio) {
    check(nosh_nls_set_amg_options(h_, max_levels, coarse_size, smooth_degree, reuse_period, strength_threshold,
                                   cheb_ratio));
  }
  int precision() const {
    int p = 0;
    check(nosh_nls_get_precision(h_, &p));
    return p;
  }
  // sorted parameter names (src/model_evaluator_nls.cpp:196-205)
  std::vector<std::string> get_p_names() const {
    int n = 0;
    check(nosh_nls_num_params(h_, &n));
    std::vector<std::string> out;
    char buf[32];
    for (int k = 0; k < n; k++) {
      check(nosh_nls_param_name(h_, k, buf, sizeof(buf)));
      out.emplace_back(buf);
    }
    return out;
  }
  const std::map<std::string, double> &nominal_parameters() const { return nominal_; }
  std::shared_ptr<parameter_matrix::keo> keo() const { return keo_; }
  std::shared_ptr<parameter_matrix::DkeoDP> dkeo_dp() const { return dkeo_; }

  // evalModel pieces
  void compute_f(const vec &x, const std::map<std::string, double> &params, vec &f) const {
    const vec p = params_vector(params, nominal_);
    f.resize(x.size());
    check(nosh_nls_compute_f(h_, x.data(), p.data(), f.data()));
  }
  // DfDp by column (one column per sorted parameter name)
  std::vector<vec> compute_dfdp(const vec &x, const std::map<std::string, double> &params) const {
    const vec p = params_vector(params, nominal_);
    vec all(2 * x.size());
    check(nosh_nls_compute_dfdp(h_, x.data(), p.data(), all.data()));
    return {vec(all.begin(), all.begin() + x.size()), vec(all.begin() + x.size(), all.end())};
  }
  std::shared_ptr<jacobian_operator> create_W_op() const {
    return std::make_shared<jacobian_operator>(h_, &nominal_);
  }
  std::shared_ptr<keo_regularized> create_W_prec() const {
    return std::make_shared<keo_regularized>(h_, &nominal_);
  }
  double gibbs_energy(const vec &psi) const {
    double e = 0.0;
    check(nosh_nls_gibbs_energy(h_, psi.data(), &e));
    return e;
  }
  double inner_product(const vec &phi, const vec &psi) const {
    double r = 0.0;
    check(nosh_nls_inner_product(h_, phi.data(), psi.data(), &r));
    return r;
  }
  // Newton solve to ||F|| <= tol (NOX "Line Search Based", full step)
  nosh_newton_stats newton(vec &x, const std::map<std::string, double> &params, double tol = 1e-10) const {
    const vec p = params_vector(params, nominal_);
    nosh_newton_options o;
    nosh_newton_default_options(&o);
    o.tol = tol;
    nosh_newton_stats st;
    const int rc = nosh_newton_solve(h_, x.data(), p.data(), &o, &st);
    if (rc != NOSH_OK && rc != NOSH_ERR_NOT_CONVERGED) check(rc);
    return st;
  }

 private:
  std::shared_ptr<const mesh> mesh_;
  std::shared_ptr<const vec> x0_;
  std::map<std::string, double> nominal_;
  nosh_nls h_ = nullptr;
  std::shared_ptr<parameter_matrix::keo> keo_;
  std::shared_ptr<parameter_matrix::DkeoDP> dkeo_;
};
}  // namespace model_evaluator

// ---------------------------------------------------------- continuation
// The LOCA stepper loop of the reference's driver (executables/nosh-cont/
// nosh-cont.cpp:226-345; parameters of examples/conf.xml:35-75) over the
// device-resident continuation handle, and the continuation statistics
// observer (src/observer.cpp:136-159, written in the layout of
// src/csv_writer.cpp).  LOCA itself is a Trilinos package; the step-size
// rule restated here: after a successful step of n nonlinear iterations
// ds *= 1 + aggressiveness ((n_max - n) / (n_max - 1))^2, clipped to the
// maximum step; after a failed one ds /= 2, and the run fails below the
// minimum step.
namespace continuation {

// nosh_continuation: the last converged states stay on the GPU
class run {
 public:
  run(const model_evaluator::nls &model, const vec &x0, double mu0) : n_(x0.size()) {
    check(nosh_continuation_create(model.handle(), x0.data(), mu0, &h_));
  }
  ~run() { nosh_continuation_destroy(h_); }
  run(const run &) = delete;
  run &operator=(const run &) = delete;

  double mu() const {
    double m = 0.0;
    check(nosh_continuation_state(h_, nullptr, &m));
    return m;
  }
  void state(vec &x, double &m) const {
    x.resize(n_);
    check(nosh_continuation_state(h_, x.data(), &m));
  }
  // a natural step to mu_new; a step that did not converge (or hit NaN or a
  // Krylov breakdown) reports it in status and leaves the state unchanged
  nosh_newton_stats advance(double mu_new, int predictor, const nosh_newton_options &opt) {
    nosh_newton_stats st{};
    return finish(nosh_continuation_advance(h_, mu_new, predictor, &opt, &st), st);
  }
  nosh_newton_stats advance_arclength(double ds, int predictor, double theta, const nosh_newton_options &opt) {
    nosh_newton_stats st{};
    return finish(nosh_continuation_advance_arclength(h_, ds, predictor, theta, &opt, &st), st);
  }
  double tangent_mu() const {
    double t = 0.0, th = 0.0;
    check(nosh_continuation_tangent(h_, &t, &th));
    return t;
  }
  // the learned predictor (NOSH_PREDICT_LEARNED): online training window,
  // then overlapped inference every `period`-th learned step
  void learning(int train_steps, int iters_per_step, double learning_rate) {
    check(nosh_continuation_learning(h_, train_steps, iters_per_step, learning_rate));
  }
  void inference_period(int period) { check(nosh_continuation_inference_period(h_, period)); }
  // ||F|| at mu_new of the secant, quadratic, cubic and learned predictions
  // from the current history (NaN where one is not available)
  std::array<double, 4> predictor_residuals(double mu_new) const {
    std::array<double, 4> r{};
    check(nosh_continuation_predictor_residuals(h_, mu_new, r.data()));
    return r;
  }

 private:
  static nosh_newton_stats finish(int rc, nosh_newton_stats st) {
    if (rc == NOSH_ERR_NOT_CONVERGED || rc == NOSH_ERR_NAN || rc == NOSH_ERR_BREAKDOWN) {
      st.status = rc;
      return st;
    }
    check(rc);
    return st;
  }
  nosh_continuation h_ = nullptr;
  size_t n_;
};

// The statistics table of the reference's csv_writer: "# " and the labels,
// doubles in %.15e in columns 22 wide, integers in columns as wide as their
// label (at least 5), three spaces between columns, rows indented by two.
class csv_writer {
 public:
  explicit csv_writer(std::FILE *f) : f_(f) {}
  struct cell {
    std::string label;
    bool integer;
    double value;
  };
  void write_header(const std::vector<cell> &row) const {
    std::fputs("# ", f_);
    line(row, true);
  }
  void write_row(const std::vector<cell> &row) const {
    std::fputs("  ", f_);
    line(row, false);
  }

 private:
  void line(const std::vector<cell> &row, bool header) const {
    for (size_t k = 0; k < row.size(); k++) {
      if (k) std::fputs("   ", f_);
      const cell &c = row[k];
      const int w = c.integer ? (int)std::max<size_t>(5, c.label.size()) : 22;
      if (header)
        std::fprintf(f_, "%-*s", w, c.label.c_str());
      else if (c.integer)
        std::fprintf(f_, "%-*lld", w, (long long)c.value);
      else
        std::fprintf(f_, "%-*.15e", w, c.value);
    }
    std::fputs("\n", f_);
    std::fflush(f_);
  }
  std::FILE *f_;
};

// Per converged state: step, the parameter, the Gibbs energy and
// sqrt(<psi, psi>) (src/model_evaluator_base.hpp norm).
class statistics_observer {
 public:
  statistics_observer(const model_evaluator::nls &model, std::FILE *f, const std::string &param = "mu")
      : model_(model), w_(f), param_(param) {}
  void operator()(int index, const vec &x, double m) const {
    const double ip = model_.inner_product(x, x);
    const std::vector<csv_writer::cell> row = {{"(0) step", true, (double)index},
                                               {"(1) " + param_, false, m},
                                               {"(2) Gibbs energy", false, model_.gibbs_energy(x)},
                                               {"(2) ||x||_2 scaled", false, std::sqrt(ip > 0 ? ip : 0.0)}};
    if (index == 0) w_.write_header(row);
    w_.write_row(row);
  }

 private:
  const model_evaluator::nls &model_;
  csv_writer w_;
  std::string param_;
};

struct stepper_parameters {
  bool arc_length = true;                 // "Continuation Method": Arc Length / Natural
  int predictor = NOSH_PREDICT_TANGENT;   // "Predictor" Method
  double initial_step = 1e-3, max_step = 1e-2, min_step = 1e-7;  // "Step Size"
  double aggressiveness = 2.0;
  bool adaptive = true;                   // "Adaptive" or "Constant"
  int max_steps = 1000;                   // "Max Steps"
  double max_value = 100.0, min_value = -100.0;
  int max_nonlinear_iters = 15;
  double theta = 1.0;                     // arclength parameter scale
};

struct step_record {
  int step;
  double mu, ds;
  int newton_iters, krylov_iters;
};

struct stepper_result {
  bool failed = false;  // the step size fell below the minimum
  int steps = 0, failed_steps = 0;
  std::vector<step_record> records;
};

// The stepper loop, generic over the run (any type with mu(), state(x, mu),
// advance(mu, predictor, opt), advance_arclength(ds, predictor, theta, opt)
// and tangent_mu()) and the observer (called as obs(index, x, mu)).
template <class Run, class Observer>
stepper_result step(Run &r, const stepper_parameters &p, nosh_newton_options opt, Observer &&obs) {
  if (!(p.min_step > 0 && p.min_step <= std::fabs(p.initial_step) && std::fabs(p.initial_step) <= p.max_step))
    throw error(NOSH_ERR_INVALID, "need 0 < min step <= |initial step| <= max step");
  if (p.max_nonlinear_iters < 2) throw error(NOSH_ERR_INVALID, "max nonlinear iterations must be at least 2");
  if (p.arc_length && p.predictor != NOSH_PREDICT_TANGENT && p.predictor != NOSH_PREDICT_SECANT)
    throw error(NOSH_ERR_INVALID, "arclength steps predict TANGENT or SECANT");
  opt.max_newton = p.max_nonlinear_iters;
  stepper_result out;
  vec x;
  double m = 0.0;
  r.state(x, m);
  obs(0, x, m);
  out.records.push_back({0, m, 0.0, 0, 0});
  double ds = p.initial_step;
  auto clip = [&](double d, double mu, double dmu_ds, bool &last) {
    last = false;
    if (!(std::isfinite(dmu_ds)) || dmu_ds == 0.0) return d;
    const double target = mu + d * dmu_ds;
    for (double bound : {p.max_value, p.min_value})
      if ((target - bound) * (mu - bound) < 0.0 || target == bound) {
        last = true;
        return (bound - mu) / dmu_ds;
      }
    return d;
  };
  while (out.steps < p.max_steps) {
    const double mu = r.mu();
    if (mu >= p.max_value || mu <= p.min_value) break;
    bool last = false;
    double d;
    nosh_newton_stats st;
    if (!p.arc_length) {
      d = clip(ds, mu, 1.0, last);
      st = r.advance(mu + d, p.predictor, opt);
    } else {
      d = clip(ds, mu, out.steps > 0 ? r.tangent_mu() : std::nan(""), last);
      st = r.advance_arclength(d, p.predictor, p.theta, opt);
    }
    if (st.status != NOSH_OK) {
      out.failed_steps++;
      ds = 0.5 * d;
      if (std::fabs(ds) < p.min_step) {
        out.failed = true;
        break;
      }
      continue;
    }
    out.steps++;
    r.state(x, m);
    obs(out.steps, x, m);
    out.records.push_back({out.steps, m, d, st.newton_iters, st.krylov_iters});
    if (last) break;
    if (p.adaptive) {
      const double ratio = std::max(0.0, (double)(p.max_nonlinear_iters - st.newton_iters) /
                                              (double)(p.max_nonlinear_iters - 1));
      ds = d * (1.0 + p.aggressiveness * ratio * ratio);
      ds = std::copysign(std::min(std::fabs(ds), p.max_step), ds);
    } else {
      ds = d;
    }
    // from the second arclength step on the tangent follows the last secant
    if (p.arc_length) ds = std::fabs(ds);
    if (std::fabs(ds) < p.min_step) ds = std::copysign(p.min_step, ds);
  }
  return out;
}

}  // namespace continuation

// ------------------------------------------------------- eigenvalues
// The stability of a state: the k smallest eigenvalues of the real-symmetric
// Jacobian, the role of the reference's nosh-eig (executables/nosh-eig/
// nosh-eig.cpp, Anasazi on the Jacobian operator).  LOBPCG (Knyazev 2001)
// in the Hetmaniuk-Lehoucq basis form: J applies in FP64 through the C ABI,
// one AMG V-cycle of the regularised KEO preconditions, the U(1) gauge mode
// i psi (J(i psi) = i F) is deflated, guard vectors keep a cluster at the
// k-th eigenvalue from slowing the iteration, and the W and P blocks are
// scaled to unit rows before each orthonormalisation.  Block algebra on the
// host; the projected problem by cyclic Jacobi rotations.
namespace eig {

struct result {
  std::vector<double> values;  // ascending
  std::vector<vec> vectors;    // unit, orthogonal to i psi
  int iterations = 0;
};

// The k smallest eigenvalues of the FP64 Jacobian J(psi, params) and their
// eigenvectors, the stability test of a state (the reference's nosh-eig,
// executables/nosh-eig/nosh-eig.cpp:57-, hands J to Anasazi).  LOBPCG runs
// inside the library on the GPU (nosh_eig_lowest): the block algebra is the
// library's own kernels, the preconditioner one AMG V-cycle of the
// regularised KEO, and the gauge mode i psi is deflated.
inline result lowest_eigenpairs(model_evaluator::nls &model, const vec &psi,
                                const std::map<std::string, double> &params, int k, double tol = 1e-8,
                                int maxit = 500, unsigned seed = 1) {
  const size_t n = psi.size();
  const int guard = std::max(2, k), mb = k + guard;
  if (k < 1 || 3 * mb > 64 || (size_t)(3 * mb + 1) >= n)
    throw error(NOSH_ERR_INVALID, "need 1 <= k, 3 (k + guard) <= 64 and 3 (k + guard) + 1 < 2N");
  const vec p = params_vector(params, model.nominal_parameters());
  result out;
  out.values.resize(k);
  std::vector<double> flat((size_t)k * n);
  int its = 0;
  check(nosh_eig_lowest(model.handle(), psi.data(), p.data(), k, tol, maxit, guard, 1, seed, out.values.data(),
                        flat.data(), &its));
  out.iterations = its;
  out.vectors.resize(k);
  for (int j = 0; j < k; j++) out.vectors[j].assign(flat.begin() + (size_t)j * n, flat.begin() + (size_t)(j + 1) * n);
  return out;
}

}  // namespace eig

// ------------------------------------------------------------------ files
// Mesh and state files as VTK XML unstructured grids (.vtu), the format of
// nosh_gb300/io.py: the reference reads psi, A and V vertex tags through
// MOAB (src/mesh_reader.cpp:20-162) and writes one state per continuation
// step (src/continuation_data_saver.hpp:26-50); MOAB's .h5m needs HDF5,
// which the library does not depend on.  Arrays are base64 with UInt64 size
// headers, little endian, and round-trip bit for bit; the reader also takes
// ASCII arrays.
namespace io {

struct array {
  std::string name;
  int components = 1;
  std::vector<double> values;  // tuples of `components`
};

struct grid {
  std::vector<double> coords;  // 3 per point
  std::vector<int32_t> cells;  // nvc per cell
  int nvc = 0;                 // 3: triangles, 4: tetrahedra
  std::vector<array> point_data;
  std::vector<std::pair<std::string, double>> field_data;
  const array *find(const std::string &name) const {
    for (const array &a : point_data)
      if (a.name == name) return &a;
    return nullptr;
  }
};

namespace detail {
inline std::string b64(const unsigned char *p, size_t n) {
  static const char *t = "ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789+/";
  std::string o;
  o.reserve((n + 2) / 3 * 4);
  for (size_t i = 0; i < n; i += 3) {
    const unsigned v = (unsigned)p[i] << 16 | (i + 1 < n ? (unsigned)p[i + 1] << 8 : 0u) | (i + 2 < n ? p[i + 2] : 0u);
    o += t[v >> 18 & 63];
    o += t[v >> 12 & 63];
    o += i + 1 < n ? t[v >> 6 & 63] : '=';
    o += i + 2 < n ? t[v & 63] : '=';
  }
  return o;
}
inline std::vector<unsigned char> unb64(const std::string &s) {
  std::vector<unsigned char> o;
  unsigned v = 0;
  int bits = 0;
  for (char ch : s) {
    int d;
    if (ch >= 'A' && ch <= 'Z') d = ch - 'A';
    else if (ch >= 'a' && ch <= 'z') d = ch - 'a' + 26;
    else if (ch >= '0' && ch <= '9') d = ch - '0' + 52;
    else if (ch == '+') d = 62;
    else if (ch == '/') d = 63;
    else continue;  // padding and whitespace
    v = v << 6 | (unsigned)d;
    bits += 6;
    if (bits >= 8) {
      bits -= 8;
      o.push_back((unsigned char)(v >> bits & 255u));
    }
  }
  return o;
}
// host byte order is little endian on every supported platform (x86-64,
// aarch64)
template <class T>
inline std::string encode(const std::vector<T> &v) {
  const uint64_t n = v.size() * sizeof(T);
  std::vector<unsigned char> raw(8 + n);
  std::memcpy(raw.data(), &n, 8);
  if (n) std::memcpy(raw.data() + 8, v.data(), n);
  return b64(raw.data(), raw.size());
}
inline std::string attr(const std::string &tag, const std::string &key) {
  const std::string k = " " + key + "=\"";
  const size_t a = tag.find(k);
  if (a == std::string::npos) return "";
  const size_t b = tag.find('"', a + k.size());
  return tag.substr(a + k.size(), b - a - k.size());
}
inline size_t type_size(const std::string &t) {
  if (t == "Float64" || t == "Int64" || t == "UInt64") return 8;
  if (t == "Float32" || t == "Int32" || t == "UInt32") return 4;
  if (t == "UInt8" || t == "Int8") return 1;
  throw error(NOSH_ERR_INVALID, "unsupported DataArray type " + t);
}
inline double element(const unsigned char *p, const std::string &t) {
  if (t == "Float64") { double v; std::memcpy(&v, p, 8); return v; }
  if (t == "Float32") { float v; std::memcpy(&v, p, 4); return v; }
  if (t == "Int64") { int64_t v; std::memcpy(&v, p, 8); return (double)v; }
  if (t == "UInt64") { uint64_t v; std::memcpy(&v, p, 8); return (double)v; }
  if (t == "Int32") { int32_t v; std::memcpy(&v, p, 4); return v; }
  if (t == "UInt32") { uint32_t v; std::memcpy(&v, p, 4); return v; }
  if (t == "Int8") return (double)(int8_t)*p;
  return (double)*p;
}
inline std::vector<double> values(const std::string &tag, const std::string &body) {
  const std::string type = attr(tag, "type"), fmt = attr(tag, "format");
  std::vector<double> out;
  if (fmt == "binary") {
    const std::vector<unsigned char> raw = unb64(body);
    if (raw.size() < 8) throw error(NOSH_ERR_INVALID, "truncated binary DataArray");
    uint64_t n = 0;
    std::memcpy(&n, raw.data(), 8);
    const size_t es = type_size(type);
    if (raw.size() < 8 + n || n % es) throw error(NOSH_ERR_INVALID, "binary DataArray size mismatch");
    for (uint64_t i = 0; i < n / es; i++) out.push_back(element(raw.data() + 8 + i * es, type));
  } else if (fmt == "ascii" || fmt.empty()) {
    type_size(type);
    const char *c = body.c_str();
    char *end = nullptr;
    for (;;) {
      const double v = std::strtod(c, &end);
      if (end == c) break;
      out.push_back(v);
      c = end;
    }
  } else {
    throw error(NOSH_ERR_INVALID, "unsupported DataArray format " + fmt);
  }
  return out;
}
}  // namespace detail

inline void write_vtu(const std::string &path, const grid &g) {
  if (g.nvc != 3 && g.nvc != 4) throw error(NOSH_ERR_INVALID, "cells must be triangles (3) or tetrahedra (4)");
  const size_t n = g.coords.size() / 3, t = g.cells.size() / (size_t)g.nvc;
  std::FILE *f = std::fopen(path.c_str(), "w");
  if (!f) throw error(NOSH_ERR_INVALID, "cannot write " + path);
  std::fprintf(f, "<?xml version='1.0' encoding='utf-8'?>\n<VTKFile type=\"UnstructuredGrid\" version=\"1.0\" "
                  "byte_order=\"LittleEndian\" header_type=\"UInt64\"><UnstructuredGrid>");
  auto arr = [&](const char *type, const std::string &name, int nc, const std::string &data, long ntuples) {
    std::fprintf(f, "<DataArray type=\"%s\" Name=\"%s\" format=\"binary\"", type, name.c_str());
    if (nc > 1) std::fprintf(f, " NumberOfComponents=\"%d\"", nc);
    if (ntuples >= 0) std::fprintf(f, " NumberOfTuples=\"%ld\"", ntuples);
    std::fprintf(f, ">%s</DataArray>", data.c_str());
  };
  if (!g.field_data.empty()) {
    std::fprintf(f, "<FieldData>");
    for (const auto &kv : g.field_data) arr("Float64", kv.first, 1, detail::encode(std::vector<double>{kv.second}), 1);
    std::fprintf(f, "</FieldData>");
  }
  std::fprintf(f, "<Piece NumberOfPoints=\"%zu\" NumberOfCells=\"%zu\">", n, t);
  if (!g.point_data.empty()) {
    std::fprintf(f, "<PointData>");
    for (const array &a : g.point_data) {
      if (a.values.size() != n * (size_t)a.components) {
        std::fclose(f);
        throw error(NOSH_ERR_INVALID, "point data " + a.name + " does not match the points");
      }
      arr("Float64", a.name, a.components, detail::encode(a.values), -1);
    }
    std::fprintf(f, "</PointData>");
  }
  std::fprintf(f, "<Points>");
  arr("Float64", "Points", 3, detail::encode(g.coords), -1);
  std::fprintf(f, "</Points><Cells>");
  std::vector<int64_t> conn(g.cells.begin(), g.cells.end()), off(t);
  for (size_t k = 0; k < t; k++) off[k] = (int64_t)((k + 1) * (size_t)g.nvc);
  arr("Int64", "connectivity", 1, detail::encode(conn), -1);
  arr("Int64", "offsets", 1, detail::encode(off), -1);
  arr("UInt8", "types", 1, detail::encode(std::vector<uint8_t>(t, g.nvc == 3 ? 5 : 10)), -1);
  std::fprintf(f, "</Cells></Piece></UnstructuredGrid></VTKFile>\n");
  std::fclose(f);
}

inline grid read_vtu(const std::string &path) {
  std::FILE *f = std::fopen(path.c_str(), "rb");
  if (!f) throw error(NOSH_ERR_INVALID, "cannot read " + path);
  std::string doc;
  char buf[1 << 16];
  size_t got;
  while ((got = std::fread(buf, 1, sizeof buf, f)) > 0) doc.append(buf, got);
  std::fclose(f);
  if (doc.find("type=\"UnstructuredGrid\"") == std::string::npos)
    throw error(NOSH_ERR_INVALID, "not a VTK unstructured grid");
  grid g;
  std::vector<double> conn, off, types;
  std::string section;
  for (size_t pos = 0;;) {
    const size_t lt = doc.find('<', pos);
    if (lt == std::string::npos) break;
    const size_t gt = doc.find('>', lt);
    if (gt == std::string::npos) break;
    const std::string tag = doc.substr(lt, gt - lt + 1);
    pos = gt + 1;
    for (const char *sec : {"PointData", "Points", "Cells", "FieldData"}) {
      const std::string s = sec;
      if (tag.compare(0, s.size() + 1, "<" + s) == 0 && (tag[s.size() + 1] == '>' || tag[s.size() + 1] == ' '))
        section = s;
      if (tag == "</" + s + ">") section.clear();
    }
    if (tag.compare(0, 10, "<DataArray") != 0) continue;
    const size_t close = doc.find("</DataArray>", pos);
    if (close == std::string::npos) throw error(NOSH_ERR_INVALID, "unterminated DataArray");
    const std::vector<double> v = detail::values(tag, doc.substr(pos, close - pos));
    pos = close + 12;
    const std::string name = detail::attr(tag, "Name");
    const std::string ncs = detail::attr(tag, "NumberOfComponents");
    const int nc = ncs.empty() ? 1 : std::stoi(ncs);
    if (section == "Points") g.coords = v;
    else if (section == "Cells" && name == "connectivity") conn = v;
    else if (section == "Cells" && name == "offsets") off = v;
    else if (section == "Cells" && name == "types") types = v;
    else if (section == "PointData") g.point_data.push_back({name, nc, v});
    else if (section == "FieldData" && !v.empty()) g.field_data.push_back({name, v[0]});
  }
  if (types.empty()) throw error(NOSH_ERR_INVALID, "no cells");
  for (double ty : types)
    if (ty != types[0]) throw error(NOSH_ERR_INVALID, "cells must all be triangles or all tetrahedra");
  g.nvc = types[0] == 5 ? 3 : types[0] == 10 ? 4 : 0;
  if (!g.nvc) throw error(NOSH_ERR_INVALID, "cells must be triangles or tetrahedra");
  const size_t n = g.coords.size() / 3;
  for (size_t k = 0; k < off.size(); k++)
    if (off[k] != (double)((k + 1) * (size_t)g.nvc)) throw error(NOSH_ERR_INVALID, "cell offsets do not match the type");
  g.cells.resize(conn.size());
  for (size_t k = 0; k < conn.size(); k++) {
    if (conn[k] < 0 || conn[k] >= (double)n) throw error(NOSH_ERR_INVALID, "cell connectivity out of range");
    g.cells[k] = (int32_t)conn[k];
  }
  return g;
}

// One state file per converged continuation state, <prefix>0000.vtu, ...,
// as the reference's continuation data saver names them; usable as the
// stepper's observer.
class data_saver {
 public:
  data_saver(const std::vector<double> &coords, const std::vector<int32_t> &cells, int nvc,
             const std::string &prefix = "out", const std::vector<double> *A = nullptr)
      : coords_(coords), cells_(cells), nvc_(nvc), prefix_(prefix), A_(A) {}
  void operator()(int index, const vec &psi, double mu) {
    grid g;
    g.coords = coords_;
    g.cells = cells_;
    g.nvc = nvc_;
    g.point_data.push_back({"psi", 2, psi});
    if (A_) g.point_data.push_back({"A", 3, *A_});
    g.field_data = {{"mu", mu}, {"step", (double)index}};
    char name[32];
    std::snprintf(name, sizeof name, "%04d.vtu", count_++);
    paths_.push_back(prefix_ + name);
    write_vtu(paths_.back(), g);
  }
  const std::vector<std::string> &paths() const { return paths_; }

 private:
  std::vector<double> coords_;
  std::vector<int32_t> cells_;
  int nvc_;
  std::string prefix_;
  const std::vector<double> *A_;
  int count_ = 0;
  std::vector<std::string> paths_;
};

}  // namespace io
}  // namespace nosh

#endif  // NOSH_GB300_HPP
