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
//
// Trilinos types are replaced by std::vector<double> (interleaved complex
// vectors of length 2N, multivectors as a vector of columns) and parameter
// maps by std::map<std::string, double>, as the reference's own set_parameters
// takes.  Errors surface as nosh::error exceptions carrying the C ABI status
// (the reference throws std::logic_error via TEUCHOS_TEST_FOR_EXCEPT_MSG).
#ifndef NOSH_GB300_HPP
#define NOSH_GB300_HPP

#include <array>
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
}  // namespace nosh

#endif  // NOSH_GB300_HPP
