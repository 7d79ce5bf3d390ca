// The C++ stability eigensolver (nosh::eig) on the GPU: a 17 x 17 unit
// square at mu = 0.3, converged by Newton; the four lowest eigenpairs of the
// Jacobian have small residuals and no gauge component.  The state and the
// eigenvalues go to <path>.vtu and stdout for the oracle comparison that
// tests/test_cpp_api.py makes.  Usage: test_eig <path>
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "nosh_gb300.hpp"

static int failures = 0;

#define CHECK(cond)                                                 \
  do {                                                              \
    if (!(cond)) {                                                  \
      std::printf("FAIL %s:%d  %s\n", __FILE__, __LINE__, #cond); \
      failures++;                                                   \
    }                                                               \
  } while (0)

int main(int argc, char **argv) {
  if (argc != 2) {
    std::printf("usage: test_eig <state.vtu>\n");
    return 2;
  }
  try {
    const int s = 17;
    std::vector<double> coords;
    std::vector<int32_t> cells;
    for (int j = 0; j < s; j++)
      for (int i = 0; i < s; i++) coords.insert(coords.end(), {(double)i / (s - 1), (double)j / (s - 1), 0.0});
    for (int j = 0; j + 1 < s; j++)
      for (int i = 0; i + 1 < s; i++) {
        const int a = j * s + i, b = a + 1, c = a + s, d = c + 1;
        cells.insert(cells.end(), {a, b, d, a, d, c});
      }
    auto m = std::make_shared<nosh::mesh>(coords, cells, 3);
    const int64_t N = m->num_vertices();
    std::vector<double> A(3 * N);
    for (int64_t k = 0; k < N; k++) {
      A[3 * k] = -0.5 * coords[3 * k + 1];
      A[3 * k + 1] = 0.5 * coords[3 * k];
    }
    const double mu = 0.3;
    auto mvp = std::make_shared<nosh::vector_field::explicit_values>(*m, A, mu);
    auto V = std::make_shared<nosh::scalar_field::constant>(*m, -1.0);
    auto t = std::make_shared<nosh::scalar_field::constant>(*m, 1.0);
    auto x0 = std::make_shared<nosh::vec>(2 * N, 0.0);
    for (int64_t k = 0; k < N; k++) (*x0)[2 * k] = 1.0;
    nosh::model_evaluator::nls model(m, mvp, V, 1.0, t, x0, "mu");
    nosh::vec psi = *x0;
    const std::map<std::string, double> p = {{"mu", mu}, {"g", 1.0}};
    CHECK(model.newton(psi, p, 1e-12).status == NOSH_OK);
    const int prec0 = model.precision();
    const auto r = nosh::eig::lowest_eigenpairs(model, psi, p, 4, 1e-9);
    CHECK(model.precision() == prec0);
    CHECK(r.values.size() == 4 && r.iterations < 500);
    // residuals and the gauge component, with the FP64 Jacobian
    model.set_precision(NOSH_PREC_FP64);
    auto J = model.create_W_op();
    J->rebuild(p, psi);
    std::vector<nosh::vec> Y;
    J->apply(r.vectors, Y);
    double unorm = 0.0;
    for (int64_t k = 0; k < N; k++) unorm += psi[2 * k] * psi[2 * k] + psi[2 * k + 1] * psi[2 * k + 1];
    unorm = std::sqrt(unorm);
    for (size_t j = 0; j < r.values.size(); j++) {
      double res = 0.0, nv = 0.0, g = 0.0;
      for (int64_t i = 0; i < 2 * N; i++) {
        const double d = Y[j][i] - r.values[j] * r.vectors[j][i];
        res += d * d;
        nv += r.vectors[j][i] * r.vectors[j][i];
      }
      for (int64_t k = 0; k < N; k++)
        g += -psi[2 * k + 1] * r.vectors[j][2 * k] + psi[2 * k] * r.vectors[j][2 * k + 1];
      CHECK(std::fabs(std::sqrt(nv) - 1.0) < 1e-10);
      CHECK(std::sqrt(res) < 1e-7);
      CHECK(std::fabs(g) / unorm < 1e-8);
      if (j) CHECK(r.values[j] >= r.values[j - 1]);
    }
    nosh::io::grid gr;
    gr.coords = coords;
    gr.cells = cells;
    gr.nvc = 3;
    gr.point_data.push_back({"psi", 2, psi});
    gr.point_data.push_back({"A", 3, A});
    gr.field_data = {{"mu", mu}};
    nosh::io::write_vtu(argv[1], gr);
    for (double v : r.values) std::printf("eigenvalue %.17g\n", v);
  } catch (const std::exception &e) {
    std::printf("exception: %s\n", e.what());
    return 1;
  }
  if (failures) {
    std::printf("%d failure(s)\n", failures);
    return 1;
  }
  std::printf("all eig checks passed\n");
  return 0;
}
