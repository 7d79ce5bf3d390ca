// The reference's own test cases (test/mesh.cpp, test/keo.cpp, test/jac.cpp,
// test/compute_f.cpp, test/dfdp.cpp), written against the C++ API of
// include/nosh_gb300.hpp on the reconstructed "rectanglesmall" and
// "cubesmall" meshes whose constants those files print.  Exit code 0 when
// every check passes.
#include <cmath>
#include <cstdio>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "nosh_gb300.hpp"

static int failures = 0;

#define REQUIRE_CLOSE(a, b, tol)                                                            \
  do {                                                                                      \
    const double a_ = (a), b_ = (b);                                                        \
    if (!(std::fabs(a_ - b_) <= (tol))) {                                                   \
      std::printf("FAIL %s:%d  %s = %.17g, expected %.17g\n", __FILE__, __LINE__, #a, a_, b_); \
      failures++;                                                                           \
    }                                                                                       \
  } while (0)

struct Case {
  std::string name;
  std::vector<double> coords;
  std::vector<int32_t> cells;
  int nvc;
};

static Case rectanglesmall() {
  return {"rectanglesmall",
          {-5, -0.5, 0, 5, 0.5, 0, -5, 0.5, 0, 5, -0.5, 0},
          {0, 3, 1, 0, 1, 2},
          3};
}

static Case cubesmall() {
  Case c{"cubesmall", {}, {0, 1, 2, 4, 1, 2, 3, 7, 1, 4, 5, 7, 2, 4, 6, 7, 1, 2, 4, 7}, 4};
  for (int v = 0; v < 8; v++) {
    c.coords.push_back((v & 1) ? 0.5 : -0.5);
    c.coords.push_back((v & 2) ? 0.5 : -0.5);
    c.coords.push_back((v & 4) ? 5.0 : -5.0);
  }
  return c;
}

static std::vector<double> mvp(const std::vector<double> &x) {
  std::vector<double> A(x.size(), 0.0);
  for (size_t i = 0; i < x.size() / 3; i++) {
    A[3 * i] = -0.5 * x[3 * i + 1];
    A[3 * i + 1] = 0.5 * x[3 * i];
  }
  return A;
}

static double dot(const std::vector<double> &a, const std::vector<double> &b) {
  double s = 0.0;
  for (size_t i = 0; i < a.size(); i++) s += a[i] * b[i];
  return s;
}

int main() {
  struct Expect {
    double cv1, cv2, cvinf;
    double keo_sum, keo_even;
    double jac[3];
    double f1, f2, finf;
  };
  // constants: test/mesh.cpp:44-47,93-95; test/keo.cpp:137-138,163-164;
  // test/jac.cpp:120-122,145-147; test/compute_f.cpp:81-83,105-107
  const Expect ex[2] = {
      {10.0, 5.0, 2.5, 0.01262434246161348, 0.0063121712308067401,
       {20.0126243424616, 20.0063121712308, 0.00631217123080606},
       0.50126061034211067, 0.24749434381636057, 0.12373710977782607},
      {10.0, 3.535533905932738, 1.25, 1.67083246311428e-4, 8.3541623155714007e-05,
       {20.000167083246311, 20.000083541623155, 8.3541623155658495e-05},
       8.3541623156163313e-05, 2.9536515963905867e-05, 1.0468744547749431e-05},
  };
  const Case cases[2] = {rectanglesmall(), cubesmall()};
  const double mu = 1.0e-2;
  for (int c = 0; c < 2; c++) {
    const Case &cs = cases[c];
    const Expect &e = ex[c];
    auto m = std::make_shared<const nosh::mesh>(cs.coords, cs.cells, cs.nvc);
    const int64_t N = m->num_vertices();
    // testMesh
    auto cv = m->control_volumes();
    double n1 = 0, n2 = 0, ni = 0;
    for (double v : cv) {
      n1 += std::fabs(v);
      n2 += v * v;
      ni = std::fmax(ni, std::fabs(v));
    }
    REQUIRE_CLOSE(n1, e.cv1, 1e-12 * e.cv1);
    REQUIRE_CLOSE(std::sqrt(n2), e.cv2, 1e-12 * e.cv2);
    REQUIRE_CLOSE(ni, e.cvinf, 1e-12 * e.cvinf);
    // fields as in the tests: A explicit, V = -1, thickness = 1, psi = 1
    auto A = std::make_shared<nosh::vector_field::explicit_values>(*m, mvp(cs.coords), mu);
    auto sp = std::make_shared<nosh::scalar_field::constant>(*m, -1.0);
    auto th = std::make_shared<nosh::scalar_field::constant>(*m, 1.0);
    std::vector<double> psi(2 * N, 0.0);
    for (int64_t k = 0; k < N; k++) psi[2 * k] = 1.0;
    auto psi_ptr = std::make_shared<const std::vector<double>>(psi);
    nosh::model_evaluator::nls model(m, A, sp, 1.0, th, psi_ptr, "mu");
    model.set_precision(NOSH_PREC_FP64);
    const auto names = model.get_p_names();
    if (names.size() != 2 || names[0] != "g" || names[1] != "mu") {
      std::printf("FAIL p_names\n");
      failures++;
    }
    const std::map<std::string, double> params{{"g", 1.0}, {"mu", mu}};
    std::vector<double> ones(2 * N, 1.0), even(2 * N, 0.0), odd(2 * N, 0.0), Ku;
    for (int64_t k = 0; k < N; k++) {
      even[2 * k] = 1.0;
      odd[2 * k + 1] = 1.0;
    }
    // testKeo
    model.keo()->set_parameters({{"mu", mu}});
    model.keo()->apply(ones, Ku);
    REQUIRE_CLOSE(dot(ones, Ku), e.keo_sum, 1e-10);
    model.keo()->apply(even, Ku);
    REQUIRE_CLOSE(dot(even, Ku), e.keo_even, 1e-10);
    model.keo()->apply(odd, Ku);
    REQUIRE_CLOSE(std::fabs(dot(even, Ku)), 0.0, 1e-10);
    // testJac
    auto jac = model.create_W_op();
    jac->rebuild(params, psi);
    const std::vector<std::vector<double>> S{ones, even, odd};
    std::vector<std::vector<double>> JS;
    jac->apply(S, JS);
    for (int k = 0; k < 3; k++) REQUIRE_CLOSE(dot(S[k], JS[k]), e.jac[k], 1e-10);
    bool threw = false;
    try {
      jac->apply(S, JS, NOSH_NO_TRANS, 2.0, 0.0);
    } catch (const nosh::error &err) {
      threw = err.code == NOSH_ERR_UNSUPPORTED;
    }
    if (!threw) {
      std::printf("FAIL alpha != 1 must be rejected\n");
      failures++;
    }
    // testComputeF
    std::vector<double> f;
    model.compute_f(psi, params, f);
    double f1 = 0, f2 = 0, fi = 0;
    for (double v : f) {
      f1 += std::fabs(v);
      f2 += v * v;
      fi = std::fmax(fi, std::fabs(v));
    }
    REQUIRE_CLOSE(f1, e.f1, 1e-10 * e.f1);
    REQUIRE_CLOSE(std::sqrt(f2), e.f2, 1e-10 * e.f2);
    REQUIRE_CLOSE(fi, e.finf, 1e-10 * e.finf);
    std::printf("%s: checked (failures so far %d)\n", cs.name.c_str(), failures);
  }
  // test_dfdp: dF/dg vs a central difference (eps 1e-8) with DkeoDP built for
  // "g", as test/dfdp.cpp:20-47,136-137 does
  {
    const Case cs = cubesmall();
    auto m = std::make_shared<const nosh::mesh>(cs.coords, cs.cells, cs.nvc);
    const int64_t N = m->num_vertices();
    auto A = std::make_shared<nosh::vector_field::explicit_values>(*m, mvp(cs.coords), 0.0);
    auto sp = std::make_shared<nosh::scalar_field::constant>(*m, -1.0);
    auto th = std::make_shared<nosh::scalar_field::constant>(*m, 1.0);
    std::vector<double> z(2 * N);
    for (size_t i = 0; i < z.size(); i++) z[i] = (i % 2 ? 0.0 : 1.0) + 0.1 * std::sin(1.0 + 3.0 * i);
    nosh::model_evaluator::nls model(m, A, sp, 1.0, th, std::make_shared<const std::vector<double>>(z), "g");
    const double eps = 1e-8;
    std::vector<double> fp, fm;
    model.compute_f(z, {{"g", 1.0 + eps}, {"mu", 0.0}}, fp);
    model.compute_f(z, {{"g", 1.0 - eps}, {"mu", 0.0}}, fm);
    auto dfdp = model.compute_dfdp(z, {{"g", 1.0}, {"mu", 0.0}});
    double worst = 0.0;
    for (size_t i = 0; i < z.size(); i++) worst = std::fmax(worst, std::fabs((fp[i] - fm[i]) / (2 * eps) - dfdp[0][i]));
    REQUIRE_CLOSE(worst, 0.0, 1e-6);
  }
  std::printf(failures ? "FAILED (%d)\n" : "all reference-API checks passed\n", failures);
  return failures ? 1 : 0;
}
