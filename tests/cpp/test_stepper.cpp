// The C++ continuation stepper of include/nosh_gb300.hpp.
//
// Host logic (no GPU): a fake run that follows the fold curve mu = 1 - x^2
// checks the adaptive step size, failed-step halving, landing on a bound,
// turning around the fold with arclength steps, and the statistics table in
// the reference's csv_writer layout.  With --gpu: natural and arclength runs
// of the device-resident handle on a 2-D square whose every state solves
// F = 0.  Exit code 0 when every check passes.
#include <cmath>
#include <cstdio>
#include <cstring>
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

namespace cont = nosh::continuation;

// (x, mu) on mu = 1 - x^2 from x = 1; steps fail when longer than fail_above
struct fold_run {
  double x = 1.0, m = 0.0, tmu = std::nan(""), fail_above = 1e9;
  int iters = 2;
  bool have_prev = false;
  double px = 0.0, pm = 0.0;
  double mu() const { return m; }
  void state(nosh::vec &v, double &mu_out) const {
    v.assign(2, 0.0);
    v[0] = x;
    mu_out = m;
  }
  nosh_newton_stats ok() const {
    nosh_newton_stats st{};
    st.newton_iters = iters;
    st.krylov_iters = 10;
    return st;
  }
  nosh_newton_stats fail() const {
    nosh_newton_stats st{};
    st.status = NOSH_ERR_NOT_CONVERGED;
    return st;
  }
  nosh_newton_stats advance(double mu_new, int, const nosh_newton_options &) {
    if (std::fabs(mu_new - m) > fail_above || mu_new > 1.0) return fail();
    x = std::sqrt(1.0 - mu_new);
    m = mu_new;
    return ok();
  }
  nosh_newton_stats advance_arclength(double ds, int, double, const nosh_newton_options &) {
    if (std::fabs(ds) > fail_above) return fail();
    double dx = -1.0, dm = 2.0 * x;
    const double nrm = std::sqrt(dx * dx + dm * dm);
    dx /= nrm;
    dm /= nrm;
    if (have_prev && dx * (x - px) + dm * (m - pm) < 0) {
      dx = -dx;
      dm = -dm;
    }
    have_prev = true;
    px = x;
    pm = m;
    x += ds * dx;
    m = 1.0 - x * x;
    tmu = dm;
    return ok();
  }
  double tangent_mu() const { return tmu; }
};

static nosh_newton_options defaults() {
  nosh_newton_options o;
  nosh_newton_default_options(&o);
  return o;
}

static void host_checks() {
  auto none = [](int, const nosh::vec &, double) {};
  {
    // adaptive growth: 2 of 15 nonlinear iterations -> x (1 + 2 (13/14)^2)
    fold_run r;
    cont::stepper_parameters p;
    p.arc_length = false;
    p.predictor = NOSH_PREDICT_SECANT;
    p.initial_step = 1e-3;
    p.max_step = 1e-2;
    p.max_steps = 6;
    const auto out = cont::step(r, p, defaults(), none);
    const double grow = 1.0 + 2.0 * (13.0 / 14.0) * (13.0 / 14.0);
    CHECK(out.steps == 6 && !out.failed);
    CHECK(std::fabs(out.records[1].ds - 1e-3) < 1e-15);
    CHECK(std::fabs(out.records[2].ds - 1e-3 * grow) < 1e-15);
    CHECK(std::fabs(out.records[6].ds - 1e-2) < 1e-15);
  }
  {
    // failures halve the step; below the minimum the run fails
    fold_run r;
    r.fail_above = 3e-3;
    cont::stepper_parameters p;
    p.arc_length = false;
    p.initial_step = 1e-2;
    p.max_step = 1e-2;
    p.max_steps = 2;
    auto out = cont::step(r, p, defaults(), none);
    CHECK(out.failed_steps >= 2 && std::fabs(out.records[1].ds - 2.5e-3) < 1e-15);
    fold_run r2;
    r2.fail_above = 1e-9;
    p.initial_step = 1e-3;
    p.min_step = 1e-7;
    out = cont::step(r2, p, defaults(), none);
    CHECK(out.failed && out.steps == 0 && out.failed_steps == 14);
  }
  {
    // natural steps land exactly on the max value
    fold_run r;
    cont::stepper_parameters p;
    p.arc_length = false;
    p.initial_step = 0.03;
    p.max_step = 0.03;
    p.max_value = 0.1;
    const auto out = cont::step(r, p, defaults(), none);
    CHECK(out.records.back().mu == 0.1 && !out.failed);
  }
  {
    // arclength steps turn around the fold at mu = 1
    fold_run r;
    r.iters = 3;
    cont::stepper_parameters p;
    p.initial_step = 0.05;
    p.max_step = 0.1;
    p.max_steps = 60;
    p.min_value = -0.5;
    p.max_value = 2.0;
    const auto out = cont::step(r, p, defaults(), none);
    double top = 0.0;
    for (const auto &rec : out.records) top = std::max(top, rec.mu);
    CHECK(top > 0.99 && out.records.back().mu < 0.5 && r.x < 0.0);
  }
  {
    // the statistics table: header and a row in csv_writer's layout
    std::FILE *f = std::tmpfile();
    cont::csv_writer w(f);
    const std::vector<cont::csv_writer::cell> row = {{"(0) step", true, 1.0},
                                                     {"(1) mu", false, 0.25},
                                                     {"(2) Gibbs energy", false, -0.1875}};
    w.write_header(row);
    w.write_row(row);
    std::rewind(f);
    char l0[256] = {0}, l1[256] = {0};
    CHECK(std::fgets(l0, sizeof l0, f) && std::fgets(l1, sizeof l1, f));
    std::fclose(f);
    const std::string want0 = std::string("# (0) step   ") + "(1) mu                " + "   " +
                              "(2) Gibbs energy      " + "\n";
    const std::string want1 = std::string("  1          ") + "2.500000000000000e-01 " + "   " +
                              "-1.875000000000000e-01" + "\n";
    CHECK(want0 == l0);
    CHECK(want1 == l1);
  }
}

// 2-D unit square (no jitter), s x s vertices, one diagonal per square
static void square(int s, std::vector<double> &coords, std::vector<int32_t> &cells) {
  coords.clear();
  cells.clear();
  for (int j = 0; j < s; j++)
    for (int i = 0; i < s; i++) {
      coords.push_back((double)i / (s - 1));
      coords.push_back((double)j / (s - 1));
      coords.push_back(0.0);
    }
  for (int j = 0; j + 1 < s; j++)
    for (int i = 0; i + 1 < s; i++) {
      const int a = j * s + i, b = a + 1, c = a + s, d = c + 1;
      cells.insert(cells.end(), {a, b, d, a, d, c});
    }
}

static void gpu_checks() {
  std::vector<double> coords;
  std::vector<int32_t> cells;
  square(17, coords, cells);
  auto m = std::make_shared<nosh::mesh>(coords, cells, 3);
  const int64_t N = m->num_vertices();
  std::vector<double> A(3 * N);
  for (int64_t k = 0; k < N; k++) {
    A[3 * k] = -0.5 * coords[3 * k + 1];
    A[3 * k + 1] = 0.5 * coords[3 * k];
  }
  auto mvp = std::make_shared<nosh::vector_field::explicit_values>(*m, A, 0.0);
  auto V = std::make_shared<nosh::scalar_field::constant>(*m, -1.0);
  auto t = std::make_shared<nosh::scalar_field::constant>(*m, 1.0);
  auto x0 = std::make_shared<nosh::vec>(2 * N, 0.0);
  for (int64_t k = 0; k < N; k++) (*x0)[2 * k] = 1.0;
  nosh::model_evaluator::nls model(m, mvp, V, 1.0, t, x0, "mu");
  nosh::vec x = *x0;
  CHECK(model.newton(x, {{"mu", 0.0}}).status == NOSH_OK);
  for (bool arc : {false, true}) {
    cont::run r(model, x, 0.0);
    cont::stepper_parameters p;
    p.arc_length = arc;
    p.predictor = arc ? NOSH_PREDICT_TANGENT : NOSH_PREDICT_SECANT;
    p.initial_step = 0.05;
    p.max_step = 0.2;
    p.max_steps = 5;
    std::FILE *f = std::tmpfile();
    cont::statistics_observer obs(model, f);
    int seen = 0;
    double worst = 0.0;
    const auto out = cont::step(r, p, defaults(), [&](int i, const nosh::vec &xs, double mu) {
      obs(i, xs, mu);
      nosh::vec fx;
      model.compute_f(xs, {{"mu", mu}}, fx);
      double n2 = 0.0;
      for (double v : fx) n2 += v * v;
      worst = std::max(worst, std::sqrt(n2));
      seen++;
    });
    CHECK(out.steps == 5 && !out.failed && seen == 6);
    CHECK(worst <= 1.5e-10);
    CHECK(out.records.back().mu > 0.1);
    std::rewind(f);
    char l0[256] = {0};
    CHECK(std::fgets(l0, sizeof l0, f) && std::strncmp(l0, "# (0) step", 10) == 0);
    std::fclose(f);
  }
  // the predictors' residuals from a four-state history: every one finite,
  // the extrapolations below the secant on this smooth branch
  {
    cont::run r(model, x, 0.0);
    r.learning(4, 2, 1e-3);
    r.inference_period(2);
    model.set_forcing_aim(0.5);
    nosh_newton_options o;
    nosh_newton_default_options(&o);
    for (int k = 1; k <= 4; k++) CHECK(r.advance(0.01 * k, NOSH_PREDICT_SECANT, o).status == NOSH_OK);
    const auto res = r.predictor_residuals(0.05);
    for (double v : res) CHECK(std::isfinite(v) && v > 0.0);
    CHECK(res[1] < res[0] && res[2] < res[0]);
  }
}

int main(int argc, char **argv) {
  host_checks();
  if (argc > 1 && std::strcmp(argv[1], "--gpu") == 0) gpu_checks();
  if (failures) {
    std::printf("%d failure(s)\n", failures);
    return 1;
  }
  std::printf("all stepper checks passed\n");
  return 0;
}
