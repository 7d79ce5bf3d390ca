// Mesh and state files of include/nosh_gb300.hpp (nosh::io), no GPU.
//
//   test_io               round trips (bit-exact), an ASCII file, the
//                         reader's checks, the data saver's file names
//   test_io write <path>  writes the fixed sample grid (for the Python reader)
//   test_io read <path>   prints the sums of a file's arrays (%.17g), for
//                         comparison with the Python writer's data
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

// two tetrahedra on five points, psi, A, V and field data
static nosh::io::grid sample() {
  nosh::io::grid g;
  g.coords = {0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1, 1, 1, 1};
  g.cells = {0, 1, 2, 3, 1, 2, 3, 4};
  g.nvc = 4;
  std::vector<double> psi(10), A(15), V(5);
  for (int i = 0; i < 10; i++) psi[i] = std::sin(0.7 * i + 0.1) / 3.0;
  for (int i = 0; i < 15; i++) A[i] = std::cos(1.3 * i) * 1e-3;
  for (int i = 0; i < 5; i++) V[i] = -1.0 + i / 7.0;
  g.point_data = {{"psi", 2, psi}, {"A", 3, A}, {"V", 1, V}};
  g.field_data = {{"mu", 0.25}, {"step", 3}};
  return g;
}

static void self_test() {
  const std::string p = "nosh_io_selftest.vtu";
  const nosh::io::grid g = sample();
  nosh::io::write_vtu(p, g);
  const nosh::io::grid r = nosh::io::read_vtu(p);
  CHECK(r.nvc == 4 && r.cells == g.cells && r.coords == g.coords);
  CHECK(r.point_data.size() == 3);
  for (const auto &a : g.point_data) {
    const auto *b = r.find(a.name);
    CHECK(b && b->components == a.components && b->values == a.values);
  }
  CHECK(r.field_data.size() == 2 && r.field_data[0].first == "mu" && r.field_data[0].second == 0.25);
  std::remove(p.c_str());
  // ASCII arrays (Int32 connectivity and offsets)
  const char *ascii =
      "<?xml version=\"1.0\"?><VTKFile type=\"UnstructuredGrid\" version=\"1.0\"><UnstructuredGrid>"
      "<Piece NumberOfPoints=\"4\" NumberOfCells=\"2\"><PointData><DataArray type=\"Float64\" Name=\"psi\" "
      "NumberOfComponents=\"2\" format=\"ascii\">1 0 1 0 0.5 0.5 1 -1</DataArray></PointData><Points>"
      "<DataArray type=\"Float64\" NumberOfComponents=\"3\" format=\"ascii\">0 0 0 1 0 0 0 1 0 1 1 0</DataArray>"
      "</Points><Cells><DataArray type=\"Int32\" Name=\"connectivity\" format=\"ascii\">0 1 2 1 3 2</DataArray>"
      "<DataArray type=\"Int32\" Name=\"offsets\" format=\"ascii\">3 6</DataArray><DataArray type=\"UInt8\" "
      "Name=\"types\" format=\"ascii\">5 5</DataArray></Cells></Piece></UnstructuredGrid></VTKFile>";
  const std::string pa = "nosh_io_ascii.vtu";
  std::FILE *f = std::fopen(pa.c_str(), "w");
  std::fputs(ascii, f);
  std::fclose(f);
  const nosh::io::grid ra = nosh::io::read_vtu(pa);
  CHECK(ra.nvc == 3 && ra.cells == (std::vector<int32_t>{0, 1, 2, 1, 3, 2}));
  CHECK(ra.find("psi") && ra.find("psi")->values[5] == 0.5);
  // out-of-range connectivity is rejected
  std::string bad = ascii;
  bad.replace(bad.find(">0 1 2 1 3 2<"), 13, ">0 1 2 1 3 7<");
  f = std::fopen(pa.c_str(), "w");
  std::fputs(bad.c_str(), f);
  std::fclose(f);
  bool threw = false;
  try {
    nosh::io::read_vtu(pa);
  } catch (const nosh::error &) {
    threw = true;
  }
  CHECK(threw);
  std::remove(pa.c_str());
  // the data saver's names and contents
  nosh::io::data_saver saver(g.coords, g.cells, 4, "nosh_io_out");
  for (int k = 0; k < 3; k++) saver(k, std::vector<double>(10, (double)k), 0.1 * k);
  CHECK(saver.paths().size() == 3 && saver.paths()[2] == "nosh_io_out0002.vtu");
  const nosh::io::grid s2 = nosh::io::read_vtu(saver.paths()[2]);
  CHECK(s2.find("psi") && s2.find("psi")->values[7] == 2.0 && s2.field_data[0].second == 0.1 * 2);
  for (const auto &q : saver.paths()) std::remove(q.c_str());
}

int main(int argc, char **argv) {
  try {
    if (argc == 3 && std::strcmp(argv[1], "write") == 0) {
      nosh::io::write_vtu(argv[2], sample());
      return 0;
    }
    if (argc == 3 && std::strcmp(argv[1], "read") == 0) {
      const nosh::io::grid g = nosh::io::read_vtu(argv[2]);
      double sc = 0, cs = 0;
      for (double v : g.coords) sc += v;
      for (int32_t c : g.cells) cs += c;
      std::printf("points %.17g\ncells %.17g\nnvc %d\n", sc, cs, g.nvc);
      for (const auto &a : g.point_data) {
        double t = 0;
        for (double v : a.values) t += v;
        std::printf("%s %d %.17g\n", a.name.c_str(), a.components, t);
      }
      for (const auto &kv : g.field_data) std::printf("field %s %.17g\n", kv.first.c_str(), kv.second);
      return 0;
    }
    self_test();
  } catch (const std::exception &e) {
    std::printf("exception: %s\n", e.what());
    return 1;
  }
  if (failures) {
    std::printf("%d failure(s)\n", failures);
    return 1;
  }
  std::printf("all io checks passed\n");
  return 0;
}
