// Mesh handle: host integer data + device geometry / KEO graph.
#pragma once

#include "common.cuh"

namespace nosh {

struct MeshImpl {
  int nvc = 0, ne = 0;  // vertices / edges per cell
  int64_t N = 0, E = 0, T = 0;
  cudaStream_t stream = nullptr;

  // host: input and integer work
  std::vector<double> x;          // 3N
  std::vector<int32_t> cells;     // nvc*T
  std::vector<int32_t> edges;     // 2E, v0 < v1, lexicographic
  std::vector<int32_t> cell_edges;  // ne*T
  std::vector<int64_t> edge_base;   // N+1: first edge id whose v0 == v
  // off-diagonal KEO graph ("adjacency CSR"): row v = sorted neighbours
  std::vector<int64_t> rp;        // N+1
  std::vector<int32_t> ci;        // 2E
  std::vector<int32_t> nz_edge;   // 2E: edge of each nonzero (~e if row is v1)
  std::vector<int32_t> pos_fwd, pos_bwd;  // E: nonzero of (v0,v1) / (v1,v0)
  std::vector<int64_t> vc_ptr;    // N+1, vertex -> cell*nvc+slot (cell order)
  std::vector<int32_t> vc_idx;
  std::vector<int64_t> ec_ptr;    // E+1, edge -> cell*ne+slot (cell order)
  std::vector<int32_t> ec_idx;
  std::vector<double> h_len, h_covol, h_cv;

  // device
  DevBuf<double> d_x, d_len, d_covol, d_cv;
  DevBuf<int32_t> d_edges;
  DevBuf<int64_t> d_rp64;
  DevBuf<int32_t> d_rp, d_ci, d_nz_edge, d_pos_fwd, d_pos_bwd;

  // expects a description that validate() accepted
  MeshImpl(const double *coords, int64_t n_vertices, const int32_t *cells,
           int64_t n_cells, int verts_per_cell);
  ~MeshImpl();
  // host-only checks of a mesh description (sizes, cell type, every vertex
  // index in range, no cell repeating a vertex); throws nosh::Error
  static void validate(int64_t n_vertices, const int32_t *cells, int64_t n_cells,
                       int verts_per_cell);
  MeshImpl(const MeshImpl &) = delete;
  MeshImpl &operator=(const MeshImpl &) = delete;

  // complex graph with the diagonal (row_ptr[N+1], cols[N+2E])
  void complex_graph(int32_t *row_ptr, int32_t *cols) const;

 private:
  void build_topology();
  void build_geometry();
};

}  // namespace nosh
