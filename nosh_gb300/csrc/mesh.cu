// Mesh set-up: integer work on the host (edges, KEO graph, edge -> nonzero
// scatter map), geometry on the GPU in FP64 (edge coefficients, covolumes,
// control volumes).
//
// Reference: nosh::mesh + mesh_tri / mesh_tetra (src/mesh.cpp,
// src/mesh_tri.cpp, src/mesh_tetra.cpp).  Edge order: the reference takes
// MOAB's entity order, which is not reproducible without MOAB; here edges are
// the canonical sorted pairs (v0 < v1) in lexicographic order, and the KEO
// graph (sorted columns per row) is identical to Tpetra's after fillComplete.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

#include "mesh.cuh"

namespace nosh {

namespace {

constexpr int TRI_PAIRS[3][2] = {{0, 1}, {0, 2}, {1, 2}};
constexpr int TET_PAIRS[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};

// local edge k of a simplex joins local vertices (pair0(k), pair1(k)):
// triangles (0,1),(0,2),(1,2); tetrahedra (0,1),(0,2),(0,3),(1,2),(1,3),(2,3).
// constexpr so that unrolled loops index register arrays statically.
template <int nvc>
__host__ __device__ constexpr int pair0(int k) {
  return nvc == 3 ? (k < 2 ? 0 : 1) : (k < 3 ? 0 : (k < 5 ? 1 : 2));
}
template <int nvc>
__host__ __device__ constexpr int pair1(int k) {
  return nvc == 3 ? (k == 0 ? 1 : 2) : (k < 3 ? k + 1 : (k == 3 ? 2 : 3));
}

struct V3 {
  double x, y, z;
};
__device__ __forceinline__ V3 ld3(const double *p) { return V3{p[0], p[1], p[2]}; }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 operator*(double s, V3 a) { return V3{s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
  return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ double norm(V3 a) { return sqrt(dot(a, a)); }

// In-place Cholesky solve of the SPD system A c = r (n <= 6), fully unrolled.
// The edge-coefficient matrix A_ij = (e_i . e_j)^2 is the Gram matrix of the
// rank-one tensors e_i e_i^T, SPD for a non-degenerate simplex.
template <int n>
__device__ __forceinline__ bool chol_solve(double (&A)[n][n], double (&r)[n]) {
#pragma unroll
  for (int j = 0; j < n; j++) {
    double d = A[j][j];
#pragma unroll
    for (int k = 0; k < j; k++) d -= A[j][k] * A[j][k];
    if (!(d > 0.0)) return false;
    d = sqrt(d);
    A[j][j] = d;
    const double inv = 1.0 / d;
#pragma unroll
    for (int i = j + 1; i < n; i++) {
      double s = A[i][j];
#pragma unroll
      for (int k = 0; k < j; k++) s -= A[i][k] * A[j][k];
      A[i][j] = s * inv;
    }
  }
#pragma unroll
  for (int i = 0; i < n; i++) {
    double s = r[i];
#pragma unroll
    for (int k = 0; k < i; k++) s -= A[i][k] * r[k];
    r[i] = s / A[i][i];
  }
#pragma unroll
  for (int i = n - 1; i >= 0; i--) {
    double s = r[i];
#pragma unroll
    for (int k = i + 1; k < n; k++) s -= A[k][i] * r[k];
    r[i] = s / A[i][i];
  }
  return true;
}

// Triangle circumcenter in barycentric form (src/mesh.cpp:897-928).
__device__ __forceinline__ V3 tri_cc(V3 n0, V3 n1, V3 n2, int *err) {
  const V3 a = n0 - n1, b = n1 - n2, c = n2 - n0;
  const V3 ab = cross(a, b);
  const double omega = 2.0 * dot(ab, ab);
  // degenerate triangle (the reference tests |omega| < 1e-10 absolutely,
  // src/mesh.cpp:917-927; a scale-free test keeps fine meshes valid)
  if (!(omega > 1.0e-20 * dot(a, a) * dot(b, b))) atomicOr(err, 1);
  const double al = -dot(b, b) * dot(a, c) / omega;
  const double be = -dot(c, c) * dot(b, a) / omega;
  const double ga = -dot(a, a) * dot(c, b) / omega;
  return al * n0 + be * n1 + ga * n2;
}

// Per simplex: edge coefficients (src/mesh_tri.cpp:107-151,
// src/mesh_tetra.cpp:107-160) times edge length, one value per local edge,
// and the control-volume share of each local vertex (circumcentric
// splitting, src/mesh.cpp:931-1027, src/mesh_tetra.cpp:196-331).
template <int nvc>
__global__ void cell_geometry_kernel(int64_t T, const int32_t *__restrict__ cells,
                                     const double *__restrict__ x,
                                     double *__restrict__ coef_len,
                                     double *__restrict__ cv_part, int *err) {
  constexpr int ne = nvc == 3 ? 3 : 6;
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= T) return;
  V3 v[nvc];
#pragma unroll
  for (int k = 0; k < nvc; k++) v[k] = ld3(x + 3 * (int64_t)cells[nvc * c + k]);
  V3 ev[ne];
  double len[ne];
#pragma unroll
  for (int k = 0; k < ne; k++) {
    ev[k] = v[pair0<nvc>(k)] - v[pair1<nvc>(k)];
    len[k] = norm(ev[k]);
  }
  double vol;
  if (nvc == 3) {
    vol = 0.5 * norm(cross(ev[0], ev[1]));
  } else {
    // local edges 0,1,2 share local vertex 0: never coplanar
    const double t = dot(ev[0], cross(ev[1], ev[2]));
    if (fabs(t) / (len[0] * len[1] * len[2]) < 1.0e-5) atomicOr(err, 2);
    vol = fabs(t) / 6.0;
  }
  double A[ne][ne], r[ne];
#pragma unroll
  for (int i = 0; i < ne; i++) {
    const double a = dot(ev[i], ev[i]);
    r[i] = vol * a;
#pragma unroll
    for (int j = 0; j < ne; j++) {
      const double d = dot(ev[i], ev[j]);
      A[i][j] = d * d;
    }
  }
  if (!chol_solve<ne>(A, r)) atomicOr(err, 4);
#pragma unroll
  for (int k = 0; k < ne; k++) coef_len[ne * c + k] = r[k] * len[k];

  // control volumes
  double share[nvc];
#pragma unroll
  for (int k = 0; k < nvc; k++) share[k] = 0.0;
  if (nvc == 3) {
    const V3 cc = tri_cc(v[0], v[1], v[2], err);
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const int e0 = pair0<3>(k), e1 = pair1<3>(k), o = 3 - e0 - e1;
      const V3 mp = 0.5 * (v[e0] + v[e1]);
      const double coedge = norm(mp - cc);
      const V3 cell_n = cross(v[o] - v[e0], mp - v[e0]);
      const V3 cc_n = cross(cc - v[e0], mp - v[e0]);
      const double cov = copysign(coedge, dot(cc_n, cell_n));
      const double pyr = 0.5 * len[k] * cov / 2;
      share[e0] += pyr;
      share[e1] += pyr;
    }
  } else {
    // tetrahedron circumcenter (src/mesh_tetra.cpp:377-415)
    const V3 r0 = v[1] - v[0], r1 = v[2] - v[0], r2 = v[3] - v[0];
    const V3 c12 = cross(r1, r2), c20 = cross(r2, r0), c01 = cross(r0, r1);
    const double omega = 2.0 * dot(r0, c12);
    if (!(fabs(omega) > 1.0e-10 * norm(r0) * norm(r1) * norm(r2))) atomicOr(err, 8);
    const V3 cc = v[0] + (dot(r0, r0) / omega) * c12 + (dot(r1, r1) / omega) * c20 +
                  (dot(r2, r2) / omega) * c01;
#pragma unroll
    for (int k = 0; k < 6; k++) {
      const int e0 = pair0<4>(k), e1 = pair1<4>(k);
      int o0 = -1, o1 = -1;
#pragma unroll
      for (int q = 0; q < 4; q++)
        if (q != e0 && q != e1) {
          if (o0 < 0) o0 = q;
          else o1 = q;
        }
      const V3 x0 = v[e0], x1 = v[e1], p0 = v[o0], p1 = v[o1];
      const V3 mp = 0.5 * (x0 + x1);
      const V3 f0 = tri_cc(x0, x1, p0, err), f1 = tri_cc(x0, x1, p1, err);
      const V3 gauge = cross(p0 - mp, p1 - mp);
      const double a0 = 0.5 * norm(mp - f0) * norm(f0 - cc);
      const double a1 = 0.5 * norm(mp - f1) * norm(f1 - cc);
      const double cov = copysign(a0, dot(cross(f0 - mp, cc - mp), gauge)) +
                         copysign(a1, dot(cross(cc - mp, f1 - mp), gauge));
      const double pyr = 0.5 * len[k] * cov / 3;
      share[e0] += pyr;
      share[e1] += pyr;
    }
  }
#pragma unroll
  for (int k = 0; k < nvc; k++) cv_part[nvc * c + k] = share[k];
}

// out[i] = sum_{j in [ptr[i], ptr[i+1])} src[idx[j]] in list order
// (deterministic segmented sum; the lists are in cell order, the order in
// which the reference accumulates).
__global__ void segmented_gather_sum(int64_t n, const int64_t *__restrict__ ptr,
                                     const int32_t *__restrict__ idx,
                                     const double *__restrict__ src,
                                     double *__restrict__ out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int64_t j = ptr[i]; j < ptr[i + 1]; j++) s += src[idx[j]];
  out[i] = s;
}

__global__ void edge_length_kernel(int64_t E, const int32_t *__restrict__ edges,
                                   const double *__restrict__ x,
                                   double *__restrict__ len) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= E) return;
  const V3 d = ld3(x + 3 * (int64_t)edges[2 * e]) - ld3(x + 3 * (int64_t)edges[2 * e + 1]);
  len[e] = norm(d);
}

}  // namespace

// ------------------------------------------------------------------------
void MeshImpl::validate(int64_t n_vertices, const int32_t *cells, int64_t n_cells,
                        int verts_per_cell) {
  NOSH_CHECK(verts_per_cell == 3 || verts_per_cell == 4, NOSH_ERR_INVALID,
             "verts_per_cell must be 3 (triangles) or 4 (tetrahedra)");
  NOSH_CHECK(n_vertices > 0 && n_cells > 0, NOSH_ERR_INVALID, "empty mesh");
  NOSH_CHECK(n_cells * verts_per_cell < (int64_t)1 << 31 && n_vertices < (int64_t)1 << 30,
             NOSH_ERR_INVALID, "mesh too large for 32-bit indices");
  const int nvc = verts_per_cell;
  // bounds of every index before anything is uploaded
  for (int64_t k = 0; k < nvc * n_cells; k++)
    NOSH_CHECK(cells[k] >= 0 && cells[k] < n_vertices, NOSH_ERR_INVALID,
               "cell vertex index out of range at entry " + std::to_string(k));
  for (int64_t c = 0; c < n_cells; c++)
    for (int a = 0; a < nvc; a++)
      for (int b = a + 1; b < nvc; b++)
        NOSH_CHECK(cells[nvc * c + a] != cells[nvc * c + b], NOSH_ERR_MESH,
                   "cell " + std::to_string(c) + " repeats a vertex");
}

MeshImpl::MeshImpl(const double *coords, int64_t n_vertices, const int32_t *cells_in,
                   int64_t n_cells, int verts_per_cell) {
  // the description has passed validate() (nosh_mesh_create runs it before
  // it looks for a device): one pass over the cells, not two
  nvc = verts_per_cell;
  ne = nvc == 3 ? 3 : 6;
  N = n_vertices;
  T = n_cells;
  x.assign(coords, coords + 3 * N);
  cells.assign(cells_in, cells_in + nvc * T);
  NOSH_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  try {
    build_topology();
    build_geometry();
  } catch (...) {
    // a throwing constructor runs no destructor: release the stream here
    // (the device buffers free themselves)
    cudaStreamSynchronize(stream);
    cudaStreamDestroy(stream);
    stream = nullptr;
    throw;
  }
}

MeshImpl::~MeshImpl() {
  if (stream) cudaStreamDestroy(stream);
}

void MeshImpl::build_topology() {
  // vertex -> (cell*nvc + slot) incidence, in cell order
  vc_ptr.assign(N + 1, 0);
  for (int64_t k = 0; k < nvc * T; k++) vc_ptr[cells[k] + 1]++;
  for (int64_t i = 0; i < N; i++) vc_ptr[i + 1] += vc_ptr[i];
  vc_idx.resize(nvc * T);
  {
    std::vector<int64_t> fill(vc_ptr.begin(), vc_ptr.end() - 1);
    for (int64_t k = 0; k < nvc * T; k++) vc_idx[fill[cells[k]]++] = (int32_t)k;
  }
  // neighbour sets: per vertex, sorted unique vertices of incident cells
  auto neighbours = [&](int64_t v, std::vector<int32_t> &buf) {
    buf.clear();
    for (int64_t j = vc_ptr[v]; j < vc_ptr[v + 1]; j++) {
      const int64_t c = vc_idx[j] / nvc;
      for (int q = 0; q < nvc; q++) {
        const int32_t w = cells[nvc * c + q];
        if (w != v) buf.push_back(w);
      }
    }
    std::sort(buf.begin(), buf.end());
    buf.erase(std::unique(buf.begin(), buf.end()), buf.end());
  };
  std::vector<int32_t> deg(N), up(N);
  parallel_for(N, [&](int64_t v) {
    thread_local std::vector<int32_t> buf;
    neighbours(v, buf);
    deg[v] = (int32_t)buf.size();
    up[v] = (int32_t)(buf.end() - std::upper_bound(buf.begin(), buf.end(), (int32_t)v));
  });
  rp.assign(N + 1, 0);
  edge_base.assign(N + 1, 0);
  for (int64_t v = 0; v < N; v++) {
    rp[v + 1] = rp[v] + deg[v];
    edge_base[v + 1] = edge_base[v] + up[v];
  }
  NOSH_CHECK(rp[N] < (int64_t)1 << 31, NOSH_ERR_INVALID, "too many edges");
  E = edge_base[N];
  ci.resize(rp[N]);
  parallel_for(N, [&](int64_t v) {
    thread_local std::vector<int32_t> buf;
    neighbours(v, buf);
    std::copy(buf.begin(), buf.end(), ci.begin() + rp[v]);
  });
  // edges in lexicographic order: the upper neighbours of each vertex
  edges.resize(2 * E);
  pos_fwd.resize(E);
  pos_bwd.resize(E);
  nz_edge.resize(rp[N]);
  parallel_for(N, [&](int64_t v) {
    const int32_t *b = ci.data() + rp[v], *e = ci.data() + rp[v + 1];
    const int32_t *u = std::upper_bound(b, e, (int32_t)v);
    int64_t id = edge_base[v];
    for (const int32_t *q = u; q < e; q++, id++) {
      edges[2 * id] = (int32_t)v;
      edges[2 * id + 1] = *q;
      pos_fwd[id] = (int32_t)(q - ci.data());
      const int32_t *wb = ci.data() + rp[*q], *we = ci.data() + rp[*q + 1];
      pos_bwd[id] = (int32_t)(std::lower_bound(wb, we, (int32_t)v) - ci.data());
    }
  });
  parallel_for(E, [&](int64_t e) {
    nz_edge[pos_fwd[e]] = (int32_t)e;
    nz_edge[pos_bwd[e]] = ~(int32_t)e;
  });
  // cell -> edge ids
  const int(*pairs)[2] = nvc == 3 ? TRI_PAIRS : TET_PAIRS;
  cell_edges.resize(ne * T);
  parallel_for(T, [&](int64_t c) {
    for (int k = 0; k < ne; k++) {
      int32_t a = cells[nvc * c + pairs[k][0]], b = cells[nvc * c + pairs[k][1]];
      const int32_t lo = std::min(a, b), hi = std::max(a, b);
      const int32_t *rb = ci.data() + rp[lo], *re = ci.data() + rp[lo + 1];
      const int32_t *u = std::upper_bound(rb, re, lo);
      cell_edges[ne * c + k] = (int32_t)(edge_base[lo] + (std::lower_bound(u, re, hi) - u));
    }
  });
  // edge -> (cell*ne + slot) incidence in cell order (covolume accumulation)
  ec_ptr.assign(E + 1, 0);
  for (int64_t k = 0; k < ne * T; k++) ec_ptr[cell_edges[k] + 1]++;
  for (int64_t e = 0; e < E; e++) ec_ptr[e + 1] += ec_ptr[e];
  ec_idx.resize(ne * T);
  {
    std::vector<int64_t> fill(ec_ptr.begin(), ec_ptr.end() - 1);
    for (int64_t k = 0; k < ne * T; k++) ec_idx[fill[cell_edges[k]]++] = (int32_t)k;
  }
}

void MeshImpl::build_geometry() {
  cudaStream_t s = stream;
  d_x.upload(x, s);
  d_edges.upload(edges, s);
  DevBuf<int32_t> d_cells;
  d_cells.upload(cells, s);
  DevBuf<double> coef_len(ne * T), cv_part(nvc * T);
  DevBuf<int> err(1);
  err.zero(s);
  const int B = 128;
  if (nvc == 3)
    cell_geometry_kernel<3><<<div_up(T, B), B, 0, s>>>(T, d_cells.p, d_x.p, coef_len.p, cv_part.p, err.p);
  else
    cell_geometry_kernel<4><<<div_up(T, B), B, 0, s>>>(T, d_cells.p, d_x.p, coef_len.p, cv_part.p, err.p);
  NOSH_CUDA(cudaGetLastError());
  d_len.alloc(E);
  d_covol.alloc(E);
  d_cv.alloc(N);
  edge_length_kernel<<<div_up(E, 256), 256, 0, s>>>(E, d_edges.p, d_x.p, d_len.p);
  {
    DevBuf<int64_t> p(E + 1);
    DevBuf<int32_t> idx;
    p.upload(ec_ptr, s);
    idx.upload(ec_idx, s);
    segmented_gather_sum<<<div_up(E, 256), 256, 0, s>>>(E, p.p, idx.p, coef_len.p, d_covol.p);
    DevBuf<int64_t> vp(N + 1);
    DevBuf<int32_t> vidx;
    vp.upload(vc_ptr, s);
    vidx.upload(vc_idx, s);
    segmented_gather_sum<<<div_up(N, 256), 256, 0, s>>>(N, vp.p, vidx.p, cv_part.p, d_cv.p);
    NOSH_CUDA(cudaGetLastError());
    int herr = 0;
    err.download(&herr, 1, s);
    NOSH_CUDA(cudaStreamSynchronize(s));
    NOSH_CHECK(herr == 0, NOSH_ERR_MESH,
               "degenerate cell(s) in the mesh (flags " + std::to_string(herr) + ")");
  }
  // device copies of the KEO graph / scatter map used by every operator
  {
    std::vector<int32_t> rp32(rp.begin(), rp.end());
    d_rp.upload(rp32, s);
    NOSH_CUDA(cudaStreamSynchronize(s));
  }
  // column indices padded by kPad entries so that 128-bit staged loads of a
  // row block may run past its end
  d_ci.alloc(ci.size() + kPad);
  NOSH_CUDA(cudaMemsetAsync(d_ci.p, 0, (ci.size() + kPad) * sizeof(int32_t), s));
  NOSH_CUDA(cudaMemcpyAsync(d_ci.p, ci.data(), ci.size() * sizeof(int32_t), cudaMemcpyHostToDevice, s));
  d_pos_fwd.upload(pos_fwd, s);
  d_pos_bwd.upload(pos_bwd, s);
  d_nz_edge.upload(nz_edge, s);
  NOSH_CUDA(cudaStreamSynchronize(s));
  // host copies of the geometry for the query entry points
  h_len.resize(E);
  h_covol.resize(E);
  h_cv.resize(N);
  d_len.download(h_len.data(), E, s);
  d_covol.download(h_covol.data(), E, s);
  d_cv.download(h_cv.data(), N, s);
  NOSH_CUDA(cudaStreamSynchronize(s));
}

void MeshImpl::complex_graph(int32_t *row_ptr, int32_t *cols) const {
  row_ptr[0] = 0;
  for (int64_t v = 0; v < N; v++) {
    const int64_t b = rp[v], e = rp[v + 1], o = row_ptr[v];
    int64_t k = 0;
    bool placed = false;
    for (int64_t q = b; q < e; q++) {
      if (!placed && ci[q] > v) {
        cols[o + k++] = (int32_t)v;
        placed = true;
      }
      cols[o + k++] = ci[q];
    }
    if (!placed) cols[o + k++] = (int32_t)v;
    row_ptr[v + 1] = (int32_t)(o + k);
  }
}

}  // namespace nosh
