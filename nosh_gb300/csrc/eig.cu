// Lowest eigenpairs of the Jacobian (the stability of a state), LOBPCG on
// the GPU.
//
// The reference's eigen tool (executables/nosh-eig/nosh-eig.cpp:57-) hands
// the Jacobian operator to an Anasazi solver; its continuation
// configuration asks for the eigenvalues of J nearest zero
// (examples/conf.xml:50-66).  J is real symmetric; a converged state is
// stable when no eigenvalue of J is negative apart from the U(1) gauge mode
// i psi, which J maps to i F = 0.
//
// Here: LOBPCG (Knyazev 2001) for the smallest algebraic eigenvalues, with
// every operation on a block of vectors done by this file's kernels on the
// handle's stream:
//   * J applies: the FP64 Jacobian SpMV (ops.cu), one launch per vector;
//   * preconditioner: one AMG V-cycle of the regularised KEO (amg.cu);
//   * block Gram matrices S T^T: per-CTA partial sums over column tiles
//     staged in shared memory, then a fixed-order sum over the CTAs
//     (deterministic);
//   * block combinations Y = C^T S and the row-wise updates;
//   * orthonormalisation by SVQB (Stathopoulos & Wu 2002): the Gram matrix
//     of the rows, scaled to a unit diagonal, is diagonalised on the host
//     and directions with negligible eigenvalues are dropped; applied twice;
//   * the gauge mode is projected out of every block.
// Only the small projected eigenproblems (at most 3 (k + guard) rows) are
// solved on the host, by cyclic Jacobi rotations.
#include <algorithm>
#include <cmath>
#include <vector>

#include "amg.cuh"
#include "nls.cuh"
#include "solver.cuh"
#include "spmv.cuh"

namespace nosh {

using namespace dev;

namespace {

constexpr int kMaxRows = 64;   // rows of a block operand
constexpr int kTile = 32;      // columns staged per pass of the Gram kernel
constexpr int kGramThreads = 256;
constexpr int kGramAcc = kMaxRows * kMaxRows / kGramThreads;  // entries per thread

// partial[blockIdx][a * p + b] = sum over this CTA's column tiles of
// S[a][i] T[b][i]; rows of S and T are contiguous with stride n.
__global__ void __launch_bounds__(kGramThreads) gram_partial(int m, int p, int64_t n, const double *__restrict__ S,
                                                             const double *__restrict__ T, double *partial) {
  __shared__ double sS[kMaxRows][kTile + 1], sT[kMaxRows][kTile + 1];
  double acc[kGramAcc];
#pragma unroll
  for (int r = 0; r < kGramAcc; r++) acc[r] = 0.0;
  const int mp = m * p;
  for (int64_t c0 = (int64_t)blockIdx.x * kTile; c0 < n; c0 += (int64_t)gridDim.x * kTile) {
    __syncthreads();
    for (int q = threadIdx.x; q < kMaxRows * kTile; q += kGramThreads) {
      const int a = q / kTile, c = q % kTile;
      const int64_t i = c0 + c;
      if (a < m) sS[a][c] = i < n ? S[(int64_t)a * n + i] : 0.0;
      if (a < p) sT[a][c] = i < n ? T[(int64_t)a * n + i] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kGramAcc; r++) {
      const int e = threadIdx.x + r * kGramThreads;
      if (e < mp) {
        const int a = e / p, b = e % p;
        double s = 0.0;
#pragma unroll 8
        for (int c = 0; c < kTile; c++) s += sS[a][c] * sT[b][c];
        acc[r] += s;
      }
    }
  }
#pragma unroll
  for (int r = 0; r < kGramAcc; r++) {
    const int e = threadIdx.x + r * kGramThreads;
    if (e < mp) partial[(int64_t)blockIdx.x * mp + e] = acc[r];
  }
}

// G[e] = sum over the CTAs of partial[.][e], in CTA order
__global__ void gram_finish(int mp, int blocks, const double *__restrict__ partial, double *G) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= mp) return;
  double s = 0.0;
  for (int b = 0; b < blocks; b++) s += partial[(int64_t)b * mp + e];
  G[e] = s;
}

// Y[j][i] = beta Y[j][i] + sum_a C[a * q + j] S[a][i] for j < q (C: m x q,
// row major, device); outputs in chunks of 16 per pass.
constexpr int kCombOut = 16;
__global__ void combine_rows(int m, int q, int64_t n, const double *__restrict__ C, const double *__restrict__ S,
                             double beta, double *__restrict__ Y) {
  __shared__ double sC[kMaxRows * kMaxRows];
  for (int e = threadIdx.x; e < m * q; e += blockDim.x) sC[e] = C[e];
  __syncthreads();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    for (int j0 = 0; j0 < q; j0 += kCombOut) {
      double acc[kCombOut];
#pragma unroll
      for (int j = 0; j < kCombOut; j++) acc[j] = 0.0;
      for (int a = 0; a < m; a++) {
        const double s = S[(int64_t)a * n + i];
#pragma unroll
        for (int j = 0; j < kCombOut; j++)
          if (j0 + j < q) acc[j] += sC[a * q + j0 + j] * s;
      }
#pragma unroll
      for (int j = 0; j < kCombOut; j++)
        if (j0 + j < q) {
          double *y = Y + (int64_t)(j0 + j) * n + i;
          *y = beta == 0.0 ? acc[j] : beta * *y + acc[j];
        }
    }
  }
}

// Y[j][i] = a[j] A[j][i] + b[j] B[j][i]  (row-wise axpby; a, b device)
__global__ void rows_axpby(int rows, int64_t n, const double *__restrict__ a, const double *__restrict__ A,
                           const double *__restrict__ b, const double *__restrict__ B, double *__restrict__ Y) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)rows * n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(t / n);
    Y[t] = a[j] * A[t] + (B ? b[j] * B[t] : 0.0);
  }
}

// V[j][i] -= c[j] U[i]  (projection of each row off one unit vector U)
__global__ void rows_minus_outer(int rows, int64_t n, const double *__restrict__ c, const double *__restrict__ U,
                                 double *__restrict__ V) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)rows * n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(t / n);
    V[t] -= c[j] * U[t - (int64_t)j * n];
  }
}

// u = i psi (interleaved complex)
__global__ void gauge_vector(int64_t N, const double *__restrict__ psi, double *__restrict__ u) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < N; k += (int64_t)gridDim.x * blockDim.x) {
    u[2 * k] = -psi[2 * k + 1];
    u[2 * k + 1] = psi[2 * k];
  }
}

inline int elem_grid(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>(div_up(n, 256), kNumSMs * 8)); }

// symmetric A (m x m, row major) -> ascending eigenvalues w and eigenvectors
// as the columns of V (cyclic Jacobi rotations)
void jacobi_eig(std::vector<double> A, int m, std::vector<double> &w, std::vector<double> &V) {
  V.assign((size_t)m * m, 0.0);
  for (int i = 0; i < m; i++) V[(size_t)i * m + i] = 1.0;
  for (int sweep = 0; sweep < 100; sweep++) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < m; i++)
      for (int j = 0; j < m; j++) (i == j ? tot : off) += A[(size_t)i * m + j] * A[(size_t)i * m + j];
    if (off <= 1e-30 * (tot + off)) break;
    for (int p = 0; p < m; p++)
      for (int q = p + 1; q < m; q++) {
        const double apq = A[(size_t)p * m + q];
        if (apq == 0.0) continue;
        const double th = (A[(size_t)q * m + q] - A[(size_t)p * m + p]) / (2.0 * apq);
        const double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int r = 0; r < m; r++) {
          const double a = A[(size_t)r * m + p], b = A[(size_t)r * m + q];
          A[(size_t)r * m + p] = c * a - s * b;
          A[(size_t)r * m + q] = s * a + c * b;
        }
        for (int r = 0; r < m; r++) {
          const double a = A[(size_t)p * m + r], b = A[(size_t)q * m + r];
          A[(size_t)p * m + r] = c * a - s * b;
          A[(size_t)q * m + r] = s * a + c * b;
        }
        for (int r = 0; r < m; r++) {
          const double a = V[(size_t)r * m + p], b = V[(size_t)r * m + q];
          V[(size_t)r * m + p] = c * a - s * b;
          V[(size_t)r * m + q] = s * a + c * b;
        }
      }
  }
  std::vector<int> order(m);
  for (int i = 0; i < m; i++) order[i] = i;
  std::sort(order.begin(), order.end(), [&](int a, int b) { return A[(size_t)a * m + a] < A[(size_t)b * m + b]; });
  w.resize(m);
  std::vector<double> Vs((size_t)m * m);
  for (int j = 0; j < m; j++) {
    w[j] = A[(size_t)order[j] * m + order[j]];
    for (int r = 0; r < m; r++) Vs[(size_t)r * m + j] = V[(size_t)r * m + order[j]];
  }
  V.swap(Vs);
}

// Device block algebra of one LOBPCG run (n-long rows, contiguous).
struct BlockOps {
  NlsImpl &s;
  int64_t n;
  int gram_blocks;
  DevBuf<double> partial, G, C;
  std::vector<double> hG;
  BlockOps(NlsImpl &nls, int64_t len) : s(nls), n(len) {
    gram_blocks = (int)std::max<int64_t>(1, std::min<int64_t>(div_up(n, kTile), 2 * kNumSMs));
    partial.alloc((size_t)gram_blocks * kMaxRows * kMaxRows);
    G.alloc(kMaxRows * kMaxRows);
    C.alloc(kMaxRows * kMaxRows);
  }
  // host G (m x p) = S T^T
  const std::vector<double> &gram(const double *S, int m, const double *T, int p) {
    NOSH_CHECK(m >= 1 && p >= 1 && m <= kMaxRows && p <= kMaxRows, NOSH_ERR_INVALID, "block too wide");
    gram_partial<<<gram_blocks, kGramThreads, 0, s.stream>>>(m, p, n, S, T, partial.p);
    gram_finish<<<div_up(m * p, 256), 256, 0, s.stream>>>(m * p, gram_blocks, partial.p, G.p);
    s.launch_count += 2;
    NOSH_CUDA(cudaGetLastError());
    hG.resize((size_t)m * p);
    NOSH_CUDA(cudaMemcpyAsync(hG.data(), G.p, hG.size() * sizeof(double), cudaMemcpyDeviceToHost, s.stream));
    s.sync();
    return hG;
  }
  // Y (q rows) = beta Y + Cm^T S (Cm: m x q host, row major); Y must not
  // alias S
  void combine(const double *S, int m, const std::vector<double> &Cm, int q, double *Y, double beta = 0.0) {
    NOSH_CHECK(m <= kMaxRows && q <= kMaxRows, NOSH_ERR_INVALID, "block too wide");
    NOSH_CUDA(cudaMemcpyAsync(C.p, Cm.data(), (size_t)m * q * sizeof(double), cudaMemcpyHostToDevice, s.stream));
    combine_rows<<<elem_grid(n), 256, 0, s.stream>>>(m, q, n, C.p, S, beta, Y);
    ++s.launch_count;
    NOSH_CUDA(cudaGetLastError());
    // the coefficient buffer is reused by the next call: wait for this one
    s.sync();
  }
  void axpby(int rows, const std::vector<double> &a, const double *A, const std::vector<double> &b, const double *B,
             double *Y) {
    std::vector<double> ab(a);
    ab.insert(ab.end(), b.begin(), b.end());
    NOSH_CUDA(cudaMemcpyAsync(C.p, ab.data(), ab.size() * sizeof(double), cudaMemcpyHostToDevice, s.stream));
    rows_axpby<<<elem_grid((int64_t)rows * n), 256, 0, s.stream>>>(rows, n, C.p, A, C.p + rows, B, Y);
    ++s.launch_count;
    NOSH_CUDA(cudaGetLastError());
    s.sync();
  }
  // V (rows) -= (V U^T) U for a unit row U
  void project_off(double *V, int rows, const double *U) {
    const std::vector<double> c = gram(V, rows, U, 1);
    NOSH_CUDA(cudaMemcpyAsync(C.p, c.data(), rows * sizeof(double), cudaMemcpyHostToDevice, s.stream));
    rows_minus_outer<<<elem_grid((int64_t)rows * n), 256, 0, s.stream>>>(rows, n, C.p, U, V);
    ++s.launch_count;
    NOSH_CUDA(cudaGetLastError());
    s.sync();
  }
  // rows scaled to unit norm (zero rows stay zero)
  void unit_rows(double *V, int rows) {
    if (rows == 0) return;
    const std::vector<double> g = gram(V, rows, V, rows);
    std::vector<double> a(rows), z(rows, 0.0);
    for (int j = 0; j < rows; j++) {
      const double d = g[(size_t)j * rows + j];
      a[j] = d > 0.0 ? 1.0 / std::sqrt(d) : 0.0;
    }
    axpby(rows, a, V, z, nullptr, V);
  }
  // SVQB: the rows of S (m) -> an orthonormal basis Q of their span (kept
  // rows returned); Q must not alias S
  int svqb(const double *S, int m, double *Q) {
    const std::vector<double> g = gram(S, m, S, m);
    std::vector<double> d(m), H((size_t)m * m);
    for (int a = 0; a < m; a++) {
      const double v = g[(size_t)a * m + a];
      d[a] = v > 0.0 ? 1.0 / std::sqrt(v) : 0.0;
    }
    for (int a = 0; a < m; a++)
      for (int b = 0; b < m; b++)
        H[(size_t)a * m + b] = 0.5 * (g[(size_t)a * m + b] + g[(size_t)b * m + a]) * d[a] * d[b];
    std::vector<double> w, V;
    jacobi_eig(H, m, w, V);
    const double wmax = std::max(w.empty() ? 0.0 : w.back(), 0.0);
    std::vector<int> keep;
    for (int j = 0; j < m; j++)
      if (w[j] > 1e-20 * wmax && w[j] > 0.0) keep.push_back(j);
    const int q = (int)keep.size();
    if (q == 0) return 0;
    std::vector<double> K((size_t)m * q);
    for (int a = 0; a < m; a++)
      for (int jj = 0; jj < q; jj++) {
        const int j = keep[jj];
        K[(size_t)a * q + jj] = d[a] * V[(size_t)a * m + j] / std::sqrt(w[j]);
      }
    combine(S, m, K, q, Q);
    return q;
  }
  // Ritz pairs of span(S) (orthonormal rows) with AS = J S: ascending
  // values w and the coefficient matrix Cs (m x m, columns = vectors)
  void ritz(const double *S, const double *AS, int m, std::vector<double> &w, std::vector<double> &Cs) {
    const std::vector<double> h = gram(S, m, AS, m);
    std::vector<double> H((size_t)m * m);
    for (int a = 0; a < m; a++)
      for (int b = 0; b < m; b++) H[(size_t)a * m + b] = 0.5 * (h[(size_t)a * m + b] + h[(size_t)b * m + a]);
    jacobi_eig(H, m, w, Cs);
  }
};

}  // namespace

int lowest_eigenpairs(NlsImpl &s, const double *psi_dev, double g, double mu, int k, double tol, int maxit,
                      int guard, bool deflate_gauge, uint64_t seed, double *values, double *vectors_dev) {
  const int64_t N = s.N, n = 2 * N;
  if (guard < 0) guard = std::max(2, k);
  const int mb = k + guard;
  NOSH_CHECK(k >= 1 && 3 * mb <= kMaxRows && 3 * mb + 1 < n, NOSH_ERR_INVALID,
             "need 1 <= k, 3 (k + guard) <= 64 and 3 (k + guard) + 1 < 2N");
  // FP64 operators at psi
  s.jac_rebuild(psi_dev, g, mu);
  s.reg_rebuild(psi_dev, g, mu);
  ensure_preconditioner(s).refresh<double>();
  BlockOps B(s, n);
  DevBuf<double> U(n), X((size_t)mb * n), AX((size_t)mb * n), P((size_t)mb * n), R((size_t)mb * n);
  DevBuf<double> S((size_t)3 * mb * n), Q((size_t)3 * mb * n), AS((size_t)3 * mb * n);
  DevBuf<double> Xn((size_t)mb * n);
  const double *Ug = nullptr;
  if (deflate_gauge) {
    gauge_vector<<<elem_grid(N), 256, 0, s.stream>>>(N, psi_dev, U.p);
    ++s.launch_count;
    NOSH_CUDA(cudaGetLastError());
    const double nu = std::sqrt(B.gram(U.p, 1, U.p, 1)[0]);
    if (nu > 0.0) {
      B.axpby(1, {1.0 / nu}, U.p, {0.0}, nullptr, U.p);
      Ug = U.p;
    }
  }
  auto proj = [&](double *V, int rows) {
    if (Ug && rows > 0) B.project_off(V, rows, Ug);
  };
  auto applyJ = [&](const double *V, double *AV, int rows) {
    for (int j = 0; j < rows; j++) s.jac_apply<double>(V + (size_t)j * n, AV + (size_t)j * n);
    NOSH_CUDA(cudaGetLastError());
  };
  auto applyT = [&](const double *V, double *TV, int rows) {
    for (int j = 0; j < rows; j++) s.amg->apply<double>(V + (size_t)j * n, TV + (size_t)j * n);
    NOSH_CUDA(cudaGetLastError());
  };
  // random start (splitmix64, uniform in [-0.5, 0.5)), projected and
  // orthonormalised
  {
    std::vector<double> h((size_t)mb * n);
    uint64_t st = seed;
    for (double &x : h) {
      uint64_t z = (st += 0x9E3779B97F4A7C15ULL);
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
      x = (double)((z ^ (z >> 31)) >> 11) * 0x1.0p-53 - 0.5;
    }
    NOSH_CUDA(cudaMemcpyAsync(S.p, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, s.stream));
    s.sync();
  }
  proj(S.p, mb);
  int nx = B.svqb(S.p, mb, Q.p);
  nx = B.svqb(Q.p, nx, X.p);
  NOSH_CHECK(nx == mb, NOSH_ERR_BREAKDOWN, "LOBPCG: the random start block is rank deficient");
  applyJ(X.p, AX.p, nx);
  std::vector<double> lam, Cs;
  B.ritz(X.p, AX.p, nx, lam, Cs);
  B.combine(X.p, nx, Cs, nx, Q.p);
  NOSH_CUDA(cudaMemcpyAsync(X.p, Q.p, (size_t)nx * n * sizeof(double), cudaMemcpyDeviceToDevice, s.stream));
  B.combine(AX.p, nx, Cs, nx, Q.p);
  NOSH_CUDA(cudaMemcpyAsync(AX.p, Q.p, (size_t)nx * n * sizeof(double), cudaMemcpyDeviceToDevice, s.stream));
  double jnorm = 0.0;
  {
    const std::vector<double> ga = B.gram(AX.p, nx, AX.p, nx);
    for (int j = 0; j < nx; j++) jnorm = std::max(jnorm, std::sqrt(std::max(ga[(size_t)j * nx + j], 0.0)));
  }
  int np = 0;  // rows of P
  int it = 0;
  for (it = 1; it <= maxit; it++) {
    // R = AX - lam X and its row norms
    std::vector<double> one(nx, 1.0), mlam(nx);
    for (int j = 0; j < nx; j++) {
      mlam[j] = -lam[j];
      jnorm = std::max(jnorm, std::fabs(lam[j]));
    }
    B.axpby(nx, one, AX.p, mlam, X.p, R.p);
    const std::vector<double> gr = B.gram(R.p, nx, R.p, nx);
    bool done = true;
    for (int j = 0; j < std::min(k, nx); j++)
      if (!(std::sqrt(std::max(gr[(size_t)j * nx + j], 0.0)) <= tol * jnorm)) done = false;
    if (done) break;
    // S = [X; unit(T R); unit(P)]
    NOSH_CUDA(cudaMemcpyAsync(S.p, X.p, (size_t)nx * n * sizeof(double), cudaMemcpyDeviceToDevice, s.stream));
    double *W = S.p + (size_t)nx * n;
    applyT(R.p, W, nx);
    proj(W, nx);
    B.unit_rows(W, nx);
    int m = 2 * nx;
    if (np > 0) {
      NOSH_CUDA(cudaMemcpyAsync(S.p + (size_t)m * n, P.p, (size_t)np * n * sizeof(double), cudaMemcpyDeviceToDevice,
                                s.stream));
      B.unit_rows(S.p + (size_t)m * n, np);
      m += np;
    }
    proj(S.p, m);
    int q = B.svqb(S.p, m, Q.p);
    NOSH_CHECK(q >= nx, NOSH_ERR_BREAKDOWN, "LOBPCG: the search space collapsed");
    q = B.svqb(Q.p, q, S.p);
    proj(S.p, q);
    applyJ(S.p, AS.p, q);
    std::vector<double> th;
    B.ritz(S.p, AS.p, q, th, Cs);
    const int keep = std::min(mb, q);
    std::vector<double> Ck((size_t)q * keep);
    for (int a = 0; a < q; a++)
      for (int j = 0; j < keep; j++) Ck[(size_t)a * keep + j] = Cs[(size_t)a * q + j];
    B.combine(S.p, q, Ck, keep, Xn.p);
    B.combine(AS.p, q, Ck, keep, AX.p);
    // P = Xn - (Xn X^T) X: the part of the update outside span(X)
    const std::vector<double> gx = B.gram(X.p, nx, Xn.p, keep);  // nx x keep: <x_a, xn_j>
    std::vector<double> Cp((size_t)nx * keep);
    for (int a = 0; a < nx; a++)
      for (int j = 0; j < keep; j++) Cp[(size_t)a * keep + j] = -gx[(size_t)a * keep + j];
    NOSH_CUDA(cudaMemcpyAsync(P.p, Xn.p, (size_t)keep * n * sizeof(double), cudaMemcpyDeviceToDevice, s.stream));
    B.combine(X.p, nx, Cp, keep, P.p, 1.0);
    np = keep;
    NOSH_CUDA(cudaMemcpyAsync(X.p, Xn.p, (size_t)keep * n * sizeof(double), cudaMemcpyDeviceToDevice, s.stream));
    nx = keep;
    lam.assign(th.begin(), th.begin() + keep);
  }
  s.sync();
  for (int j = 0; j < k; j++) {
    NOSH_CHECK(std::isfinite(lam[j]), NOSH_ERR_NAN, "LOBPCG produced a NaN eigenvalue");
    values[j] = lam[j];
  }
  if (vectors_dev)
    NOSH_CUDA(cudaMemcpyAsync(vectors_dev, X.p, (size_t)k * n * sizeof(double), cudaMemcpyDefault, s.stream));
  s.sync();
  return std::min(it, maxit);
}

}  // namespace nosh
