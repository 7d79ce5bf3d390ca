// Aggregation AMG preconditioner for the regularised KEO
// (keo_regularized, src/keo_regularized.cpp).  The reference applies one
// MueLu SA-AMG V-cycle with 2 equations per node (:292-336); this is a
// GB300-native aggregation AMG with the same role:
//
//  * structure (aggregates, coarse graphs, Galerkin plans) is built on the
//    host at the first rebuild and reused afterwards (MueLu "reuse: full"
//    keeps the hierarchy too); every rebuild refreshes all numeric values on
//    the GPU from the current K_reg;
//  * plain (unsmoothed) aggregation with 2x2-block identity prolongation:
//    every level keeps the fine level's compact format -- one complex value
//    per off-diagonal block plus a symmetric 2x2 diagonal block -- and the
//    Galerkin product P^T A P is a deterministic segmented sum;
//  * block-Jacobi Chebyshev smoothing (same polynomial before and after the
//    coarse correction, so the V-cycle is a fixed SPD operator as MINRES
//    requires); Gershgorin bound for lambda_max(D^-1 A);
//  * coarsest level: dense inverse (Gauss-Jordan, FP64) applied as a matvec.
#include <algorithm>
#include <cmath>
#include <complex>
#include <numeric>
#include <type_traits>

#include "amg.cuh"
#include "spmv.cuh"

namespace nosh {

using namespace dev;

namespace {

constexpr int64_t kTailMax = 1024;   // levels this small run in one CTA

struct HostLevel {
  int64_t n = 0;
  std::vector<int32_t> rp, ci;  // off-diagonal CSR
  std::vector<std::complex<double>> off;  // values (strength / next level)
  std::vector<double> dia;                // 3 per node
  // transfer to the next level
  std::vector<int32_t> agg;               // n
  std::vector<int32_t> mem_ptr, mem_idx;  // coarse node -> fine nodes
  std::vector<int32_t> seg_ptr, seg_idx;  // coarse nonzero -> fine nonzeros
  std::vector<int32_t> intra_ptr, intra_idx;  // coarse node -> fine intra nnz
  // independent systems (batched solves): nodes of system s are
  // [soff[s], soff[s+1]); a single system has soff = {0, n}
  std::vector<int64_t> soff;
};

int64_t max_block(const HostLevel &L) {
  int64_t m = 0;
  for (size_t s = 0; s + 1 < L.soff.size(); s++) m = std::max(m, L.soff[s + 1] - L.soff[s]);
  return m;
}

// Greedy aggregation on the strong graph (deterministic, vertex order):
// 1) a vertex whose strong neighbours are all free roots an aggregate with
//    them; 2) every remaining vertex joins the aggregate it is most strongly
//    connected to; 3) isolated leftovers become singletons.
int64_t aggregate(const HostLevel &L, std::vector<int32_t> &agg, double theta) {
  const int64_t n = L.n;
  std::vector<double> scale(n);
  for (int64_t i = 0; i < n; i++) scale[i] = std::max(0.5 * (L.dia[3 * i] + L.dia[3 * i + 1]), 1e-300);
  auto strong = [&](int64_t i, int64_t k) {
    const int64_t j = L.ci[k];
    return std::abs(L.off[k]) >= theta * std::sqrt(scale[i] * scale[j]);
  };
  agg.assign(n, -1);
  int64_t na = 0;
  for (int64_t i = 0; i < n; i++) {
    if (agg[i] >= 0) continue;
    bool free = true;
    for (int64_t k = L.rp[i]; k < L.rp[i + 1] && free; k++)
      if (strong(i, k) && agg[L.ci[k]] >= 0) free = false;
    if (!free) continue;
    agg[i] = (int32_t)na;
    for (int64_t k = L.rp[i]; k < L.rp[i + 1]; k++)
      if (strong(i, k)) agg[L.ci[k]] = (int32_t)na;
    na++;
  }
  std::vector<int32_t> agg1 = agg;  // phase 2 reads phase-1 state only
  for (int64_t i = 0; i < n; i++) {
    if (agg1[i] >= 0) continue;
    double best = -1.0;
    int32_t to = -1;
    for (int64_t k = L.rp[i]; k < L.rp[i + 1]; k++) {
      const int32_t a = agg1[L.ci[k]];
      if (a >= 0 && std::abs(L.off[k]) > best) {
        best = std::abs(L.off[k]);
        to = a;
      }
    }
    agg[i] = to;
  }
  for (int64_t i = 0; i < n; i++)
    if (agg[i] < 0) agg[i] = (int32_t)na++;
  return na;
}

// Coarse graph + Galerkin plans for plain aggregation, and the coarse values
// (host copy, used for the next level's strength test).
void coarsen(HostLevel &F, HostLevel &C, double theta) {
  const int64_t n = F.n;
  const int64_t na = aggregate(F, F.agg, theta);
  C.n = na;
  // aggregates never cross systems (no edges between them); number them
  // system by system so every level keeps contiguous system ranges
  {
    const int64_t ns = (int64_t)F.soff.size() - 1;
    std::vector<int32_t> asys(na, 0);
    for (int64_t sy = 0; sy < ns; sy++)
      for (int64_t i = F.soff[sy]; i < F.soff[sy + 1]; i++) asys[F.agg[i]] = (int32_t)sy;
    std::vector<int32_t> order(na);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return asys[a] < asys[b]; });
    std::vector<int32_t> renum(na);
    for (int64_t q = 0; q < na; q++) renum[order[q]] = (int32_t)q;
    for (int64_t i = 0; i < n; i++) F.agg[i] = renum[F.agg[i]];
    C.soff.assign(ns + 1, 0);
    for (int64_t a = 0; a < na; a++) C.soff[asys[order[a]] + 1]++;
    for (int64_t sy = 0; sy < ns; sy++) C.soff[sy + 1] += C.soff[sy];
  }
  // members
  F.mem_ptr.assign(na + 1, 0);
  for (int64_t i = 0; i < n; i++) F.mem_ptr[F.agg[i] + 1]++;
  for (int64_t a = 0; a < na; a++) F.mem_ptr[a + 1] += F.mem_ptr[a];
  F.mem_idx.resize(n);
  {
    std::vector<int32_t> fill(F.mem_ptr.begin(), F.mem_ptr.end() - 1);
    for (int64_t i = 0; i < n; i++) F.mem_idx[fill[F.agg[i]]++] = (int32_t)i;
  }
  // coarse rows: unique neighbour aggregates
  C.rp.assign(na + 1, 0);
  std::vector<std::vector<int32_t>> rows(na);
  for (int64_t a = 0; a < na; a++) {
    auto &r = rows[a];
    for (int32_t q = F.mem_ptr[a]; q < F.mem_ptr[a + 1]; q++) {
      const int32_t i = F.mem_idx[q];
      for (int32_t k = F.rp[i]; k < F.rp[i + 1]; k++) {
        const int32_t b = F.agg[F.ci[k]];
        if (b != a) r.push_back(b);
      }
    }
    std::sort(r.begin(), r.end());
    r.erase(std::unique(r.begin(), r.end()), r.end());
    C.rp[a + 1] = C.rp[a] + (int32_t)r.size();
  }
  C.ci.resize(C.rp[na]);
  for (int64_t a = 0; a < na; a++) std::copy(rows[a].begin(), rows[a].end(), C.ci.begin() + C.rp[a]);
  // plans: each fine nonzero goes either to one coarse nonzero or to the
  // coarse diagonal of its aggregate
  const int64_t nzc = C.rp[na];
  std::vector<int32_t> target(F.rp[n]);
  std::vector<int32_t> cnt(nzc + 1, 0), icnt(na + 1, 0);
  for (int64_t i = 0; i < n; i++) {
    const int32_t a = F.agg[i];
    for (int32_t k = F.rp[i]; k < F.rp[i + 1]; k++) {
      const int32_t b = F.agg[F.ci[k]];
      if (b == a) {
        target[k] = -1;
        icnt[a + 1]++;
      } else {
        const int32_t *rb = C.ci.data() + C.rp[a], *re = C.ci.data() + C.rp[a + 1];
        const int32_t t = (int32_t)(std::lower_bound(rb, re, b) - C.ci.data());
        target[k] = t;
        cnt[t + 1]++;
      }
    }
  }
  for (int64_t t = 0; t < nzc; t++) cnt[t + 1] += cnt[t];
  for (int64_t a = 0; a < na; a++) icnt[a + 1] += icnt[a];
  F.seg_ptr = cnt;
  F.intra_ptr = icnt;
  F.seg_idx.resize(cnt[nzc]);
  F.intra_idx.resize(icnt[na]);
  {
    std::vector<int32_t> fs(cnt.begin(), cnt.end() - 1), fi(icnt.begin(), icnt.end() - 1);
    for (int64_t i = 0; i < n; i++)
      for (int32_t k = F.rp[i]; k < F.rp[i + 1]; k++) {
        if (target[k] >= 0) F.seg_idx[fs[target[k]]++] = k;
        else F.intra_idx[fi[F.agg[i]]++] = k;
      }
  }
  // coarse values (host, same arithmetic as the GPU refresh)
  C.off.assign(nzc, 0.0);
  for (int64_t t = 0; t < nzc; t++)
    for (int32_t q = F.seg_ptr[t]; q < F.seg_ptr[t + 1]; q++) C.off[t] += F.off[F.seg_idx[q]];
  C.dia.assign(3 * na, 0.0);
  for (int64_t a = 0; a < na; a++) {
    for (int32_t q = F.mem_ptr[a]; q < F.mem_ptr[a + 1]; q++) {
      const int32_t i = F.mem_idx[q];
      for (int c = 0; c < 3; c++) C.dia[3 * a + c] += F.dia[3 * i + c];
    }
    for (int32_t q = F.intra_ptr[a]; q < F.intra_ptr[a + 1]; q++) {
      const double re = F.off[F.intra_idx[q]].real();
      C.dia[3 * a] += re;
      C.dia[3 * a + 1] += re;
    }
  }
}

// ------------------------------------------------------------- kernels
// coarse off-diagonal values: sum of the fine nonzeros of each segment
template <typename T>
__global__ void rap_offdiag(int64_t nzc, const int32_t *__restrict__ ptr,
                            const int32_t *__restrict__ idx, const C2<T> *__restrict__ fine,
                            C2<T> *__restrict__ coarse) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nzc) return;
  T sr = 0, si = 0;
  for (int32_t q = ptr[t]; q < ptr[t + 1]; q++) {
    const C2<T> v = fine[idx[q]];
    sr += v.x;
    si += v.y;
  }
  coarse[t] = C2<T>{sr, si};
}

// coarse diagonal blocks: member diagonal blocks + real parts of the
// intra-aggregate couplings (their imaginary parts cancel pairwise)
template <typename T>
__global__ void rap_diag(int64_t na, const int32_t *__restrict__ mptr,
                         const int32_t *__restrict__ midx, const int32_t *__restrict__ iptr,
                         const int32_t *__restrict__ iidx, const T *__restrict__ fdia,
                         const C2<T> *__restrict__ foff, T *__restrict__ cdia) {
  const int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (a >= na) return;
  T d0 = 0, d1 = 0, d2 = 0;
  for (int32_t q = mptr[a]; q < mptr[a + 1]; q++) {
    const int32_t i = midx[q];
    d0 += fdia[3 * i];
    d1 += fdia[3 * i + 1];
    d2 += fdia[3 * i + 2];
  }
  for (int32_t q = iptr[a]; q < iptr[a + 1]; q++) {
    const T re = foff[iidx[q]].x;
    d0 += re;
    d1 += re;
  }
  cdia[3 * a] = d0;
  cdia[3 * a + 1] = d1;
  cdia[3 * a + 2] = d2;
}

// inverse diagonal blocks and the Gershgorin bound of lambda_max(D^-1 A):
// 1 + ||D_i^-1||_2 sum_j |a_ij|, reduced by max over rows (arithmetic in T)
// sum_j |a_ij| per row (the loop dinv_gershgorin runs without rowabs)
template <typename T>
__global__ void row_abs_sums(int64_t n, const int32_t *__restrict__ rp, const C2<T> *__restrict__ off,
                             T *__restrict__ out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  T s = 0;
  for (int32_t k = rp[i]; k < rp[i + 1]; k++) {
    const C2<T> v = off[k];
    s += sqrt(v.x * v.x + v.y * v.y);
  }
  out[i] = s;
}

// (rowabs: the rows' sums of |a_ij| when known, else summed here)
template <typename T>
__global__ void dinv_gershgorin(int64_t n, const int32_t *__restrict__ rp,
                                const C2<T> *__restrict__ off, const T *__restrict__ dia,
                                T *__restrict__ dinv, unsigned long long *lmax_bits, int *err,
                                const T *__restrict__ rowabs = nullptr) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double bound = 0.0;
  if (i < n) {
    const T a = dia[3 * i], d = dia[3 * i + 1], b = dia[3 * i + 2];
    const T det = a * d - b * b;
    dinv[3 * i] = d / det;
    dinv[3 * i + 1] = a / det;
    dinv[3 * i + 2] = -b / det;
    const T lmin = (T)0.5 * (a + d) - sqrt((T)0.25 * (a - d) * (a - d) + b * b);
    T s = 0;
    if (rowabs) {
      s = rowabs[i];
    } else {
      for (int32_t k = rp[i]; k < rp[i + 1]; k++) {
        const C2<T> v = off[k];
        s += sqrt(v.x * v.x + v.y * v.y);
      }
    }
    bound = (lmin > 0 && det > 0) ? 1.0 + (double)(s / lmin) : 1e300;
    // a diagonal block that is not positive definite: the operator is not
    // SPD (a g < 0 regularisation), so neither is the V-cycle
    if (!(lmin > 0 && det > 0)) atomicOr(err, 32);
  }
  // max over the block, then one atomic per block (non-negative doubles
  // order like their bit patterns)
  __shared__ double sm[32];
  double v = bound;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    v = threadIdx.x < (blockDim.x >> 5) ? sm[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (threadIdx.x == 0) atomicMax(lmax_bits, (unsigned long long)__double_as_longlong(v));
  }
}

// Chebyshev coefficients from lambda_max: c[0] = 1/theta, then per step
// k >= 1 the pair (rho_k rho_{k-1}, 2 rho_k / delta).
template <typename T>
__global__ void cheb_coeffs(const unsigned long long *lmax_bits, int deg, double ratio, T *coef,
                            double *lmax_out) {
  // smoothing interval [lmax / ratio, 1.1 lmax]
  const double lmax = 1.1 * __longlong_as_double((long long)*lmax_bits);
  const double lmin = lmax / (1.1 * ratio);
  const double theta = 0.5 * (lmax + lmin), delta = 0.5 * (lmax - lmin);
  const double sigma = theta / delta;
  double rho = 1.0 / sigma;
  coef[0] = (T)(1.0 / theta);
  for (int k = 1; k < deg; k++) {
    const double rn = 1.0 / (2.0 * sigma - rho);
    coef[2 * k] = (T)(rn * rho);
    coef[2 * k + 1] = (T)(2.0 * rn / delta);
    rho = rn;
  }
  *lmax_out = lmax;
}

// ---- smoother building blocks (shared by the grid kernels and the tail)
// d = c0 D^-1 b, x = d  (first Chebyshev step from x = 0)
template <typename T>
__device__ __forceinline__ void cheb_first_elem(int64_t i, const T *dinv, T c0, C2<T> bi, C2<T> *d,
                                                C2<T> *x) {
  const T a = dinv[3 * i], e = dinv[3 * i + 1], f = dinv[3 * i + 2];
  const C2<T> di{c0 * (a * bi.x + f * bi.y), c0 * (f * bi.x + e * bi.y)};
  d[i] = di;
  x[i] = di;
}

// Chebyshev step k given (sr, si) = (offdiag A x_in)_i:
// r = D^-1 (b - A x_in), d = c1 d + c2 r (d = c0 r for k == 0), x_out = x_in + d
template <typename T>
struct ChebPre {
  C2<T> xi, bi, dold;
  T d0r, d0i, d1b, a, e, f;
};
template <typename T>
__device__ __forceinline__ ChebPre<T> cheb_load(int64_t i, int k, const T *dia, const T *dinv, const C2<T> *b,
                                                const C2<T> *xin, const C2<T> *d) {
  ChebPre<T> p;
  p.xi = xin[i];
  p.bi = b[i];
  p.d0r = dia[3 * i];
  p.d0i = dia[3 * i + 1];
  p.d1b = dia[3 * i + 2];
  p.a = dinv[3 * i];
  p.e = dinv[3 * i + 1];
  p.f = dinv[3 * i + 2];
  p.dold = k == 0 ? C2<T>{0, 0} : d[i];
  return p;
}
template <typename T>
__device__ __forceinline__ C2<T> cheb_apply(int64_t i, int k, T sr, T si, const ChebPre<T> &p, const T *coef,
                                            C2<T> *d, C2<T> *xout) {
  const T rr = p.bi.x - (sr + p.d0r * p.xi.x + p.d1b * p.xi.y);
  const T ri = p.bi.y - (si + p.d1b * p.xi.x + p.d0i * p.xi.y);
  const T zr = p.a * rr + p.f * ri, zi = p.f * rr + p.e * ri;
  C2<T> dn;
  if (k == 0) {
    dn = C2<T>{coef[0] * zr, coef[0] * zi};
  } else {
    const T c1 = coef[2 * k], c2 = coef[2 * k + 1];
    dn = C2<T>{c1 * p.dold.x + c2 * zr, c1 * p.dold.y + c2 * zi};
  }
  d[i] = dn;
  const C2<T> xo{p.xi.x + dn.x, p.xi.y + dn.y};
  xout[i] = xo;
  return xo;
}
template <typename T>
__device__ __forceinline__ C2<T> cheb_elem(int64_t i, int k, T sr, T si, const T *dia, const T *dinv,
                                           const T *coef, const C2<T> *b, const C2<T> *xin, C2<T> *d,
                                           C2<T> *xout) {
  return cheb_apply<T>(i, k, sr, si, cheb_load<T>(i, k, dia, dinv, b, xin, d), coef, d, xout);
}

template <typename T>
__global__ void cheb_first(int64_t n, const T *__restrict__ dinv, const T *__restrict__ coef,
                           const C2<T> *__restrict__ b, C2<T> *__restrict__ d,
                           C2<T> *__restrict__ x) {
  dep_sync();
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  cheb_first_elem<T>(i, dinv, coef[0], b[i], d, x);
}

// MINRES head fused with the first Chebyshev step of the fine level:
// r_new = J z / beta - (beta/oldb) r_old - (alfa/beta) r_cur over r_old, then
// d = c0 D^-1 r_new, x = d
template <typename T>
__global__ void lanczos_first(int64_t n, const MinresScalars *__restrict__ s,
                              const C2<T> *__restrict__ u, C2<T> *__restrict__ r_old,
                              const C2<T> *__restrict__ r_cur, const T *__restrict__ dinv,
                              const T *__restrict__ coef, C2<T> *__restrict__ d, C2<T> *__restrict__ x) {
  dep_sync();
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n || s->done >= 2) return;
  const T *la = lanczos_coef<T>(s);
  const T a = la[0], bb = la[1], c = la[2];
  const C2<T> ui = u[i], ro = r_old[i], rc = r_cur[i];
  const C2<T> bi{a * ui.x - bb * ro.x - c * rc.x, a * ui.y - bb * ro.y - c * rc.y};
  r_old[i] = bi;
  cheb_first_elem<T>(i, dinv, coef[0], bi, d, x);
}

// Chebyshev step with SpMV (grid kernel epilogue)
template <typename T>
struct ChebOp {
  static constexpr bool kReduce = false;
  const T *dia, *dinv, *coef;
  int step;
  const C2<T> *b, *xin;
  C2<T> *d, *xout;
  const int *halt = nullptr;
  using Pre = ChebPre<T>;
  __device__ Pre load(int i) const { return cheb_load<T>(i, step, dia, dinv, b, xin, d); }
  __device__ double finish(int i, T sr, T si, const Pre &p) const {
    cheb_apply<T>(i, step, sr, si, p, coef, d, xout);
    return 0.0;
  }
};

// Last post-smoothing step of the fine level inside MINRES: also reduces
// <r_new, z_new> and, in the finishing thread, advances the Givens recurrence.
template <typename T>
struct ChebMinresOp {
  static constexpr bool kReduce = true;
  static constexpr bool kHook = true;
  const T *dia, *dinv, *coef;
  int step;
  const C2<T> *b, *xin;
  C2<T> *d, *xout;
  MinresScalars *s;
  const int *halt = nullptr;
  using Pre = ChebPre<T>;
  __device__ Pre load(int i) const { return cheb_load<T>(i, step, dia, dinv, b, xin, d); }
  __device__ double finish(int i, T sr, T si, const Pre &p) const {
    const C2<T> z = cheb_apply<T>(i, step, sr, si, p, coef, d, xout);
    return (double)p.bi.x * (double)z.x + (double)p.bi.y * (double)z.y;
  }
  __device__ void hook(double total) const { minres_advance(s, total); }
};

// res = b - A x
template <typename T>
struct ResidOp {
  static constexpr bool kReduce = false;
  const T *dia;
  const C2<T> *b, *x;
  C2<T> *res;
  const int *halt = nullptr;
  struct Pre {
    C2<T> xi, bi;
    T d0r, d0i, d1b;
  };
  __device__ Pre load(int i) const { return Pre{x[i], b[i], dia[3 * i], dia[3 * i + 1], dia[3 * i + 2]}; }
  __device__ double finish(int i, T sr, T si, const Pre &p) const {
    res[i] = C2<T>{p.bi.x - (sr + p.d0r * p.xi.x + p.d1b * p.xi.y),
                   p.bi.y - (si + p.d1b * p.xi.x + p.d0i * p.xi.y)};
    return 0.0;
  }
};

// Restriction: aggregate sums of the finer level's residual, a half-warp
// per aggregate (lanes take every 16th member, then a shuffle tree), so the
// coarse levels' few thousand aggregates spread over the whole GPU instead
// of a few dozen CTAs each walking its members serially.
constexpr int kAggLanes = 16;
template <typename T>
__device__ __forceinline__ C2<T> aggregate_sum(int64_t a, int64_t na, int li, const int32_t *__restrict__ mptr,
                                               const int32_t *__restrict__ midx, const C2<T> *__restrict__ r) {
  T sr = 0, si = 0;
  if (a < na)
    for (int32_t q = mptr[a] + li; q < mptr[a + 1]; q += kAggLanes) {
      const C2<T> v = r[midx[q]];
      sr += v.x;
      si += v.y;
    }
#pragma unroll
  for (int o = kAggLanes / 2; o > 0; o >>= 1) {
    sr += __shfl_xor_sync(0xffffffffu, sr, o);
    si += __shfl_xor_sync(0xffffffffu, si, o);
  }
  return C2<T>{sr, si};
}

template <typename T>
__global__ void restrict_kernel(int64_t na, const int32_t *__restrict__ mptr,
                                const int32_t *__restrict__ midx, const C2<T> *__restrict__ r,
                                C2<T> *__restrict__ rc, const int *halt) {
  dep_sync();
  if (halt && *halt >= 2) return;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t a = t / kAggLanes;
  const int li = (int)(t % kAggLanes);
  const C2<T> b = aggregate_sum<T>(a, na, li, mptr, midx, r);
  if (a < na && li == 0) rc[a] = b;
}

// restriction fused with the coarse level's first Chebyshev step
template <typename T>
__global__ void restrict_first(int64_t na, const int32_t *__restrict__ mptr,
                               const int32_t *__restrict__ midx, const C2<T> *__restrict__ r,
                               C2<T> *__restrict__ rc, const T *__restrict__ dinv,
                               const T *__restrict__ coef, C2<T> *__restrict__ d,
                               C2<T> *__restrict__ x, const int *halt) {
  dep_sync();
  if (halt && *halt >= 2) return;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t a = t / kAggLanes;
  const int li = (int)(t % kAggLanes);
  const C2<T> b = aggregate_sum<T>(a, na, li, mptr, midx, r);
  if (a < na && li == 0) {
    rc[a] = b;
    cheb_first_elem<T>(a, dinv, coef[0], b, d, x);
  }
}

template <typename T>
__global__ void prolong_kernel(int64_t n, const int32_t *__restrict__ agg,
                               const C2<T> *__restrict__ xc, C2<T> *__restrict__ x, const int *halt) {
  dep_sync();
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n || (halt && *halt >= 2)) return;
  const C2<T> c = xc[agg[i]];
  C2<T> v = x[i];
  v.x += c.x;
  v.y += c.y;
  x[i] = v;
}

// Dense real matrix (m = 2n) of the coarsest level from its compact form.
template <typename T>
__global__ void coarse_dense(int64_t n, const int32_t *__restrict__ rp, const int32_t *__restrict__ ci,
                             const C2<T> *__restrict__ off, const T *__restrict__ dia,
                             const int32_t *__restrict__ bstart, const int64_t *__restrict__ rowoff,
                             const int32_t *__restrict__ bdim, double *A) {
  // the coarsest level is block diagonal (one block per system): node i's
  // two real rows live in its block's packed dense matrix
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t m = bdim[2 * i];
  const int64_t s0 = bstart[2 * i];  // first real row of the block
  double *r0 = A + rowoff[2 * i], *r1 = A + rowoff[2 * i + 1];
  for (int64_t j = 0; j < m; j++) {
    r0[j] = 0.0;
    r1[j] = 0.0;
  }
  const int64_t li = 2 * i - s0;
  r0[li] = dia[3 * i];
  r0[li + 1] = dia[3 * i + 2];
  r1[li] = dia[3 * i + 2];
  r1[li + 1] = dia[3 * i + 1];
  for (int32_t k = rp[i]; k < rp[i + 1]; k++) {
    const int64_t lj = 2 * (int64_t)ci[k] - s0;
    const C2<T> v = off[k];  // block [[re, -im], [im, re]]
    r0[lj] = v.x;
    r0[lj + 1] = -v.y;
    r1[lj] = v.y;
    r1[lj + 1] = v.x;
  }
}

// In-place Gauss-Jordan inversion of an SPD matrix (no pivoting needed) in
// shared memory, one CTA, m <= kDenseSmem, in the arithmetic type C (FP32 for
// the mixed path: FP64 arithmetic is slow on GB300 and the coarsest operator
// is well conditioned); writes the FP64 and FP32 copies.
constexpr int kDenseSmem = 128;
template <typename C>
__global__ void gauss_jordan_spd_smem(const int64_t *__restrict__ boff, const int32_t *__restrict__ bd, double *Ag,
                                      float *Afg, int *err) {
  // one CTA per diagonal block of the coarsest level
  const int m = bd[blockIdx.x];
  double *A = Ag + boff[blockIdx.x];
  float *Af = Afg + boff[blockIdx.x];
  extern __shared__ __align__(16) unsigned char gj_raw[];
  C *S = reinterpret_cast<C *>(gj_raw);
  __shared__ C ip_s;
  for (int q = threadIdx.x; q < m * m; q += blockDim.x) S[q] = (C)A[q];
  __syncthreads();
  for (int k = 0; k < m; k++) {
    if (threadIdx.x == 0) {
      const C piv = S[k * m + k];
      if (!(piv > (C)0)) atomicOr(err, 16);
      ip_s = (C)1 / piv;
    }
    __syncthreads();
    const C ip = ip_s;
    for (int j = threadIdx.x; j < m; j += blockDim.x) S[k * m + j] = (j == k) ? ip : S[k * m + j] * ip;
    __syncthreads();
    for (int q = threadIdx.x; q < m * m; q += blockDim.x) {
      const int i = q / m, j = q % m;
      if (i == k || j == k) continue;
      S[q] -= S[i * m + k] * S[k * m + j];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < m; i += blockDim.x)
      if (i != k) S[i * m + k] = -S[i * m + k] * ip;
    __syncthreads();
  }
  for (int q = threadIdx.x; q < m * m; q += blockDim.x) {
    A[q] = (double)S[q];
    Af[q] = (float)S[q];
  }
}

// The same in global memory for larger blocks.
__global__ void gauss_jordan_spd(const int64_t *__restrict__ boff, const int32_t *__restrict__ bd, double *Ag,
                                 float *Afg, int *err) {
  const int m = bd[blockIdx.x];
  double *A = Ag + boff[blockIdx.x];
  float *Af = Afg + boff[blockIdx.x];
  for (int k = 0; k < m; k++) {
    __syncthreads();
    const double piv = A[(int64_t)k * m + k];
    __syncthreads();
    if (threadIdx.x == 0 && !(piv > 0.0)) atomicOr(err, 16);
    const double ip = 1.0 / piv;
    for (int j = threadIdx.x; j < m; j += blockDim.x)
      A[(int64_t)k * m + j] = (j == k) ? ip : A[(int64_t)k * m + j] * ip;
    __syncthreads();
    for (int64_t q = threadIdx.x; q < (int64_t)m * m; q += blockDim.x) {
      const int i = (int)(q / m), j = (int)(q % m);
      if (i == k || j == k) continue;
      A[q] -= A[(int64_t)i * m + k] * A[(int64_t)k * m + j];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < m; i += blockDim.x)
      if (i != k) A[(int64_t)i * m + k] = -A[(int64_t)i * m + k] * ip;
  }
  __syncthreads();
  for (int64_t q = threadIdx.x; q < (int64_t)m * m; q += blockDim.x) Af[q] = (float)A[q];
}

// Packed block-diagonal dense inverse: real row i of the coarsest level is
// row rowoff[i] of the packed array, its block starts at real row bstart[i]
// and has bdim[i] columns.
struct DenseMap {
  const int64_t *rowoff;
  const int32_t *bstart, *bdim;
};
template <typename T>
__device__ __forceinline__ T dense_row(const DenseMap &D, const T *__restrict__ Ainv, int64_t i,
                                       const T *__restrict__ b) {
  const T *a = Ainv + D.rowoff[i];
  const T *bb = b + D.bstart[i];
  const int m = D.bdim[i];
  T s = 0;
  for (int j = 0; j < m; j++) s += a[j] * bb[j];
  return s;
}

template <typename T>
__global__ void dense_matvec(int m, const T *__restrict__ Ainv, DenseMap D, const T *__restrict__ b,
                             T *__restrict__ x) {
  dep_sync();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x)
    x[i] = dense_row(D, Ainv, i, b);
}

// ---- coarse-level tail: every level from `lt` down, in one launch (one CTA,
// or one thread-block cluster)
template <typename T>
struct LevelDesc {
  int64_t n;
  const int32_t *rp, *ci;
  const C2<T> *off;
  const T *dia, *dinv, *coef;
  C2<T> *b, *x, *x2, *d, *res;
  const int32_t *agg, *mem_ptr, *mem_idx;  // transfer to the next level
};


// The threads that run the tail: one CTA (barrier: __syncthreads), or the
// CTAs of one thread-block cluster (barrier: the hardware cluster barrier,
// whose arrive/wait pair has release/acquire semantics at cluster scope, so
// the vectors one CTA writes to global memory are visible to the others
// after it).  A cluster spreads the coarse levels' SpMVs over several SMs,
// whose L2 bandwidth one SM alone does not have.
struct CtaTeam {
  __device__ int rank() const { return threadIdx.x; }
  __device__ int size() const { return blockDim.x; }
  __device__ void sync() const { __syncthreads(); }
};
struct ClusterTeam {
  int r, n;  // CTA rank in the cluster, CTAs in the cluster
  __device__ static ClusterTeam here() {
    unsigned r, n;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(n));
    return ClusterTeam{(int)r, (int)n};
  }
  __device__ int rank() const { return r * (int)blockDim.x + (int)threadIdx.x; }
  __device__ int size() const { return n * (int)blockDim.x; }
  __device__ void sync() const {
    asm volatile("barrier.cluster.arrive.release.aligned;\n" ::: "memory");
    asm volatile("barrier.cluster.wait.acquire.aligned;\n" ::: "memory");
  }
};

// Threads per row for a tail level of n rows: the largest power of two
// <= 32 that still leaves a thread group per row, so the short serial chains
// of the coarse rows (and aggregates) are split across lanes.
template <class Team>
__device__ __forceinline__ int tail_tpr(const Team &tm, int64_t n) {
  int t = 1;
  while (t < 32 && (int64_t)(tm.size() / (2 * t)) >= n) t *= 2;
  return t;
}

// For every row i < n: the row's off-diagonal sum over x, reduced across its
// tpr lanes, then epi(i, sr, si) on the group's first lane.
template <typename T, class Team, class F>
__device__ __forceinline__ void tail_rows(const Team &tm, const LevelDesc<T> &A, const C2<T> *x, F &&epi) {
  const int tpr = tail_tpr(tm, A.n);
  const int groups = tm.size() / tpr, g = tm.rank() / tpr, li = tm.rank() % tpr;
  for (int64_t base = 0; base < A.n; base += groups) {
    const int64_t i = base + g;
    T sr = 0, si = 0;
    if (i < A.n)
      for (int32_t k = A.rp[i] + li; k < A.rp[i + 1]; k += tpr) {
        const C2<T> v = A.off[k], xv = x[A.ci[k]];
        sr += v.x * xv.x - v.y * xv.y;
        si += v.x * xv.y + v.y * xv.x;
      }
    for (int off = tpr >> 1; off > 0; off >>= 1) {
      sr += __shfl_xor_sync(0xffffffffu, sr, off);
      si += __shfl_xor_sync(0xffffffffu, si, off);
    }
    if (i < A.n && li == 0) epi(i, sr, si);
  }
}

template <typename T, class Team>
__device__ __forceinline__ void tail_body(const Team &tm, const LevelDesc<T> *lv, int lt, int L, int deg,
                                          const T *__restrict__ Ainv, const DenseMap &D) {
  const int tid = tm.rank(), bs = tm.size();
  for (int l = lt; l < L - 1; l++) {
    const LevelDesc<T> A = lv[l];
    C2<T> *cur = (deg % 2) ? A.x : A.x2, *oth = (deg % 2) ? A.x2 : A.x;
    for (int64_t i = tid; i < A.n; i += bs) cheb_first_elem<T>(i, A.dinv, A.coef[0], A.b[i], A.d, cur);
    tm.sync();
    for (int k = 1; k < deg; k++) {
      tail_rows<T>(tm, A, cur, [&](int64_t i, T sr, T si) {
        cheb_elem<T>(i, k, sr, si, A.dia, A.dinv, A.coef, A.b, cur, A.d, oth);
      });
      tm.sync();
      C2<T> *t = cur;
      cur = oth;
      oth = t;
    }
    tail_rows<T>(tm, A, A.x, [&](int64_t i, T sr, T si) {
      const C2<T> xi = A.x[i], bi = A.b[i];
      const T d0r = A.dia[3 * i], d0i = A.dia[3 * i + 1], d1b = A.dia[3 * i + 2];
      A.res[i] = C2<T>{bi.x - (sr + d0r * xi.x + d1b * xi.y), bi.y - (si + d1b * xi.x + d0i * xi.y)};
    });
    tm.sync();
    // restriction: aggregate sums, split across lanes like the rows
    const LevelDesc<T> Cl = lv[l + 1];
    {
      const int tpr = tail_tpr(tm, Cl.n);
      const int groups = bs / tpr, g = tid / tpr, li = tid % tpr;
      for (int64_t base = 0; base < Cl.n; base += groups) {
        const int64_t a = base + g;
        T sr = 0, si = 0;
        if (a < Cl.n)
          for (int32_t q = A.mem_ptr[a] + li; q < A.mem_ptr[a + 1]; q += tpr) {
            const C2<T> v = A.res[A.mem_idx[q]];
            sr += v.x;
            si += v.y;
          }
        for (int off = tpr >> 1; off > 0; off >>= 1) {
          sr += __shfl_xor_sync(0xffffffffu, sr, off);
          si += __shfl_xor_sync(0xffffffffu, si, off);
        }
        if (a < Cl.n && li == 0) Cl.b[a] = C2<T>{sr, si};
      }
    }
    tm.sync();
  }
  {
    const LevelDesc<T> C = lv[L - 1];
    const int m = (int)(2 * C.n);
    const T *b = reinterpret_cast<const T *>(C.b);
    T *x = reinterpret_cast<T *>(C.x);
    for (int i = tid; i < m; i += bs) x[i] = dense_row(D, Ainv, i, b);
    tm.sync();
  }
  for (int l = L - 2; l >= lt; l--) {
    const LevelDesc<T> A = lv[l];
    const C2<T> *xc = lv[l + 1].x;
    for (int64_t i = tid; i < A.n; i += bs) {
      const C2<T> c = xc[A.agg[i]];
      C2<T> v = A.x[i];
      v.x += c.x;
      v.y += c.y;
      A.x[i] = v;
    }
    tm.sync();
    C2<T> *cur = A.x, *oth = A.x2;
    for (int k = 0; k < deg; k++) {
      tail_rows<T>(tm, A, cur, [&](int64_t i, T sr, T si) {
        cheb_elem<T>(i, k, sr, si, A.dia, A.dinv, A.coef, A.b, cur, A.d, oth);
      });
      tm.sync();
      C2<T> *t = cur;
      cur = oth;
      oth = t;
    }
    if (cur != A.x) {
      for (int64_t i = tid; i < A.n; i += bs) A.x[i] = cur[i];
      tm.sync();
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(1024) tail_vcycle(const LevelDesc<T> *__restrict__ lv, int lt, int L,
                                                    int deg, const T *__restrict__ Ainv, DenseMap D,
                                                    const int *halt) {
  dep_sync();
  if (halt && *halt >= 2) return;
  tail_body(CtaTeam{}, lv, lt, L, deg, Ainv, D);
}

// The same over a thread-block cluster (launched with a cluster dimension
// equal to the grid): the halt flag is read by every CTA alike, so the
// cluster leaves or stays together.
template <typename T>
__global__ void __launch_bounds__(1024) tail_vcycle_cluster(const LevelDesc<T> *__restrict__ lv, int lt, int L,
                                                            int deg, const T *__restrict__ Ainv, DenseMap D,
                                                            const int *halt) {
  dep_sync();
  if (halt && *halt >= 2) return;
  tail_body(ClusterTeam::here(), lv, lt, L, deg, Ainv, D);
}

// plain MINRES pieces for the single-level case
template <typename T>
__global__ void lanczos_only(int64_t n, const MinresScalars *__restrict__ s, const C2<T> *__restrict__ u,
                             C2<T> *__restrict__ r_old, const C2<T> *__restrict__ r_cur) {
  dep_sync();
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const T *la = lanczos_coef<T>(s);
  const T a = la[0], bb = la[1], c = la[2];
  const C2<T> ui = u[i], ro = r_old[i], rc = r_cur[i];
  r_old[i] = C2<T>{a * ui.x - bb * ro.x - c * rc.x, a * ui.y - bb * ro.y - c * rc.y};
}

template <typename T>
__global__ void dot_advance(int64_t n, const C2<T> *__restrict__ a, const C2<T> *__restrict__ b,
                            double *partials, unsigned *counter, MinresScalars *s) {
  dep_sync();
  double v = 0.0;
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) v = (double)a[i].x * b[i].x + (double)a[i].y * b[i].y;
  double total = 0.0;
  if (grid_reduce(v, partials, counter, &s->rz, &total)) minres_advance(s, total);
}

template <typename T>
int staging_cap_of(const std::vector<int32_t> &rp, int64_t n) {
  int64_t mx = 0;
  for (int64_t r0 = 0; r0 < n; r0 += kRows) {
    const int64_t r1 = std::min<int64_t>(n, r0 + kRows);
    mx = std::max<int64_t>(mx, rp[r1] - (rp[r0] & ~(int64_t)3));
  }
  mx = (mx + 3) & ~(int64_t)3;
  return (int)std::min<int64_t>(mx, stage_limit<T>());
}

}  // namespace

// ------------------------------------------------------------ structures
struct AmgLevel {
  int64_t n = 0, nnz = 0;
  const int32_t *rp = nullptr, *ci = nullptr;  // level 0: the mesh graph
  DevBuf<int32_t> rp_own, ci_own;
  int cap32 = 0, cap64 = 0;
  bool warp32 = false, warp64 = false;  // SpMV schedule (tuned on the first refresh)
  bool tuned32 = false, tuned64 = false;
  // transfer to the next level
  DevBuf<int32_t> agg, mem_ptr, mem_idx, seg_ptr, seg_idx, intra_ptr, intra_idx;
};

template <typename T>
struct AmgVals {
  bool ready = false;
  int64_t refreshes = 0;  // numeric refreshes so far
  std::vector<DevBuf<C2<T>>> off;  // level >= 1
  std::vector<DevBuf<T>> dia;      // level >= 1
  std::vector<DevBuf<T>> dinv, coef;
  std::vector<DevBuf<C2<T>>> b, x, x2, d, res;
  DevBuf<LevelDesc<T>> desc;       // for the coarse-level tail
  // row sums of |K_ij| on the fine level for its Gershgorin bound, computed
  // once: |K_ij| = |alpha_ij| does not depend on mu (the phase factor has
  // modulus one), so only the diagonal blocks change between refreshes
  DevBuf<T> rowabs0;
  bool rowabs_ready = false;
};

struct Amg::Impl {
  NlsImpl &nls;
  AmgOptions opt;
  std::vector<AmgLevel> lev;
  int lt = 1;  // first level handled by the coarse-level tail
  AmgVals<float> vf;
  AmgVals<double> vd;
  DevBuf<unsigned long long> lmax_bits;  // one per level
  DevBuf<double> lmax;
  DevBuf<double> dense;  // coarsest (2n)^2 FP64
  DevBuf<float> densef;
  // packed block-diagonal coarsest inverse: per block (offset, dim), per real
  // row (offset, block start, dim)
  DevBuf<int64_t> blk_off, row_off;
  DevBuf<int32_t> blk_dim, row_start, row_dim;
  int nblk = 0, max_dim = 0;
  DenseMap dmap() const { return DenseMap{row_off.p, row_start.p, row_dim.p}; }
  DevBuf<int> err;
  Impl(NlsImpl &s, const AmgOptions &o) : nls(s), opt(o) {}
  template <typename T> AmgVals<T> &vals();
  template <typename T> void ensure_vals();
  template <typename T> const C2<T> *off(int l);
  template <typename T> const T *dia(int l);
  template <typename T> const T *dense_inv();
  template <typename T, class Op> void rows(int l, const C2<T> *x, const Op &op);
  template <typename T> void descend_ascend(int l, const C2<T> *b, C2<T> *x, MinresScalars *ms);
  // the MINRES state's `done` while a MINRES V-cycle is being issued: its
  // launches return at once once the solve has converged
  const int *halt = nullptr;
  template <typename T> void prime();
  // CTAs of the coarse-level tail, FP32 and FP64 (a thread-block cluster
  // when > 1).  The FP64 tail of a tetrahedral mesh runs on a cluster of 8:
  // the coarse SpMVs' FP64 arithmetic then spreads over 8 SMs (plain FP64
  // continuation at 64^3: 68.2 -> 71.2 steps/s).  The
  // FP32 tail stays on one CTA, whose vectors stay in its L1 between phases:
  // clusters of 8 and 16 took the learned line from 671 to 649 and 647
  // steps/s (in-place A/B).
  int tail_ctas[2] = {1, 1};
  // V-cycle launches overlap their predecessors (launch_dep) unless the
  // handle turned that off or times kernels with events between launches
  bool ovl() const { return nls.overlap_launches && !nls.timers[0].on && !nls.timers[1].on; }
};

template <> AmgVals<float> &Amg::Impl::vals<float>() { return vf; }
template <> AmgVals<double> &Amg::Impl::vals<double>() { return vd; }
template <> const C2<float> *Amg::Impl::off<float>(int l) {
  return l == 0 ? nls.d_keo32.p : vf.off[l].p;
}
template <> const C2<double> *Amg::Impl::off<double>(int l) {
  return l == 0 ? nls.d_keo64.p : vd.off[l].p;
}
template <> const float *Amg::Impl::dia<float>(int l) { return l == 0 ? nls.d_rd32.p : vf.dia[l].p; }
template <> const double *Amg::Impl::dia<double>(int l) { return l == 0 ? nls.d_rd64.p : vd.dia[l].p; }
template <> const float *Amg::Impl::dense_inv<float>() { return densef.p; }
template <> const double *Amg::Impl::dense_inv<double>() { return dense.p; }

Amg::Amg(NlsImpl &s, const AmgOptions &o) : impl(new Impl(s, o)) {
  Impl &I = *impl;
  cudaStream_t st = s.stream;
  MeshImpl &m = *s.mesh;
  // host copy of the current fine operator (strength tests)
  std::vector<HostLevel> H(1);
  H[0].n = m.N;
  H[0].rp.assign(m.rp.begin(), m.rp.end());
  H[0].ci = m.ci;
  {
    std::vector<C2<double>> off(2 * m.E);
    s.d_keo64.download(off.data(), 2 * m.E, st);
    H[0].dia.resize(3 * m.N);
    s.d_rd64.download(H[0].dia.data(), 3 * m.N, st);
    s.sync();
    H[0].off.resize(2 * m.E);
    for (int64_t k = 0; k < 2 * m.E; k++) H[0].off[k] = {off[k].x, off[k].y};
  }
  if (s.sys_off.empty())
    H[0].soff = {0, (int64_t)m.N};
  else
    H[0].soff = s.sys_off;
  // coarsen until every system's coarsest block is small (one system: the
  // whole level)
  while ((int)H.size() < o.max_levels && max_block(H.back()) > o.coarse_size) {
    HostLevel C;
    coarsen(H.back(), C, o.strength_threshold);
    if (C.n >= H.back().n) {  // no coarsening progress: stop here
      H.back().agg.clear();
      break;
    }
    H.push_back(std::move(C));
  }
  NOSH_CHECK(max_block(H.back()) <= 512, NOSH_ERR_INVALID,
             "AMG coarsening stalled at " + std::to_string(max_block(H.back())) + " nodes per system");
  const int L = (int)H.size();
  I.lev.resize(L);
  for (int l = 0; l < L; l++) {
    AmgLevel &A = I.lev[l];
    HostLevel &h = H[l];
    A.n = h.n;
    A.nnz = h.rp[h.n];
    if (l == 0) {
      A.rp = m.d_rp.p;
      A.ci = m.d_ci.p;
    } else {
      A.rp_own.upload(h.rp, st);
      A.ci_own.alloc(h.ci.size() + kPad);
      A.ci_own.zero(st);
      if (!h.ci.empty())
        NOSH_CUDA(cudaMemcpyAsync(A.ci_own.p, h.ci.data(), h.ci.size() * 4, cudaMemcpyHostToDevice, st));
      A.rp = A.rp_own.p;
      A.ci = A.ci_own.p;
    }
    A.cap32 = staging_cap_of<float>(h.rp, h.n);
    A.cap64 = staging_cap_of<double>(h.rp, h.n);
    if (l + 1 < L) {
      A.agg.upload(h.agg, st);
      A.mem_ptr.upload(h.mem_ptr, st);
      A.mem_idx.upload(h.mem_idx, st);
      A.seg_ptr.upload(h.seg_ptr, st);
      A.seg_idx.upload(h.seg_idx, st);
      A.intra_ptr.upload(h.intra_ptr, st);
      A.intra_idx.upload(h.intra_idx, st);
    }
  }
  // the fine level always runs on the whole grid; the first level at or
  // below kTailMax nodes and everything under it run in one CTA
  I.lt = L - 1;
  for (int l = 1; l < L; l++)
    if (I.lev[l].n <= kTailMax) {
      I.lt = l;
      break;
    }
  if (I.lt < 1) I.lt = L - 1;
  I.lmax_bits.alloc(L);
  I.lmax.alloc(L);
  {
    // the coarsest level's dense inverse: one packed block per system
    const HostLevel &Hc = H.back();
    const int64_t ns = (int64_t)Hc.soff.size() - 1;
    std::vector<int64_t> boff, roff;
    std::vector<int32_t> bdim, rstart, rdim;
    int64_t total = 0;
    for (int64_t sy = 0; sy < ns; sy++) {
      const int64_t n0 = Hc.soff[sy], nb = Hc.soff[sy + 1] - n0;
      if (nb == 0) continue;
      const int32_t m = (int32_t)(2 * nb);
      boff.push_back(total);
      bdim.push_back(m);
      for (int32_t r = 0; r < m; r++) {
        roff.push_back(total + (int64_t)r * m);
        rstart.push_back((int32_t)(2 * n0));
        rdim.push_back(m);
      }
      total += (int64_t)m * m;
      I.max_dim = std::max<int>(I.max_dim, m);
    }
    I.nblk = (int)boff.size();
    I.blk_off.upload(boff, st);
    I.blk_dim.upload(bdim, st);
    I.row_off.upload(roff, st);
    I.row_start.upload(rstart, st);
    I.row_dim.upload(rdim, st);
    I.dense.alloc(total);
    I.densef.alloc(total);
  }
  I.err.alloc(1);
  I.err.zero(st);
  NOSH_CUDA(cudaFuncSetAttribute(gauss_jordan_spd_smem<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 kDenseSmem * kDenseSmem * (int)sizeof(double)));
  NOSH_CUDA(cudaFuncSetAttribute(gauss_jordan_spd_smem<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 kDenseSmem * kDenseSmem * (int)sizeof(float)));
  s.sync();
}

Amg::~Amg() = default;

int Amg::num_levels() const { return (int)impl->lev.size(); }
int64_t Amg::level_size(int l) const { return impl->lev[l].n; }
int Amg::tail_level() const { return impl->lt; }

const int *Amg::error_flag_ptr() const { return impl->err.p; }

void Amg::clear_error() {
  // the coarse operators that failed the pivot check are replaced by the
  // next refresh, which is made a full Galerkin one
  NOSH_CUDA(cudaMemsetAsync(impl->err.p, 0, sizeof(int), impl->nls.stream));
  impl->vf.refreshes = 0;
  impl->vd.refreshes = 0;
}

int Amg::error_flag() {
  int herr = 0;
  impl->err.download(&herr, 1, impl->nls.stream);
  impl->nls.sync();
  return herr;
}

template <typename T>
void Amg::Impl::ensure_vals() {
  AmgVals<T> &V = vals<T>();
  if (V.ready) return;
  const int L = (int)lev.size();
  V.off.resize(L);
  V.dia.resize(L);
  V.dinv.resize(L);
  V.coef.resize(L);
  V.b.resize(L);
  V.x.resize(L);
  V.x2.resize(L);
  V.d.resize(L);
  V.res.resize(L);
  for (int l = 0; l < L; l++) {
    const int64_t n = lev[l].n;
    if (l > 0) {
      V.off[l].alloc(lev[l].nnz + kPad);
      V.off[l].zero(nls.stream);
      V.dia[l].alloc(3 * n);
    }
    V.dinv[l].alloc(3 * n);
    V.coef[l].alloc(2 * std::max(opt.smooth_degree, 1) + 2);
    V.b[l].alloc(n);
    V.x[l].alloc(n);
    V.x2[l].alloc(n);
    V.d[l].alloc(n);
    V.res[l].alloc(n);
  }
  std::vector<LevelDesc<T>> desc(L);
  for (int l = 0; l < L; l++) {
    LevelDesc<T> &D = desc[l];
    D.n = lev[l].n;
    D.rp = lev[l].rp;
    D.ci = lev[l].ci;
    D.off = off<T>(l);
    D.dia = dia<T>(l);
    D.dinv = V.dinv[l].p;
    D.coef = V.coef[l].p;
    D.b = V.b[l].p;
    D.x = V.x[l].p;
    D.x2 = V.x2[l].p;
    D.d = V.d[l].p;
    D.res = V.res[l].p;
    D.agg = lev[l].agg.p;
    D.mem_ptr = lev[l].mem_ptr.p;
    D.mem_idx = lev[l].mem_idx.p;
  }
  V.desc.upload(desc, nls.stream);
  nls.sync();
  prime<T>();
  V.ready = true;
}

// Numeric refresh from the current regularised KEO; stream-ordered, no host
// synchronisation (the pivot check is read later through error_flag()).
template <typename T>
void Amg::refresh() {
  Impl &I = *impl;
  I.ensure_vals<T>();
  AmgVals<T> &V = I.vals<T>();
  cudaStream_t st = I.nls.stream;
  const int L = (int)I.lev.size();
  const bool partial = I.opt.reuse_period > 1 && L > 1 && V.refreshes % I.opt.reuse_period != 0;
  ++V.refreshes;
  if (!V.rowabs_ready) {
    V.rowabs0.alloc(I.lev[0].n);
    row_abs_sums<T><<<div_up(I.lev[0].n, 256), 256, 0, st>>>(I.lev[0].n, I.lev[0].rp, I.off<T>(0), V.rowabs0.p);
    ++I.nls.launch_count;
    V.rowabs_ready = true;
  }
  if (partial) {
    // hierarchy reuse (MueLu "reuse: type full", src/keo_regularized.cpp:
    // 298-330): the fine level reads the current operator directly; only its
    // block-Jacobi inverse and Chebyshev bounds follow it, the coarse
    // operators keep their last Galerkin values (SPD, so the V-cycle stays
    // an SPD preconditioner)
    NOSH_CUDA(cudaMemsetAsync(I.lmax_bits.p, 0, sizeof(unsigned long long), st));
    dinv_gershgorin<T><<<div_up(I.lev[0].n, 256), 256, 0, st>>>(I.lev[0].n, I.lev[0].rp, I.off<T>(0), I.dia<T>(0),
                                                                V.dinv[0].p, I.lmax_bits.p, I.err.p,
                                                                V.rowabs0.p);
    cheb_coeffs<T><<<1, 1, 0, st>>>(I.lmax_bits.p, std::max(I.opt.smooth_degree, 1), I.opt.cheb_ratio, V.coef[0].p,
                                    I.lmax.p);
    I.nls.launch_count += 2;
    NOSH_CUDA(cudaGetLastError());
    return;
  }
  NOSH_CUDA(cudaMemsetAsync(I.lmax_bits.p, 0, L * sizeof(unsigned long long), st));
  for (int l = 0; l < L; l++) {
    AmgLevel &A = I.lev[l];
    if (l > 0) {
      AmgLevel &F = I.lev[l - 1];
      rap_offdiag<T><<<div_up(std::max<int64_t>(A.nnz, 1), 256), 256, 0, st>>>(
          A.nnz, F.seg_ptr.p, F.seg_idx.p, I.off<T>(l - 1), V.off[l].p);
      ++I.nls.launch_count;
      rap_diag<T><<<div_up(A.n, 256), 256, 0, st>>>(A.n, F.mem_ptr.p, F.mem_idx.p, F.intra_ptr.p,
                                                     F.intra_idx.p, I.dia<T>(l - 1), I.off<T>(l - 1),
                                                     V.dia[l].p);
      ++I.nls.launch_count;
    }
    if (l < L - 1) {  // the coarsest level is solved directly
      dinv_gershgorin<T><<<div_up(A.n, 256), 256, 0, st>>>(A.n, A.rp, I.off<T>(l), I.dia<T>(l),
                                                            V.dinv[l].p, I.lmax_bits.p + l, I.err.p,
                                                            l == 0 ? (const T *)V.rowabs0.p : nullptr);
      ++I.nls.launch_count;
      cheb_coeffs<T><<<1, 1, 0, st>>>(I.lmax_bits.p + l, std::max(I.opt.smooth_degree, 1), I.opt.cheb_ratio,
                                      V.coef[l].p, I.lmax.p + l);
      ++I.nls.launch_count;
    }
  }
  // SpMV schedule per coarse level, once (needs the level's values)
  for (int l = 1; l < L; l++) {
    AmgLevel &A = I.lev[l];
    bool &tuned = sizeof(T) == 4 ? A.tuned32 : A.tuned64;
    if (tuned) continue;
    bool &warp = sizeof(T) == 4 ? A.warp32 : A.warp64;
    if (I.nls.spmv_schedule == 0)
      warp = pick_warp_schedule<T>((int)A.n, A.rp, A.ci, I.off<T>(l), sizeof(T) == 4 ? A.cap32 : A.cap64,
                                   I.nls.red.partials.p, I.nls.red.counter.p, st);
    else
      warp = I.nls.spmv_schedule == 2;
    tuned = true;
  }
  const AmgLevel &C = I.lev.back();
  coarse_dense<T><<<div_up(C.n, 128), 128, 0, st>>>(C.n, C.rp, C.ci, I.off<T>(L - 1), I.dia<T>(L - 1),
                                                     I.row_start.p, I.row_off.p, I.row_dim.p, I.dense.p);
  ++I.nls.launch_count;
  if (I.max_dim <= kDenseSmem)
    gauss_jordan_spd_smem<T><<<I.nblk, 1024, (size_t)I.max_dim * I.max_dim * sizeof(T), st>>>(
        I.blk_off.p, I.blk_dim.p, I.dense.p, I.densef.p, I.err.p);
  else
    gauss_jordan_spd<<<I.nblk, 1024, 0, st>>>(I.blk_off.p, I.blk_dim.p, I.dense.p, I.densef.p, I.err.p);
  ++I.nls.launch_count;
  NOSH_CUDA(cudaGetLastError());
}

template <typename T>
void Amg::Impl::prime() {
  // shared-memory opt-in of every row kernel instantiation, set before any
  // stream capture
  NOSH_CUDA(cudaFuncSetAttribute(row_block_apply<T, ChebOp<T>>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024));
  NOSH_CUDA(cudaFuncSetAttribute(row_block_apply<T, ChebMinresOp<T>>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024));
  NOSH_CUDA(cudaFuncSetAttribute(row_block_apply<T, ResidOp<T>>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024));
  tail_ctas[sizeof(T) == 8] = 1;
  const int L = (int)lev.size();
  if (sizeof(T) == 8 && L >= 2 && lt < L) {
    constexpr int c = 8;  // portable cluster size
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(c);
    cfg.blockDim = dim3(1024);
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = c;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int nc = 0;
    const bool ok = cudaOccupancyMaxActiveClusters(&nc, tail_vcycle_cluster<T>, &cfg) == cudaSuccess && nc > 0;
    cudaGetLastError();  // a device without clusters of 8 keeps the one-CTA tail
    // tetrahedral hierarchies only: their coarse rows hold about twice the
    // nonzeros of triangular ones, and the FP64 tail of a 2-D 65 x 65 mesh
    // lost more to the cluster barriers than it gained (FP64 Newton solve
    // 111.8 -> 104.4 solves/s), while the 64^3 one gained
    if (ok && nls.mesh->nvc == 4) tail_ctas[1] = c;
  }
}

template <typename T, class Op>
void Amg::Impl::rows(int l, const C2<T> *x, const Op &op) {
  const AmgLevel &A = lev[l];
  const int cap = sizeof(T) == 4 ? A.cap32 : A.cap64;
  const bool warp = l == 0 ? (sizeof(T) == 4 ? nls.warp32 : nls.warp64) : (sizeof(T) == 4 ? A.warp32 : A.warp64);
  launch_spmv<T, Op>(warp, (int)A.n, A.rp, A.ci, off<T>(l), x, cap, op, nls.red.partials.p, nls.red.counter.p,
                     Op::kReduce ? &nls.red.out.p[32] : nullptr, nls.stream, ovl());
  ++nls.launch_count;
}

// Level l of the V-cycle after its first Chebyshev step: finish the
// pre-smoothing (its result ends in x), coarse correction, post-smoothing.
// With ms != nullptr the fine level's last step also advances MINRES.
template <typename T>
void Amg::Impl::descend_ascend(int l, const C2<T> *b, C2<T> *x, MinresScalars *ms) {
  AmgVals<T> &V = vals<T>();
  AmgLevel &A = lev[l];
  cudaStream_t st = nls.stream;
  const int L = (int)lev.size();
  const int deg = std::max(opt.smooth_degree, 1);
  const int B = 256;
  const T *dv = dia<T>(l);
  C2<T> *cur = (deg % 2 == 1) ? x : V.x2[l].p;
  C2<T> *oth = (deg % 2 == 1) ? V.x2[l].p : x;
  KernelTimer *tm = l == 0 ? &nls.timers[NOSH_KERNEL_SMOOTHER] : nullptr;
  // values per vertex: a Chebyshev step reads x, b, the diagonal block and
  // its inverse and the previous direction d, and writes d and x (16; the
  // first step of a sweep reads no d: 14); the residual reads x, b and the
  // diagonal block and writes the residual (9)
  const int vb = (int)sizeof(T);
  const double cheb_bytes = nls.spmv_bytes(2 * vb, 16 * vb);
  const double cheb0_bytes = nls.spmv_bytes(2 * vb, 14 * vb);
  const double res_bytes = nls.spmv_bytes(2 * vb, 9 * vb);
  // timed as one event pair around the consecutive fine-level launches of
  // the pre-smoothing and the residual (and of the post-smoothing below)
  if (tm) tm->begin(st);
  for (int k = 1; k < deg; k++) {
    ChebOp<T> op{dv, V.dinv[l].p, V.coef[l].p, k, b, cur, V.d[l].p, oth, halt};
    rows<T>(l, cur, op);
    std::swap(cur, oth);
  }
  ResidOp<T> rop{dv, b, x, V.res[l].p, halt};
  rows<T>(l, x, rop);
  if (tm) tm->end(st, (deg - 1) * cheb_bytes + res_bytes, deg);
  const AmgLevel &Cl = lev[l + 1];
  if (l + 1 < lt) {
    // restriction + first step of level l+1, whose pre-smoothing must end in
    // its x buffer
    C2<T> *first = (deg % 2 == 1) ? V.x[l + 1].p : V.x2[l + 1].p;
    launch_dep(ovl(), restrict_first<T>, dim3(div_up(Cl.n * kAggLanes, B)), dim3(B), 0, st, Cl.n, A.mem_ptr.p,
               A.mem_idx.p, V.res[l].p, V.b[l + 1].p, V.dinv[l + 1].p, V.coef[l + 1].p, V.d[l + 1].p, first,
               halt);
    ++nls.launch_count;
    descend_ascend<T>(l + 1, V.b[l + 1].p, V.x[l + 1].p, nullptr);
  } else {
    launch_dep(ovl(), restrict_kernel<T>, dim3(div_up(Cl.n * kAggLanes, B)), dim3(B), 0, st, Cl.n, A.mem_ptr.p,
               A.mem_idx.p, V.res[l].p, V.b[l + 1].p, halt);
    ++nls.launch_count;
    const int tc = tail_ctas[sizeof(T) == 8];
    if (tc > 1)
      launch_cluster_dep(ovl(), tc, tail_vcycle_cluster<T>, dim3(1024), 0, st, V.desc.p, lt, L, deg,
                         dense_inv<T>(), dmap(), halt);
    else
      launch_dep(ovl(), tail_vcycle<T>, dim3(1), dim3(1024), 0, st, V.desc.p, lt, L, deg, dense_inv<T>(), dmap(),
               halt);
    ++nls.launch_count;
  }
  launch_dep(ovl(), prolong_kernel<T>, dim3(div_up(A.n, B)), dim3(B), 0, st, A.n, A.agg.p, V.x[l + 1].p, x,
             halt);
  ++nls.launch_count;
  cur = x;
  oth = V.x2[l].p;
  if (tm) tm->begin(st);
  for (int k = 0; k < deg; k++) {
    if (ms && k == deg - 1) {
      ChebMinresOp<T> op{dv, V.dinv[l].p, V.coef[l].p, k, b, cur, V.d[l].p, oth, ms, halt};
      rows<T>(l, cur, op);
    } else {
      ChebOp<T> op{dv, V.dinv[l].p, V.coef[l].p, k, b, cur, V.d[l].p, oth, halt};
      rows<T>(l, cur, op);
    }
    std::swap(cur, oth);
  }
  if (tm) tm->end(st, cheb0_bytes + (deg - 1) * cheb_bytes, deg);
  if (cur != x) {
    NOSH_CUDA(cudaMemcpyAsync(x, cur, A.n * sizeof(C2<T>), cudaMemcpyDeviceToDevice, st));
  }
}

// z = V-cycle(r)
template <typename T>
void Amg::apply(const T *r, T *z) {
  Impl &I = *impl;
  AmgVals<T> &V = I.vals<T>();
  cudaStream_t st = I.nls.stream;
  const int L = (int)I.lev.size();
  const AmgLevel &A = I.lev[0];
  if (L == 1) {
    const int m2 = (int)(2 * A.n);
    launch_dep(I.ovl(), dense_matvec<T>, dim3(div_up(m2, 128)), dim3(128), 0, st, m2, I.dense_inv<T>(), I.dmap(),
               r, z);
    ++I.nls.launch_count;
    NOSH_CUDA(cudaGetLastError());
    return;
  }
  const int deg = std::max(I.opt.smooth_degree, 1);
  C2<T> *first = (deg % 2 == 1) ? (C2<T> *)z : V.x2[0].p;
  launch_dep(I.ovl(), cheb_first<T>, dim3(div_up(A.n, 256)), dim3(256), 0, st, A.n, V.dinv[0].p, V.coef[0].p,
             (const C2<T> *)r, V.d[0].p, first);
  ++I.nls.launch_count;
  I.descend_ascend<T>(0, (const C2<T> *)r, (C2<T> *)z, nullptr);
  NOSH_CUDA(cudaGetLastError());
}

// The fine level's pre-smoothing sweep alone, from x = 0: the first
// Chebyshev step, then degree - 1 SpMV steps (as in descend_ascend).
template <typename T>
void Amg::presmooth(const T *b, T *x) {
  Impl &I = *impl;
  NOSH_CHECK(I.lev.size() >= 2, NOSH_ERR_INVALID, "the hierarchy has one level: no smoother");
  AmgVals<T> &V = I.vals<T>();
  cudaStream_t st = I.nls.stream;
  const AmgLevel &A = I.lev[0];
  const int deg = std::max(I.opt.smooth_degree, 1);
  C2<T> *cur = (deg % 2 == 1) ? (C2<T> *)x : V.x2[0].p;
  C2<T> *oth = (deg % 2 == 1) ? V.x2[0].p : (C2<T> *)x;
  launch_dep(I.ovl(), cheb_first<T>, dim3(div_up(A.n, 256)), dim3(256), 0, st, A.n, V.dinv[0].p, V.coef[0].p,
             (const C2<T> *)b, V.d[0].p, cur);
  ++I.nls.launch_count;
  for (int k = 1; k < deg; k++) {
    ChebOp<T> op{I.dia<T>(0), V.dinv[0].p, V.coef[0].p, k, (const C2<T> *)b, cur, V.d[0].p, oth, nullptr};
    I.rows<T>(0, cur, op);
    std::swap(cur, oth);
  }
  NOSH_CUDA(cudaGetLastError());
}

// One MINRES Lanczos step around the V-cycle:
//   r_old <- J z / beta - (beta/oldb) r_old - (alfa/beta) r_cur  (= r_new)
//   z_out <- V-cycle(r_new),  <r_new, z_out> and the Givens recurrence.
template <typename T>
void Amg::apply_minres(MinresScalars *ms, const T *u, T *r_old, const T *r_cur, T *z_out) {
  Impl &I = *impl;
  AmgVals<T> &V = I.vals<T>();
  cudaStream_t st = I.nls.stream;
  const int L = (int)I.lev.size();
  const AmgLevel &A = I.lev[0];
  if (L == 1) {
    launch_dep(I.ovl(), lanczos_only<T>, dim3(div_up(A.n, 256)), dim3(256), 0, st, A.n, ms, (const C2<T> *)u,
               (C2<T> *)r_old, (const C2<T> *)r_cur);
    apply<T>(r_old, z_out);
    launch_dep(I.ovl(), dot_advance<T>, dim3(div_up(A.n, 256)), dim3(256), 0, st, A.n, (const C2<T> *)r_old,
               (const C2<T> *)z_out, I.nls.red.partials.p, I.nls.red.counter.p, ms);
    I.nls.launch_count += 2;
    NOSH_CUDA(cudaGetLastError());
    return;
  }
  const int deg = std::max(I.opt.smooth_degree, 1);
  // the fine level's right-hand side is r_new itself: point b[0] at r_old
  C2<T> *first = (deg % 2 == 1) ? (C2<T> *)z_out : V.x2[0].p;
  launch_dep(I.ovl(), lanczos_first<T>, dim3(div_up(A.n, 256)), dim3(256), 0, st, A.n, ms, (const C2<T> *)u,
             (C2<T> *)r_old, (const C2<T> *)r_cur, V.dinv[0].p, V.coef[0].p, V.d[0].p, first);
  ++I.nls.launch_count;
  I.halt = &ms->done;
  I.descend_ascend<T>(0, (const C2<T> *)r_old, (C2<T> *)z_out, ms);
  I.halt = nullptr;
  NOSH_CUDA(cudaGetLastError());
}

template void Amg::refresh<float>();
template void Amg::refresh<double>();
template void Amg::apply<float>(const float *, float *);
template void Amg::apply<double>(const double *, double *);
template void Amg::presmooth<float>(const float *, float *);
template void Amg::presmooth<double>(const double *, double *);
template void Amg::apply_minres<float>(MinresScalars *, const float *, float *, const float *, float *);
template void Amg::apply_minres<double>(MinresScalars *, const double *, double *, const double *, double *);

}  // namespace nosh
