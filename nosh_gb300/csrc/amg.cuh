// Aggregation AMG for the regularised KEO (the keo_regularized
// preconditioner).  Declared here, defined in amg.cu.
#pragma once

#include "minres_state.cuh"
#include "nls.cuh"

namespace nosh {

struct AmgLevel;

struct AmgOptions {
  int max_levels = 10;
  int coarse_size = 64;  // stop coarsening at or below this many nodes
  int smooth_degree = 2; // Chebyshev degree of pre- and post-smoothing
  // refreshes between full Galerkin refreshes; the ones in between update
  // the fine level only (hierarchy reuse)
  int reuse_period = 8;
  double strength_threshold = 0.0;   // |a_ij| >= theta sqrt(d_i d_j) is strong
  double cheb_ratio = 15.0;          // smoothing interval [lmax / ratio, 1.1 lmax]
};

struct Amg {
  explicit Amg(NlsImpl &nls, const AmgOptions &opt = AmgOptions());
  ~Amg();
  // numeric refresh from the current regularised KEO (nls.d_rd*, d_keo*)
  template <typename T>
  void refresh();
  // z = V-cycle(r); r, z device vectors of 2N (interleaved complex)
  template <typename T>
  void apply(const T *r, T *z);
  // x = the fine level's Chebyshev smoothing sweep from x = 0 on right-hand
  // side b (the V-cycle's pre-smoother alone); needs two levels or more
  template <typename T>
  void presmooth(const T *b, T *x);
  // One MINRES Lanczos step fused around the V-cycle (see amg.cu)
  template <typename T>
  void apply_minres(MinresScalars *ms, const T *u, T *r_old, const T *r_cur, T *z_out);
  int num_levels() const;
  int64_t level_size(int l) const;
  int tail_level() const;
  // pivot-failure flags of the coarsest factorisation (synchronises)
  int error_flag();
  const int *error_flag_ptr() const;  // device address of the same flags
  // clears the flags and makes the next refresh a full one (after a failed
  // pivot check, so the handle can go on with other parameters)
  void clear_error();

  struct Impl;
  std::unique_ptr<Impl> impl;
};

}  // namespace nosh
