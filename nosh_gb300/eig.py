"""Lowest eigenpairs of the Jacobian: the stability of a state.

The reference's eigen tool (``executables/nosh-eig/nosh-eig.cpp``) hands the
Jacobian operator to an Anasazi solver (LOBPCG, block Davidson or
Krylov-Schur); its continuation configuration asks for the eigenvalues of
the Jacobian nearest zero (``examples/conf.xml:50-66``, "Jacobian Inverse"
operator, "LM" order).  J is real symmetric, and a converged state is stable
when no eigenvalue of J is negative apart from the U(1) gauge mode i*psi,
which J maps to i*F = 0.

Here the solver is LOBPCG (Knyazev 2001) for the smallest algebraic
eigenvalues, run on the GPU:
* J applies are the library's FP64 Jacobian kernels (``nosh_jacobian_apply``);
* the preconditioner is one AMG V-cycle of the regularised KEO
  (``nosh_keo_regularized_apply``), the SPD operator that preconditions the
  Newton solves;
* the search space is kept orthogonal to the gauge mode, so the returned
  eigenvalues are the physical ones;
* each iteration orthonormalises the basis [X, W, P] by SVQB (two passes,
  directions with negligible Gram eigenvalues dropped) and takes the Ritz
  pairs of the projected matrix (the Hetmaniuk-Lehoucq form, which stays
  stable when the basis degenerates);
* the block carries guard vectors beyond the k wanted pairs (k by default),
  so a cluster that straddles the k-th eigenvalue does not slow the
  iteration; only the k wanted pairs are tested for convergence;
* the W and P blocks are scaled to unit rows before the orthonormalisation,
  since they shrink with the residual.

All of it runs inside the library (``nosh_eig_lowest``): the block Gram
matrices, the SVQB orthonormalisation and the block combinations are the
library's own CUDA kernels on the handle's stream, and only the small
projected eigenproblems are solved on the host.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _check, _f64, _lib, _ptr


def lowest_eigenpairs(model, psi, params, k=4, tol=1e-8, maxit=500, seed=0, deflate_gauge=True, guard=None):
    """The k smallest eigenvalues of J(psi, params) and their unit
    eigenvectors (rows of a (k, 2N) tensor).  ``psi``: host array or device
    tensor (2N reals).  Convergence: ||J x - lambda x|| <= tol * ||J||_est
    for every pair.  Returns (eigenvalues (k,) numpy, eigenvectors (k, 2N)
    torch FP64 on the device, iterations)."""
    import torch

    n = 2 * model.n
    guard = max(2, k) if guard is None else guard
    mb = k + guard
    if not (1 <= k and 3 * mb <= 64 and 3 * mb + 1 < n):
        raise ValueError("need 1 <= k, 3 (k + guard) <= 64 and 3 (k + guard) + 1 < 2N")
    dev = torch.device("cuda", torch.cuda.current_device())
    X = torch.empty((k, n), dtype=torch.float64, device=dev)
    lam = np.empty(k)
    its = C.c_int()
    torch.cuda.synchronize()
    _check(_lib.nosh_eig_lowest(model._h, _ptr(_f64(psi)), _ptr(model._pvec(params)), k, tol, maxit, guard,
                                1 if deflate_gauge else 0, C.c_uint64(seed + 1), _ptr(lam), _ptr(X), C.byref(its)))
    return lam, X, its.value
