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
* each iteration orthonormalises the basis [X, W, P] by a QR factorisation
  and takes the Ritz pairs of the projected matrix (the Hetmaniuk-Lehoucq
  form, which stays stable when the basis degenerates);
* the block carries guard vectors beyond the k wanted pairs (k by default),
  so a cluster that straddles the k-th eigenvalue does not slow the
  iteration; only the k wanted pairs are tested for convergence;
* the W and P blocks are scaled to unit rows before the QR, since they
  shrink with the residual.

Block vector algebra runs as torch FP64 operations on the library's stream.
"""
from __future__ import annotations

import numpy as np

from . import PREC_FP64, NoshError


def _gauge(psi):
    g = psi.clone()
    g[0::2], g[1::2] = -psi[1::2], psi[0::2]
    return g


def lowest_eigenpairs(model, psi, params, k=4, tol=1e-8, maxit=500, seed=0, deflate_gauge=True, guard=None):
    """The k smallest eigenvalues of J(psi, params) and their unit
    eigenvectors (rows of a (k, 2N) tensor).  ``psi``: host array or device
    tensor (2N reals).  Convergence: ||J x - lambda x|| <= tol * ||J||_est
    for every pair.  Returns (eigenvalues (k,) numpy, eigenvectors (k, 2N)
    torch FP64 on the device, iterations)."""
    import torch

    n = 2 * model.n
    guard = max(2, k) if guard is None else guard
    mb = k + guard  # block size
    if not (1 <= k and 3 * mb + 1 < n):
        raise ValueError("need 1 <= k and 3 (k + guard) + 1 < 2N")
    dev = torch.device("cuda", torch.cuda.current_device())
    prec0 = model.precision
    model.set_precision(PREC_FP64)
    stream = torch.cuda.ExternalStream(model.stream(), device=dev)
    try:
        with torch.cuda.stream(stream):
            psi_t = torch.as_tensor(np.asarray(psi, np.float64) if not hasattr(psi, "data_ptr") else psi,
                                    dtype=torch.float64, device=dev).contiguous()
            J = model.create_W_op()
            J.rebuild(params, psi_t)
            T = model.create_W_prec()
            T.rebuild(params, psi_t)
            U = None
            if deflate_gauge:
                u = _gauge(psi_t)
                nu = torch.linalg.norm(u)
                if nu > 0:
                    U = (u / nu).reshape(1, n)

            def proj(V):
                return V if U is None else V - (V @ U.T) @ U

            def apply(op, V):
                V = V.contiguous()
                out = torch.empty_like(V)
                op.apply(V, out)
                return out

            def ritz(S, AS):
                # the small projected eigenproblem on the host
                H = (S @ AS.T).cpu().numpy()
                w, C = np.linalg.eigh((H + H.T) / 2)
                return torch.from_numpy(w).to(dev), torch.from_numpy(C).to(dev)

            g = torch.Generator(device="cpu").manual_seed(seed)
            X = torch.randn(mb, n, generator=g, dtype=torch.float64).to(dev)
            X = proj(X)
            Q, _ = torch.linalg.qr(X.T)
            X = Q.T.contiguous()
            AX = apply(J, X)
            lam, C = ritz(X, AX)
            X, AX = C.T @ X, C.T @ AX
            P = None
            # ||J|| estimate for the relative test: the largest Ritz value
            # magnitude seen, at least the first residual scale
            jnorm = float(torch.linalg.norm(AX, dim=1).max())
            it = 0
            for it in range(1, maxit + 1):
                R = AX - lam[:, None] * X
                rn = torch.linalg.norm(R, dim=1)
                jnorm = max(jnorm, float(lam.abs().max()))
                if bool((rn[:k] <= tol * jnorm).all()):
                    break
                W = proj(apply(T, R))
                # unit rows before the QR: W and P shrink with the residual,
                # and orthogonalising tiny rows against X in one QR would
                # keep only their leading digits
                def unit(V):
                    return V / torch.linalg.norm(V, dim=1, keepdim=True).clamp_min(1e-300)

                blocks = [X, unit(W)] if P is None else [X, unit(W), unit(P)]
                S = torch.cat(blocks, 0)
                Q, Rq = torch.linalg.qr(S.T)
                # drop directions the QR found (numerically) dependent
                keep = Rq.diagonal().abs() > 1e-12 * Rq.diagonal().abs().max()
                Q = Q[:, keep]
                S = proj(Q.T.contiguous())
                AS = apply(J, S)
                theta, Cs = ritz(S, AS)
                Ck = Cs[:, :mb]
                Xn, AXn = Ck.T @ S, Ck.T @ AS
                # new search direction: the part of the update outside span(X)
                Pn = Xn - (Xn @ X.T) @ X
                X, AX, lam = Xn, AXn, theta[:mb]
                P = Pn
            torch.cuda.current_stream().synchronize()
            if not torch.isfinite(lam).all():
                raise NoshError(4, "eigenvalue iteration produced NaN")
            return lam[:k].cpu().numpy(), X[:k].contiguous(), it
    finally:
        model.set_precision(prec0)
