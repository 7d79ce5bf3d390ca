"""CPU FP64 oracle for nosh's NLS hot path -- TEST INFRASTRUCTURE ONLY.

Thin numpy/ctypes wrapper around ``oracle/_build/libnosh_oracle.so`` (built
from ``nosh_oracle.c`` by ``oracle/Makefile``).  Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline / reference arm
import this module; the product package never does.

The C code restates the reference (file:line cited there).  It is pinned
against the known-answer constants of the reference's own test cases
(``test/keo.cpp``, ``test/jac.cpp``, ``test/compute_f.cpp``,
``test/mesh.cpp``, ``test/io.cpp``) on the reconstructed "rectanglesmall" and
"cubesmall" meshes: ``tests/test_oracle_kat.py``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libnosh_oracle.so")

_lib = None

i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, portable flags)."""
    srcs = [os.path.join(HERE, f) for f in ("nosh_oracle.c", "nosh_solver.c", "nosh_oracle.h")]
    if force or not os.path.exists(LIB_PATH) or any(
        os.path.getmtime(s) > os.path.getmtime(LIB_PATH) for s in srcs
    ):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        I64, F64, U64, I = C.c_int64, C.c_double, C.c_uint64, C.c_int
        sig = {
            "nor_gen_square": (None, [I, U64, F64, f64p, i32p, f64p]),
            "nor_gen_cube": (None, [I, U64, F64, f64p, i32p, f64p]),
            "nor_build_edges": (I64, [I, I64, I64, i32p, i32p, i32p]),
            "nor_complex_graph": (None, [I64, I64, i32p, i32p, i32p]),
            "nor_edge_data": (None, [I, I64, f64p, I64, i32p, I64, i32p, f64p, f64p]),
            "nor_control_volumes": (None, [I, I64, f64p, I64, i32p, f64p]),
            "nor_edge_projection": (None, [I64, i32p, f64p, f64p, f64p]),
            "nor_alpha": (None, [I64, i32p, f64p, f64p, f64p, f64p]),
            "nor_keo_values": (None, [I64, I64, i32p, f64p, f64p, F64, i32p, i32p, f64p]),
            "nor_dkeo_values": (None, [I64, I64, i32p, f64p, f64p, f64p, F64, i32p, i32p, f64p]),
            "nor_keo_apply": (None, [I64, I64, i32p, f64p, f64p, F64, f64p, f64p]),
            "nor_dkeo_apply": (None, [I64, I64, i32p, f64p, f64p, f64p, F64, f64p, f64p]),
            "nor_compute_f": (None, [I64, I64, i32p, f64p, f64p, F64, F64, f64p, f64p, f64p, f64p, f64p]),
            "nor_dfdp": (None, [I64, I64, i32p, f64p, f64p, f64p, F64, I, f64p, f64p, f64p, f64p, f64p]),
            "nor_jac_diags": (None, [I64, f64p, f64p, f64p, F64, f64p, f64p, f64p]),
            "nor_jac_apply": (None, [I64, I64, i32p, f64p, f64p, F64, f64p, f64p, f64p, f64p]),
            "nor_kreg_apply": (None, [I64, I64, i32p, f64p, f64p, F64, F64, f64p, f64p, f64p, f64p, f64p]),
            "nor_energy": (F64, [I64, f64p, f64p]),
            "nor_inner_product": (F64, [I64, f64p, f64p, f64p]),
            "nor_solver_create": (C.c_void_p, [I64, I64, i32p, f64p, f64p, f64p, f64p, f64p, F64]),
            "nor_solver_destroy": (None, [C.c_void_p]),
            "nor_num_threads": (I, []),
            "nor_set_num_threads": (I, [I]),
            "nor_newton": (I, [C.c_void_p, f64p, F64, F64, I, C.POINTER(I), C.POINTER(I),
                               C.POINTER(F64), C.POINTER(F64)]),
            "nor_continuation_step": (I, [C.c_void_p, f64p, C.c_void_p, F64, F64, F64, F64, C.POINTER(I),
                                          C.POINTER(I), C.POINTER(F64), C.POINTER(F64)]),
            "nor_amg_levels": (I, [C.c_void_p, np.ctypeslib.ndpointer(dtype=np.int64)]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


# --------------------------------------------------------------------------
# meshes
@dataclass
class Mesh:
    """A simplicial mesh with the reference's derived data (nosh::mesh)."""

    x: np.ndarray  # (N, 3)
    cells: np.ndarray  # (T, nvc)
    edges: np.ndarray = field(default=None)  # (E, 2) canonical v0 < v1
    cell_edges: np.ndarray = field(default=None)
    length: np.ndarray = field(default=None)
    covolume: np.ndarray = field(default=None)
    cv: np.ndarray = field(default=None)

    @property
    def N(self):
        return self.x.shape[0]

    @property
    def T(self):
        return self.cells.shape[0]

    @property
    def E(self):
        return self.edges.shape[0]

    @property
    def nvc(self):
        return self.cells.shape[1]


def finish_mesh(x, cells) -> Mesh:
    """Edges, edge data and control volumes (src/mesh*.cpp restated in C)."""
    L = lib()
    x = np.ascontiguousarray(x, dtype=np.float64)
    cells = np.ascontiguousarray(cells, dtype=np.int32)
    N, T, nvc = x.shape[0], cells.shape[0], cells.shape[1]
    ne = 3 if nvc == 3 else 6
    edges = np.zeros((T * ne, 2), np.int32)
    cell_edges = np.zeros((T, ne), np.int32)
    E = L.nor_build_edges(nvc, N, T, cells.ravel(), edges.ravel(), cell_edges.ravel())
    edges = np.ascontiguousarray(edges[:E])
    length = np.zeros(E)
    covol = np.zeros(E)
    L.nor_edge_data(nvc, N, x.ravel(), E, edges.ravel(), T, cell_edges.ravel(), length, covol)
    cv = np.zeros(N)
    L.nor_control_volumes(nvc, N, x.ravel(), T, cells.ravel(), cv)
    return Mesh(x, cells, edges, cell_edges, length, covol, cv)


def gen_square(s: int, seed: int, jitter: float = 0.1):
    """Jittered unit square, s x s vertices, 2 right triangles per square."""
    N, T = s * s, 2 * (s - 1) ** 2
    x = np.zeros(3 * N)
    cells = np.zeros(3 * T, np.int32)
    psi = np.zeros(2 * N)
    lib().nor_gen_square(s, seed, jitter, x, cells, psi)
    return x.reshape(N, 3), cells.reshape(T, 3), psi


def gen_cube(m: int, seed: int, jitter: float = 0.1):
    """Jittered unit cube, m^3 cubes, 6 Kuhn tetrahedra per cube."""
    N, T = (m + 1) ** 3, 6 * m**3
    x = np.zeros(3 * N)
    cells = np.zeros(4 * T, np.int32)
    psi = np.zeros(2 * N)
    lib().nor_gen_cube(m, seed, jitter, x, cells, psi)
    return x.reshape(N, 3), cells.reshape(T, 4), psi


def mvp_constant_curl(x):
    """A = 1/2 (-y, x, 0) sampled per vertex (B = (0,0,1); scaled by mu)."""
    A = np.zeros_like(x)
    A[:, 0] = -0.5 * x[:, 1]
    A[:, 1] = 0.5 * x[:, 0]
    return A


def mvp_stress(x):
    """A = 1/2 (-y, x, 0) + 0.05 sin(2 pi z) (1, 0, 0), sampled per vertex."""
    A = mvp_constant_curl(x)
    A[:, 0] += 0.05 * np.sin(2.0 * np.pi * x[:, 2])
    return A


# --------------------------------------------------------------------------
# the reference's KAT meshes, reconstructed from test/*.cpp constants
def rectanglesmall() -> Mesh:
    """4 vertices at (+-5, +-0.5, 0), 2 triangles sharing the 0-1 diagonal.

    Vertex order chosen so the KEO matches the 8x8 matrix printed in
    test/keo.cpp:121-131 (vertex 0 = (-5,-0.5), its vertical neighbour 2,
    horizontal neighbour 3, opposite corner 1).
    """
    x = np.array([[-5.0, -0.5, 0.0], [5.0, 0.5, 0.0], [-5.0, 0.5, 0.0], [5.0, -0.5, 0.0]])
    cells = np.array([[0, 3, 1], [0, 1, 2]], np.int32)
    return finish_mesh(x, cells)


def cubesmall() -> Mesh:
    """8 vertices of [-.5,.5]^2 x [-5,5]; vertex id = x + 2y + 4z bits; the
    5-tet split that reproduces the constants of test/mesh.cpp:93-95."""
    x = np.array(
        [[(-0.5, 0.5)[v & 1], (-0.5, 0.5)[(v >> 1) & 1], (-5.0, 5.0)[(v >> 2) & 1]] for v in range(8)]
    )
    cells = np.array([[0, 1, 2, 4], [1, 2, 3, 7], [1, 4, 5, 7], [2, 4, 6, 7], [1, 2, 4, 7]], np.int32)
    return finish_mesh(x, cells)


# --------------------------------------------------------------------------
# operators (thin wrappers)
class Problem:
    """Fields + operators on a mesh: explicit-values A, V, thickness, g."""

    def __init__(self, mesh: Mesh, A: np.ndarray, V=-1.0, thickness=1.0):
        self.m = mesh
        N = mesh.N
        self.V = np.full(N, float(V)) if np.isscalar(V) else np.ascontiguousarray(V, np.float64)
        self.t = (
            np.full(N, float(thickness)) if np.isscalar(thickness) else np.ascontiguousarray(thickness, np.float64)
        )
        self.A = np.ascontiguousarray(A, np.float64)
        L = lib()
        E = mesh.E
        self.p = np.zeros(E)
        L.nor_edge_projection(E, mesh.edges.ravel(), mesh.x.ravel(), self.A.ravel(), self.p)
        self.alpha = np.zeros(E)
        L.nor_alpha(E, mesh.edges.ravel(), mesh.length, mesh.covolume, self.t, self.alpha)
        self.row_ptr = np.zeros(N + 1, np.int32)
        self.cols = np.zeros(N + 2 * E, np.int32)
        L.nor_complex_graph(N, E, mesh.edges.ravel(), self.row_ptr, self.cols)

    # -- KEO
    def keo_values(self, mu):
        v = np.zeros(2 * self.cols.size)
        lib().nor_keo_values(
            self.m.N, self.m.E, self.m.edges.ravel(), self.alpha, self.p, mu, self.row_ptr, self.cols, v
        )
        return v.view(np.complex128)

    def dkeo_values(self, mu, dp=None):
        dp = self.p if dp is None else dp
        v = np.zeros(2 * self.cols.size)
        lib().nor_dkeo_values(
            self.m.N, self.m.E, self.m.edges.ravel(), self.alpha, self.p, dp, mu, self.row_ptr, self.cols, v
        )
        return v.view(np.complex128)

    def keo_apply(self, mu, x):
        y = np.zeros(2 * self.m.N)
        lib().nor_keo_apply(self.m.N, self.m.E, self.m.edges.ravel(), self.alpha, self.p, mu, _f(x), y)
        return y

    def keo_real_dense(self, mu):
        """The real 2N x 2N KEO (Tpetra layout) as a dense array (tiny meshes)."""
        N = self.m.N
        Kd = np.zeros((2 * N, 2 * N))
        for k in range(2 * N):
            e = np.zeros(2 * N)
            e[k] = 1.0
            Kd[:, k] = self.keo_apply(mu, e)
        return Kd

    def compute_f(self, psi, g, mu):
        f = np.zeros(2 * self.m.N)
        lib().nor_compute_f(
            self.m.N, self.m.E, self.m.edges.ravel(), self.alpha, self.p, mu, g, self.m.cv, self.t, self.V, _f(psi), f
        )
        return f

    def dfdp(self, psi, g, mu, param: str, deriv_param: str = "mu"):
        dp = self.p if deriv_param == "mu" else np.zeros_like(self.p)
        out = np.zeros(2 * self.m.N)
        dV = np.zeros(self.m.N)
        lib().nor_dfdp(
            self.m.N, self.m.E, self.m.edges.ravel(), self.alpha, self.p, dp, mu,
            1 if param == "g" else 0, self.m.cv, self.t, dV, _f(psi), out,
        )
        return out

    def jac_diags(self, psi, g):
        d0 = np.zeros(2 * self.m.N)
        d1b = np.zeros(self.m.N)
        lib().nor_jac_diags(self.m.N, self.m.cv, self.t, self.V, g, _f(psi), d0, d1b)
        return d0, d1b

    def jac_apply(self, psi, g, mu, x):
        d0, d1b = self.jac_diags(psi, g)
        y = np.zeros(2 * self.m.N)
        lib().nor_jac_apply(self.m.N, self.m.E, self.m.edges.ravel(), self.alpha, self.p, mu, d0, d1b, _f(x), y)
        return y

    def kreg_apply(self, psi, g, mu, x):
        y = np.zeros(2 * self.m.N)
        lib().nor_kreg_apply(
            self.m.N, self.m.E, self.m.edges.ravel(), self.alpha, self.p, mu, g, self.m.cv, self.t, _f(psi), _f(x), y
        )
        return y

    def kreg_blocks(self, psi, g, mu):
        """K_reg in compact form: the off-diagonal complex values as (rows,
        cols, values) and the real 2x2 diagonal blocks (d0r, d0i, d1b) per
        vertex, K_ii included (src/keo_regularized.cpp:233-258)."""
        vals = self.keo_values(mu)
        N = self.m.N
        rows = np.repeat(np.arange(N), np.diff(self.row_ptr))
        diag = self.cols == rows
        kii = np.zeros(N)
        kii[rows[diag]] = vals[diag].real
        psi = _f(psi)
        re, im = psi[0::2], psi[1::2]
        w = g * self.m.cv * self.t
        al = w * 2.0 * (re * re + im * im)
        be = w * 2.0 * re * im
        ga = w * (re * re - im * im)
        return rows[~diag], self.cols[~diag], vals[~diag], (kii + al + ga, kii + al - ga, be)

    def cheb_presmooth(self, psi, g, mu, b, degree=2, ratio=15.0):
        """One block-Jacobi Chebyshev smoothing sweep of K_reg from x = 0 on
        right-hand side b: the pre-smoother of the GPU preconditioner's fine
        level, restated in FP64.  The reference only configures its MueLu
        smoother (src/keo_regularized.cpp:296-315), so this restates the
        smoother the GPU build defines: D the 2x2 diagonal blocks, lmax =
        1.1 max_i (1 + sum_j |K_ij| / lambda_min(D_i)) (Gershgorin), the
        Chebyshev polynomial of `degree` on [lmax / (1.1 ratio), lmax]."""
        import scipy.sparse as sp

        N = self.m.N
        r_, c_, v_, (a, d, bb) = self.kreg_blocks(psi, g, mu)
        Koff = sp.csr_matrix((v_, (r_, c_)), shape=(N, N))
        det = a * d - bb * bb
        ia, ie, if_ = d / det, a / det, -bb / det
        lmin_b = 0.5 * (a + d) - np.sqrt(0.25 * (a - d) ** 2 + bb * bb)
        rs = np.asarray(abs(Koff).sum(axis=1)).ravel()
        with np.errstate(divide="ignore"):
            bound = np.where((lmin_b > 0) & (det > 0), 1.0 + rs / lmin_b, 1e300)
        lmax = 1.1 * bound.max()
        lmin = lmax / (1.1 * ratio)
        theta, delta = 0.5 * (lmax + lmin), 0.5 * (lmax - lmin)
        sigma = theta / delta
        rho = 1.0 / sigma
        coef = [(None, None)]
        for _ in range(1, degree):
            rn = 1.0 / (2.0 * sigma - rho)
            coef.append((rn * rho, 2.0 * rn / delta))
            rho = rn
        b = _f(b)
        bz = b[0::2] + 1j * b[1::2]

        def dinv(z):
            return (ia * z.real + if_ * z.imag) + 1j * (if_ * z.real + ie * z.imag)

        def apply(z):
            y = Koff @ z
            return y + (a * z.real + bb * z.imag) + 1j * (bb * z.real + d * z.imag)

        dd = dinv(bz) / theta
        x = dd.copy()
        for k in range(1, degree):
            c1, c2 = coef[k]
            dd = c1 * dd + c2 * dinv(bz - apply(x))
            x = x + dd
        out = np.empty(2 * N)
        out[0::2], out[1::2] = x.real, x.imag
        return out

    def energy(self, psi):
        return lib().nor_energy(self.m.N, self.m.cv, _f(psi))

    def inner_product(self, phi, psi):
        return lib().nor_inner_product(self.m.N, self.m.cv, _f(phi), _f(psi))

    # -- scipy sparse forms (small cases: exact linear algebra for parity)
    def keo_csr_real(self, mu):
        import scipy.sparse as sp

        vals = self.keo_values(mu)
        return _complex_csr_to_real(self.row_ptr, self.cols, vals, self.m.N)

    def jac_csr_real(self, psi, g, mu):
        import scipy.sparse as sp

        d0, d1b = self.jac_diags(psi, g)
        N = self.m.N
        D = _diag_blocks(d0[0::2], d1b, d0[1::2])
        return (self.keo_csr_real(mu) + D).tocsr()

    def kreg_csr_real(self, psi, g, mu):
        N = self.m.N
        re, im = _f(psi)[0::2], _f(psi)[1::2]
        w = g * self.m.cv * self.t
        al = w * 2.0 * (re * re + im * im)
        be = w * 2.0 * re * im
        ga = w * (re * re - im * im)
        D = _diag_blocks(al + ga, be, al - ga)
        return (self.keo_csr_real(mu) + D).tocsr()


def _f(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _diag_blocks(a, b, d):
    """block-diagonal [[a, b], [b, d]] as a sparse 2N x 2N matrix"""
    import scipy.sparse as sp

    N = a.size
    rows = np.concatenate([2 * np.arange(N), 2 * np.arange(N), 2 * np.arange(N) + 1, 2 * np.arange(N) + 1])
    cols = np.concatenate([2 * np.arange(N), 2 * np.arange(N) + 1, 2 * np.arange(N), 2 * np.arange(N) + 1])
    vals = np.concatenate([a, b, b, d])
    return sp.csr_matrix((vals, (rows, cols)), shape=(2 * N, 2 * N))


def _complex_csr_to_real(row_ptr, cols, vals, N):
    import scipy.sparse as sp

    rows = np.repeat(np.arange(N), np.diff(row_ptr))
    cr, ci = vals.real, vals.imag
    R = np.concatenate([2 * rows, 2 * rows, 2 * rows + 1, 2 * rows + 1])
    Cc = np.concatenate([2 * cols, 2 * cols + 1, 2 * cols, 2 * cols + 1])
    V = np.concatenate([cr, -ci, ci, cr])
    return sp.csr_matrix((V, (R, Cc)), shape=(2 * N, 2 * N))


def real_graph_from_complex(row_ptr, cols):
    """Expand the complex graph into the Tpetra real 2N x 2N graph (0-based):
    rows 2i and 2i+1 both hold columns 2j, 2j+1 for every j in row i."""
    N = row_ptr.size - 1
    deg = np.diff(row_ptr)
    rp = np.zeros(2 * N + 1, np.int64)
    rp[1::2] = 2 * deg
    rp[2::2] = 2 * deg
    rp = np.cumsum(rp)
    out = np.empty(rp[-1], np.int32)
    for i in range(N):
        c = cols[row_ptr[i] : row_ptr[i + 1]]
        pair = np.stack([2 * c, 2 * c + 1], axis=1).ravel()
        out[rp[2 * i] : rp[2 * i + 1]] = pair
        out[rp[2 * i + 1] : rp[2 * i + 2]] = pair
    return rp, out


# --------------------------------------------------------------------------
# Newton with exact linear algebra (small cases): the converged-state oracle.
def newton_exact(P: Problem, psi0, g, mu, tol=1e-12, max_it=30, phase_fix=False):
    """Full-step Newton on F(psi) = 0 with MINRES preconditioned by an exact
    LU of the regularised KEO (scipy), FP64.  The Jacobian is singular along
    the gauge direction i*psi; MINRES handles the consistent singular system.
    With ``phase_fix`` every update is made orthogonal to i*psi, the
    solution of the reference's bordered system
    (src/bordering/ModelEvaluator_Bordered.cpp).  Returns
    (psi, [||F|| per step])."""
    import scipy.sparse.linalg as spla

    psi = np.array(psi0, dtype=np.float64, copy=True)
    hist = [np.linalg.norm(P.compute_f(psi, g, mu))]
    for _ in range(max_it):
        if hist[-1] <= tol:
            break
        F = P.compute_f(psi, g, mu)
        J = P.jac_csr_real(psi, g, mu)
        lu = spla.splu(P.kreg_csr_real(psi, g, mu).tocsc())
        M = spla.LinearOperator(J.shape, matvec=lu.solve)
        dx, _ = spla.minres(J, -F, M=M, rtol=1e-13, maxiter=2000)
        if phase_fix:
            ip = _gauge(psi)
            dx = dx - (ip @ dx) / (ip @ ip) * ip
        psi = psi + dx
        hist.append(np.linalg.norm(P.compute_f(psi, g, mu)))
    return psi, hist


def _exact_minres(P: Problem, psi, g, mu, rhs, rtol=1e-13):
    import scipy.sparse.linalg as spla

    J = P.jac_csr_real(psi, g, mu)
    lu = spla.splu(P.kreg_csr_real(psi, g, mu).tocsc())
    M = spla.LinearOperator(J.shape, matvec=lu.solve)
    x, _ = spla.minres(J, rhs, M=M, rtol=rtol, maxiter=4000)
    return x


def _gauge(psi):
    """i*psi in the interleaved real layout (the U(1) null direction of J)."""
    out = np.empty_like(psi)
    out[0::2], out[1::2] = -psi[1::2], psi[0::2]
    return out


def tangent(P: Problem, psi, g, mu):
    """dpsi/dmu at a converged state: J v = -dF/dmu (LOCA "Tangent"
    predictor; dF/dmu = (dK/dmu) psi, src/model_evaluator_nls.cpp:632-695),
    with the component along the gauge direction i*psi removed."""
    v = _exact_minres(P, psi, g, mu, -P.dfdp(psi, g, mu, "mu"))
    ip = _gauge(psi)
    return v - (ip @ v) / (ip @ ip) * ip


def arclength_step(P: Problem, psi0, mu0, ds, g=1.0, prev=None, predictor="tangent", theta=1.0, tol=1e-12,
                   max_it=20):
    """One pseudo-arclength step (Keller; LOCA "Arc Length",
    examples/conf.xml:43) with exact-LU-preconditioned MINRES solves.

    Norm: ||(x, m)||^2 = x.x/n + theta^2 m^2 (n = 2N).  The unit tangent is
    (tangent(psi0), 1) or the phase-aligned secant (psi0 - psi1, mu0 - mu1)
    from ``prev = (psi1, mu1)``, oriented along that secant when given.
    Corrector: Newton on F and the constraint
    <tau, psi - psi0>/n + theta^2 tau_mu (mu - mu0) = ds by bordering.
    Returns (psi, mu, tau_mu, newton_iters)."""
    n = psi0.size
    th2 = theta * theta
    sec = None
    if prev is not None:
        sec = psi0 - align_phase(prev[0], psi0)
        sec_mu = mu0 - prev[1]
    if predictor == "tangent" or sec is None:
        tx, tm = tangent(P, psi0, g, mu0), 1.0
    else:
        tx, tm = sec.copy(), sec_mu
    sc = 1.0 / np.sqrt(tx @ tx / n + th2 * tm * tm)
    if sec is not None and tx @ sec / n + th2 * tm * sec_mu < 0:
        sc = -sc
    tx, tm = tx * sc, tm * sc
    psi, mu = psi0 + ds * tx, mu0 + ds * tm
    its = 0
    for its in range(max_it + 1):
        F = P.compute_f(psi, g, mu)
        if np.linalg.norm(F) <= tol or its == max_it:
            break
        a = _exact_minres(P, psi, g, mu, F)
        b = _exact_minres(P, psi, g, mu, P.dfdp(psi, g, mu, "mu"))
        dmu = (tx @ a / n) / (th2 * tm - tx @ b / n)
        psi = psi - a - dmu * b
        mu = mu + dmu
    return psi, mu, tm, its


def lowest_eigenvalues(P: Problem, psi, g, mu, k, sigma=-0.1):
    """The k eigenvalues of the real-symmetric Jacobian nearest ``sigma``
    from below the spectrum (shift-invert Lanczos, scipy eigsh), without the
    U(1) gauge mode i*psi (the eigenvector overlapping it most is dropped).
    Stands in for the reference's Anasazi solve on the Jacobian
    (executables/nosh-eig/nosh-eig.cpp)."""
    import scipy.sparse.linalg as spla

    J = P.jac_csr_real(psi, g, mu).tocsc()
    vals, vecs = spla.eigsh(J, k=k + 1, sigma=sigma, which="LM")
    u = _gauge(psi)
    u = u / np.linalg.norm(u)
    drop = int(np.argmax(np.abs(u @ vecs)))
    return np.sort(np.delete(vals, drop))


def align_phase(psi, ref):
    """Rotate psi by the global phase that best matches ref (U(1) gauge)."""
    z = psi[0::2] + 1j * psi[1::2]
    zr = ref[0::2] + 1j * ref[1::2]
    c = np.vdot(z, zr)
    z = z * (c / abs(c))
    out = np.empty_like(psi)
    out[0::2], out[1::2] = z.real, z.imag
    return out


# --------------------------------------------------------------------------
class CpuSolver:
    """The C FP64 Newton / AMG-MINRES / continuation solver (nosh_solver.c):
    the CPU baseline, OpenMP over OMP_NUM_THREADS host cores."""

    def __init__(self, P: Problem, g=1.0):
        L = lib()
        m = P.m
        self.P = P
        self._h = L.nor_solver_create(m.N, m.E, m.edges.ravel(), P.alpha, P.p, m.cv, P.t, P.V, g)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().nor_solver_destroy(self._h)
            self._h = None

    @staticmethod
    def threads():
        return lib().nor_num_threads()

    @staticmethod
    def set_threads(n):
        """OpenMP threads of the solver calls that follow on this thread;
        returns the previous count."""
        return lib().nor_set_num_threads(int(n))

    def newton(self, psi, mu, tol=1e-10, max_newton=20):
        ni, ki = C.c_int(), C.c_int()
        f0, f1 = C.c_double(), C.c_double()
        rc = lib().nor_newton(self._h, psi, mu, tol, max_newton, C.byref(ni), C.byref(ki), C.byref(f0), C.byref(f1))
        return {"status": rc, "newton_iters": ni.value, "krylov_iters": ki.value, "f_norm0": f0.value,
                "f_norm": f1.value}

    def continuation_step(self, x, x_prev, mu_new, mu_cur, mu_prev, tol=1e-10):
        ni, ki = C.c_int(), C.c_int()
        f0, f1 = C.c_double(), C.c_double()
        xp = None if x_prev is None else C.c_void_p(x_prev.ctypes.data)
        rc = lib().nor_continuation_step(self._h, x, xp, mu_new, mu_cur, mu_prev, tol, C.byref(ni), C.byref(ki),
                                         C.byref(f0), C.byref(f1))
        return {"status": rc, "newton_iters": ni.value, "krylov_iters": ki.value, "f_norm0": f0.value,
                "f_norm": f1.value}

    def amg_levels(self):
        s = np.zeros(16, np.int64)
        n = lib().nor_amg_levels(self._h, s)
        return list(s[:n])
