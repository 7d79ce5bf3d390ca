"""nosh_gb300 -- GB300-native Newton-Krylov core for nosh's GL / NLS problem.

Python host mirror of the reference's C++ classes over the C ABI of
``libnosh_gb300.so`` (``include/nosh_gb300.h``).  Class and method names
follow nschloe/nosh:

=========================================  ====================================
reference (src/...)                        here
=========================================  ====================================
``nosh::mesh`` (mesh.hpp)                  :class:`mesh`
``vector_field::explicit_values``          ``mvp`` array given to :class:`nls`
``parameter_matrix::keo`` / ``DkeoDP``     :attr:`nls.keo` / :attr:`nls.dkeo_dp`
``jacobian_operator``                      :meth:`nls.create_W_op`
``keo_regularized``                        :meth:`nls.create_W_prec`
``model_evaluator::nls``                   :class:`nls`
=========================================  ====================================

Vectors are numpy float64 arrays (host) or anything exposing a CUDA device
pointer via ``data_ptr()`` (e.g. a torch tensor); complex states are
interleaved ``[Re0, Im0, Re1, Im1, ...]``.  There is no CPU fallback: the
compiled library is mapped on the first call that needs it (so the numpy-only
modules :mod:`nosh_gb300.meshgen` and :mod:`nosh_gb300.batch` import without
it), that call raises ImportError when the library is missing, and every
compute call fails with :class:`NoshError` when no GPU is present.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libnosh_gb300.so")


class _Library:
    """The ctypes view of ``libnosh_gb300.so``, mapped on first attribute
    access with every entry point's signature set."""

    def __init__(self):
        self._cdll = None

    def load(self):
        if self._cdll is None:
            if not os.path.exists(LIB_PATH):
                raise ImportError(
                    f"nosh_gb300: compiled library {LIB_PATH} is missing; build it with "
                    "`python nosh_gb300/build.py` (nvcc, sm_103a)"
                )
            cdll = C.CDLL(LIB_PATH)
            for name, (res, args) in _SIGS.items():
                fn = getattr(cdll, name)
                fn.restype = res
                fn.argtypes = args
            self._cdll = cdll
        return self._cdll

    def __getattr__(self, name):
        return getattr(self.load(), name)


_lib = _Library()

OK = 0
ERR_INVALID, ERR_CUDA, ERR_NOT_CONVERGED, ERR_NAN, ERR_BREAKDOWN = 1, 2, 3, 4, 5
ERR_UNSUPPORTED, ERR_MESH, ERR_NO_MEMORY = 6, 7, 8
PREC_FP64, PREC_MIXED = 0, 1
SPMV_AUTO, SPMV_STAGED, SPMV_WARP = 0, 1, 2
NO_TRANS, TRANS = 0, 1
PREDICT_NONE, PREDICT_SECANT, PREDICT_TANGENT, PREDICT_QUADRATIC, PREDICT_LEARNED, PREDICT_CUBIC = 0, 1, 2, 3, 4, 5
KERNEL_JACOBIAN, KERNEL_SMOOTHER, KERNEL_ALL = 0, 1, 2


class NoshError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class NewtonOptions(C.Structure):
    _fields_ = [
        ("tol", C.c_double),
        ("max_newton", C.c_int),
        ("forcing", C.c_double),
        ("max_krylov", C.c_int),
        ("precision", C.c_int),
        ("verbose", C.c_int),
        ("refine", C.c_double),
        ("phase_fix", C.c_int),
    ]


class NewtonStats(C.Structure):
    _fields_ = [
        ("newton_iters", C.c_int),
        ("krylov_iters", C.c_int),
        ("f_norm", C.c_double),
        ("f_norm0", C.c_double),
        ("status", C.c_int),
        ("residual_updates", C.c_int),
        ("f_norm_bound", C.c_double),
    ]


_P, _I64, _D, _I = C.c_void_p, C.c_int64, C.c_double, C.c_int
_SIGS = {
    "nosh_last_error": (C.c_char_p, []),
    "nosh_version": (_I, []),
    "nosh_device_count": (_I, [C.POINTER(_I)]),
    "nosh_mesh_create": (_I, [_P, _I64, _P, _I64, _I, C.POINTER(_P)]),
    "nosh_mesh_destroy": (_I, [_P]),
    "nosh_mesh_sizes": (_I, [_P, C.POINTER(_I64), C.POINTER(_I64), C.POINTER(_I64), C.POINTER(_I64)]),
    "nosh_mesh_edges": (_I, [_P, _P]),
    "nosh_mesh_edge_gids_complex": (_I, [_P, _P]),
    "nosh_mesh_edge_data": (_I, [_P, _P, _P]),
    "nosh_mesh_control_volumes": (_I, [_P, _P]),
    "nosh_mesh_complex_graph": (_I, [_P, _P, _P]),
    "nosh_nls_create": (_I, [_P, _P, _D, _P, _D, _P, C.c_char_p, C.POINTER(_P)]),
    "nosh_nls_destroy": (_I, [_P]),
    "nosh_nls_num_params": (_I, [_P, C.POINTER(_I)]),
    "nosh_nls_param_name": (_I, [_P, _I, C.c_char_p, C.c_size_t]),
    "nosh_nls_set_precision": (_I, [_P, _I]),
    "nosh_nls_set_amg_options": (_I, [_P, _I, _I, _I, _I, _D, _D]),
    "nosh_nls_set_spmv_schedule": (_I, [_P, _I]),
    "nosh_nls_set_stage_wait_limit": (_I, [_P, _I64]),
    "nosh_diag_stream_read": (_I, [_P, _I64, _P, _P]),
    "nosh_nls_set_index_checks": (_I, [_P, _I]),
    "nosh_nls_set_forcing_aim": (_I, [_P, _D]),
    "nosh_nls_set_launch_overlap": (_I, [_P, _I]),
    "nosh_graph_check": (_I, [_I64, _I64, _P, _P, _P]),
    "nosh_nls_amg_levels": (_I, [_P, C.POINTER(_I), _P, _I, C.POINTER(_I)]),
    "nosh_nls_set_systems": (_I, [_P, _I64, _P, _P]),
    "nosh_nls_system_norms": (_I, [_P, _P]),
    "nosh_nls_system_iterations": (_I, [_P, _P, _P]),
    "nosh_nls_stream": (_I, [_P, C.POINTER(_P)]),
    "nosh_nls_compute_f": (_I, [_P, _P, _P, _P]),
    "nosh_nls_compute_f_norm": (_I, [_P, _P, _P, _P, C.POINTER(_D)]),
    "nosh_nls_compute_dfdp": (_I, [_P, _P, _P, _P]),
    "nosh_nls_gibbs_energy": (_I, [_P, _P, C.POINTER(_D)]),
    "nosh_nls_inner_product": (_I, [_P, _P, _P, C.POINTER(_D)]),
    "nosh_keo_set_parameters": (_I, [_P, _P]),
    "nosh_keo_values": (_I, [_P, _P]),
    "nosh_keo_apply": (_I, [_P, _P, _P]),
    "nosh_dkeo_set_parameters": (_I, [_P, _P]),
    "nosh_dkeo_values": (_I, [_P, _P]),
    "nosh_dkeo_apply": (_I, [_P, _P, _P]),
    "nosh_jacobian_rebuild": (_I, [_P, _P, _P]),
    "nosh_jacobian_apply": (_I, [_P, _P, _P, _I, _I, _D, _D]),
    "nosh_keo_regularized_rebuild": (_I, [_P, _P, _P]),
    "nosh_keo_regularized_apply": (_I, [_P, _P, _P, _I, _I, _D, _D]),
    "nosh_keo_regularized_operator_apply": (_I, [_P, _P, _P]),
    "nosh_keo_regularized_smoother_apply": (_I, [_P, _P, _P]),
    "nosh_eig_lowest": (_I, [_P, _P, _P, _I, _D, _I, _I, _I, C.c_uint64, _P, _P, C.POINTER(_I)]),
    "nosh_newton_default_options": (None, [C.POINTER(NewtonOptions)]),
    "nosh_newton_solve": (_I, [_P, _P, _P, C.POINTER(NewtonOptions), C.POINTER(NewtonStats)]),
    "nosh_continuation_step": (_I, [_P, _P, _P, _P, _D, _D, _I, C.POINTER(NewtonOptions),
                                    C.POINTER(NewtonStats)]),
    "nosh_continuation_create": (_I, [_P, _P, _D, C.POINTER(_P)]),
    "nosh_continuation_destroy": (_I, [_P]),
    "nosh_continuation_advance": (_I, [_P, _D, _I, C.POINTER(NewtonOptions), C.POINTER(NewtonStats)]),
    "nosh_continuation_state": (_I, [_P, _P, C.POINTER(_D)]),
    "nosh_nls_get_precision": (_I, [_P, C.POINTER(_I)]),
    "nosh_continuation_advance_arclength": (_I, [_P, _D, _I, _D, C.POINTER(NewtonOptions),
                                                 C.POINTER(NewtonStats)]),
    "nosh_continuation_tangent": (_I, [_P, C.POINTER(_D), C.POINTER(_D)]),
    "nosh_continuation_learning": (_I, [_P, _I, _I, _D]),
    "nosh_continuation_inference_period": (_I, [_P, _I]),
    "nosh_continuation_predictor_residuals": (_I, [_P, _D, _P]),
    "nosh_continuation_last_prediction": (_I, [_P, C.POINTER(_I), C.POINTER(_D), C.POINTER(_D), C.POINTER(_D),
                                               C.POINTER(_D)]),
    "nosh_mpnn_create": (_I, [_P, C.POINTER(_P)]),
    "nosh_mpnn_destroy": (_I, [_P]),
    "nosh_mpnn_num_params": (_I, [_P, C.POINTER(_I64)]),
    "nosh_mpnn_params": (_I, [_P, _P, _P]),
    "nosh_mpnn_edge_features": (_I, [_P, _P]),
    "nosh_mpnn_forward": (_I, [_P, _P, _P]),
    "nosh_mpnn_loss_grad": (_I, [_P, _P, _P, C.POINTER(_D), _P]),
    "nosh_nls_profile_enable": (_I, [_P, _I]),
    "nosh_nls_profile_read": (_I, [_P, _I, C.POINTER(_I64), C.POINTER(_D), C.POINTER(_D)]),
}


def lib():
    """The loaded ctypes library (for low-level use and tests); maps it on
    first use."""
    return _lib.load()


def _check(rc, allow=()):
    if rc != OK and rc not in allow:
        raise NoshError(rc, _lib.nosh_last_error().decode())
    return rc


def _ptr(a):
    """Raw pointer of a numpy array (host) or a device tensor (data_ptr)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    if isinstance(a, np.ndarray):
        if not a.flags["C_CONTIGUOUS"]:
            raise ValueError("array must be C-contiguous")
        return C.c_void_p(a.ctypes.data)
    raise TypeError(f"unsupported vector type {type(a)}")


def _f64(a):
    if hasattr(a, "data_ptr"):
        return a
    return np.ascontiguousarray(a, dtype=np.float64)


def stream_read(buf, nbytes, out_word, stream=None):
    """Diagnostics: one launch streaming ``nbytes`` of the device buffer
    ``buf`` (XOR-folded into the 32-bit device word ``out_word``), enqueued
    on ``stream`` (a cudaStream_t handle, default stream when None)."""
    _check(_lib.nosh_diag_stream_read(_ptr(buf), int(nbytes), _ptr(out_word), C.c_void_p(stream or 0)))


def graph_check(row_ptr, cols, stream=None):
    """Validate an off-diagonal CSR graph held in device memory (tensors with
    data_ptr); raises NoshError naming the first offending position."""
    n = int(row_ptr.numel()) - 1
    _check(_lib.nosh_graph_check(n, int(cols.numel()), _ptr(row_ptr), _ptr(cols), C.c_void_p(stream or 0)))


def device_count() -> int:
    n = C.c_int(0)
    rc = _lib.nosh_device_count(C.byref(n))
    return n.value if rc == OK else 0


# ---------------------------------------------------------------------------
class mesh:
    """``nosh::mesh`` (src/mesh.hpp): simplicial mesh with edges, edge data
    (length, covolume), control volumes and the KEO graph.  Built from
    vertex coordinates ``(N, 3)`` and cells ``(T, 3|4)``."""

    def __init__(self, coords, cells):
        x = np.ascontiguousarray(coords, dtype=np.float64)
        c = np.ascontiguousarray(cells, dtype=np.int32)
        if x.ndim != 2 or x.shape[1] != 3 or c.ndim != 2 or c.shape[1] not in (3, 4):
            raise ValueError("coords must be (N,3) and cells (T,3) or (T,4)")
        h = C.c_void_p()
        _check(_lib.nosh_mesh_create(_ptr(x), x.shape[0], _ptr(c), c.shape[0], c.shape[1], C.byref(h)))
        self._h = h
        n, e, t, z = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
        _check(_lib.nosh_mesh_sizes(h, C.byref(n), C.byref(e), C.byref(t), C.byref(z)))
        self.num_vertices, self.num_edges, self.num_cells, self.nnz_blocks = n.value, e.value, t.value, z.value
        self.vertices_per_cell = c.shape[1]

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            _lib.nosh_mesh_destroy(h)
            self._h = None

    def my_edges(self) -> np.ndarray:
        out = np.empty((self.num_edges, 2), np.int32)
        _check(_lib.nosh_mesh_edges(self._h, _ptr(out)))
        return out

    @property
    def edge_gids_complex(self) -> np.ndarray:
        out = np.empty((self.num_edges, 4), np.int32)
        _check(_lib.nosh_mesh_edge_gids_complex(self._h, _ptr(out)))
        return out

    def get_edge_data(self):
        ln = np.empty(self.num_edges)
        cov = np.empty(self.num_edges)
        _check(_lib.nosh_mesh_edge_data(self._h, _ptr(ln), _ptr(cov)))
        return ln, cov

    def control_volumes(self) -> np.ndarray:
        out = np.empty(self.num_vertices)
        _check(_lib.nosh_mesh_control_volumes(self._h, _ptr(out)))
        return out

    def build_complex_graph(self):
        rp = np.empty(self.num_vertices + 1, np.int32)
        ci = np.empty(self.nnz_blocks, np.int32)
        _check(_lib.nosh_mesh_complex_graph(self._h, _ptr(rp), _ptr(ci)))
        return rp, ci


# ---------------------------------------------------------------------------
class _Matrix:
    """``parameter_matrix::keo`` / ``DkeoDP`` view of an nls handle."""

    def __init__(self, owner, kind):
        self._o, self._k = owner, kind

    def set_parameters(self, params: dict):
        p = self._o._pvec(params)
        fn = _lib.nosh_keo_set_parameters if self._k == "keo" else _lib.nosh_dkeo_set_parameters
        _check(fn(self._o._h, _ptr(p)))

    def values(self) -> np.ndarray:
        """Complex values in ``mesh.build_complex_graph()`` order."""
        out = np.empty(2 * self._o.mesh.nnz_blocks)
        fn = _lib.nosh_keo_values if self._k == "keo" else _lib.nosh_dkeo_values
        _check(fn(self._o._h, _ptr(out)))
        return out.view(np.complex128)

    def apply(self, x, y=None):
        x = _f64(x)
        y = np.empty(2 * self._o.n) if y is None else y
        fn = _lib.nosh_keo_apply if self._k == "keo" else _lib.nosh_dkeo_apply
        _check(fn(self._o._h, _ptr(x), _ptr(y)))
        return y


class jacobian_operator:
    """``nosh::jacobian_operator`` (src/jacobian_operator.hpp)."""

    def __init__(self, owner):
        self._o = owner

    def rebuild(self, params: dict, x):
        _check(_lib.nosh_jacobian_rebuild(self._o._h, _ptr(self._o._pvec(params)), _ptr(_f64(x))))

    def apply(self, X, Y=None, mode=NO_TRANS, alpha=1.0, beta=0.0):
        X = _f64(X)
        nvec = 1 if getattr(X, "ndim", 1) == 1 else X.shape[0]
        Y = np.empty_like(X) if Y is None else Y
        _check(_lib.nosh_jacobian_apply(self._o._h, _ptr(X), _ptr(Y), nvec, mode, alpha, beta))
        return Y


class keo_regularized:
    """``nosh::keo_regularized`` (src/keo_regularized.hpp): regularised KEO
    and its AMG V-cycle (``apply`` = one cycle, as ``num_cycles_ == 1``)."""

    def __init__(self, owner):
        self._o = owner

    def rebuild(self, params: dict, x):
        _check(_lib.nosh_keo_regularized_rebuild(self._o._h, _ptr(self._o._pvec(params)), _ptr(_f64(x))))

    def apply(self, X, Y=None, mode=NO_TRANS, alpha=1.0, beta=0.0):
        X = _f64(X)
        nvec = 1 if getattr(X, "ndim", 1) == 1 else X.shape[0]
        Y = np.empty_like(X) if Y is None else Y
        _check(_lib.nosh_keo_regularized_apply(self._o._h, _ptr(X), _ptr(Y), nvec, mode, alpha, beta))
        return Y

    def smoother_apply(self, x, y=None):
        """The fine level's Chebyshev smoothing sweep from zero on right-hand
        side x (the V-cycle's pre-smoother alone), in the handle's precision."""
        x = _f64(x)
        y = np.empty(2 * self._o.n) if y is None else y
        _check(_lib.nosh_keo_regularized_smoother_apply(self._o._h, _ptr(x), _ptr(y)))
        return y

    def operator_apply(self, x, y=None):
        x = _f64(x)
        y = np.empty(2 * self._o.n) if y is None else y
        _check(_lib.nosh_keo_regularized_operator_apply(self._o._h, _ptr(x), _ptr(y)))
        return y


class nls:
    """``nosh::model_evaluator::nls`` (src/model_evaluator_nls.cpp:57-138).

    ``mvp``: (N,3) vector potential sampled per vertex (explicit values);
    ``scalar_potential``, ``thickness``: scalars or (N,) arrays.
    """

    def __init__(self, mesh_: mesh, mvp, scalar_potential=-1.0, g=1.0, thickness=1.0, mu=0.0,
                 deriv_parameter="mu", precision=PREC_MIXED):
        self.mesh = mesh_
        self.n = mesh_.num_vertices
        N = self.n
        A = np.ascontiguousarray(mvp, dtype=np.float64).reshape(N, 3)
        V = np.full(N, float(scalar_potential)) if np.isscalar(scalar_potential) else np.ascontiguousarray(
            scalar_potential, np.float64)
        t = np.full(N, float(thickness)) if np.isscalar(thickness) else np.ascontiguousarray(thickness, np.float64)
        h = C.c_void_p()
        _check(_lib.nosh_nls_create(mesh_._h, _ptr(A), mu, _ptr(V), g, _ptr(t), deriv_parameter.encode(),
                                    C.byref(h)))
        self._h = h
        self.keo = _Matrix(self, "keo")
        self.dkeo_dp = _Matrix(self, "dkeo")
        self.set_precision(precision)
        self.nominal = {"g": g, "mu": mu}

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            _lib.nosh_nls_destroy(h)
            self._h = None

    def set_precision(self, precision):
        _check(_lib.nosh_nls_set_precision(self._h, precision))
        self.precision = precision

    def get_p_names(self):
        n = C.c_int()
        _check(_lib.nosh_nls_num_params(self._h, C.byref(n)))
        buf = C.create_string_buffer(32)
        names = []
        for k in range(n.value):
            _check(_lib.nosh_nls_param_name(self._h, k, buf, 32))
            names.append(buf.value.decode())
        return names

    def _pvec(self, params):
        if isinstance(params, dict):
            p = {**self.nominal, **params}
            return np.array([p["g"], p["mu"]], np.float64)
        return np.ascontiguousarray(params, np.float64)

    def set_amg_options(self, max_levels=10, coarse_size=64, smooth_degree=2, reuse_period=8,
                        strength_threshold=None, cheb_ratio=None):
        """Preconditioner options (MueLu parameter list of the reference);
        the hierarchy is rebuilt at the next Newton step."""
        tri = self.mesh.vertices_per_cell == 3
        if strength_threshold is None:
            strength_threshold = 0.05 if tri else 0.0
        if cheb_ratio is None:
            cheb_ratio = 30.0 if tri else 15.0
        _check(_lib.nosh_nls_set_amg_options(self._h, max_levels, coarse_size, smooth_degree, reuse_period,
                                             strength_threshold, cheb_ratio))

    def set_systems(self, vertex_offsets, mu):
        """Batched independent solves: the mesh is the disjoint union of
        len(mu) systems, system s owning vertices [offsets[s], offsets[s+1])
        and using its own mu (see nosh_nls_set_systems)."""
        off = np.ascontiguousarray(vertex_offsets, np.int64)
        mu = np.ascontiguousarray(mu, np.float64)
        if off.size != mu.size + 1:
            raise ValueError("need len(mu) + 1 offsets")
        _check(_lib.nosh_nls_set_systems(self._h, mu.size, _ptr(off), _ptr(mu)))
        self.num_systems = mu.size

    def system_norms(self):
        """Per-system ||F_s|| of the last residual a Newton solve evaluated."""
        out = np.empty(self.num_systems)
        _check(_lib.nosh_nls_system_norms(self._h, _ptr(out)))
        return out

    def system_iterations(self):
        """(Newton steps, MINRES iterations) per system of the last Newton
        solve (each system has its own MINRES recurrence)."""
        nw = np.zeros(self.num_systems, np.int32)
        kr = np.zeros(self.num_systems, np.int32)
        _check(_lib.nosh_nls_system_iterations(self._h, _ptr(nw), _ptr(kr)))
        return nw, kr

    def amg_levels(self):
        """(level sizes, first tail level) of the preconditioner hierarchy
        (empty before the first Newton step)."""
        n, tl = C.c_int(), C.c_int()
        sizes = np.zeros(16, np.int64)
        _check(_lib.nosh_nls_amg_levels(self._h, C.byref(n), _ptr(sizes), 16, C.byref(tl)))
        return sizes[: n.value].tolist(), tl.value

    def set_spmv_schedule(self, schedule):
        """SPMV_AUTO, SPMV_STAGED or SPMV_WARP (see nosh_gb300.h)."""
        _check(_lib.nosh_nls_set_spmv_schedule(self._h, schedule))

    def set_forcing_aim(self, aim):
        """Fraction of the Newton target a step's forcing term aims at
        (default 0.5; see nosh_nls_set_forcing_aim)."""
        _check(_lib.nosh_nls_set_forcing_aim(self._h, float(aim)))

    def set_launch_overlap(self, enable=True):
        """Overlapped launches of the MINRES iteration and V-cycle kernels
        (programmatic dependent launch; on by default; see
        nosh_nls_set_launch_overlap)."""
        _check(_lib.nosh_nls_set_launch_overlap(self._h, 1 if enable else 0))

    def set_index_checks(self, enable=True):
        """Index-check mode: the KEO graph is validated on the device before
        every compute call (see nosh_nls_set_index_checks)."""
        _check(_lib.nosh_nls_set_index_checks(self._h, 1 if enable else 0))

    def set_stage_wait_limit(self, polls):
        """Diagnostics: bound (mbarrier polls) of the staged SpMV's waits for
        its row copies; < 0 restores the default, 0 makes them give up at
        once (see nosh_nls_set_stage_wait_limit)."""
        _check(_lib.nosh_nls_set_stage_wait_limit(self._h, int(polls)))

    def stream(self) -> int:
        s = C.c_void_p()
        _check(_lib.nosh_nls_stream(self._h, C.byref(s)))
        return s.value or 0

    # -- evalModel pieces
    def compute_f(self, x, params, f=None, with_norm=False):
        x = _f64(x)
        f = np.empty(2 * self.n) if f is None else f
        nrm = C.c_double()
        _check(_lib.nosh_nls_compute_f_norm(self._h, _ptr(x), _ptr(self._pvec(params)), _ptr(f),
                                            C.byref(nrm) if with_norm else None))
        return (f, nrm.value) if with_norm else f

    def compute_dfdp(self, x, params):
        out = np.empty((2, 2 * self.n))
        _check(_lib.nosh_nls_compute_dfdp(self._h, _ptr(_f64(x)), _ptr(self._pvec(params)), _ptr(out)))
        return out

    def create_W_op(self):
        return jacobian_operator(self)

    def create_W_prec(self):
        return keo_regularized(self)

    def gibbs_energy(self, psi):
        out = C.c_double()
        _check(_lib.nosh_nls_gibbs_energy(self._h, _ptr(_f64(psi)), C.byref(out)))
        return out.value

    def inner_product(self, phi, psi):
        out = C.c_double()
        _check(_lib.nosh_nls_inner_product(self._h, _ptr(_f64(phi)), _ptr(_f64(psi)), C.byref(out)))
        return out.value

    # -- kernel timing (roofline figures)
    def profile(self, enable: bool):
        _check(_lib.nosh_nls_profile_enable(self._h, 1 if enable else 0))

    def profile_read(self, kernel):
        """(launches, total device ms, total algorithmic bytes) since the
        last read of this kernel class; resets it."""
        n, ms, b = C.c_int64(), C.c_double(), C.c_double()
        _check(_lib.nosh_nls_profile_read(self._h, kernel, C.byref(n), C.byref(ms), C.byref(b)))
        return n.value, ms.value, b.value

    # -- solvers
    def _options(self, tol, max_newton, forcing, max_krylov, precision, verbose, refine=0.0, phase_fix=False):
        o = NewtonOptions()
        _lib.nosh_newton_default_options(C.byref(o))
        o.tol, o.max_newton, o.forcing, o.max_krylov = tol, max_newton, forcing, max_krylov
        o.refine = refine
        o.phase_fix = 1 if phase_fix else 0
        o.precision = self.precision if precision is None else precision
        o.verbose = verbose
        return o

    @staticmethod
    def _stats(st):
        return {
            "newton_iters": st.newton_iters,
            "krylov_iters": st.krylov_iters,
            "f_norm": st.f_norm,
            "f_norm0": st.f_norm0,
            "status": st.status,
            "residual_updates": st.residual_updates,
            "f_norm_bound": st.f_norm_bound,
        }

    def continuation_step(self, x, x_prev, mu_new, mu_cur, mu_prev=float("nan"), predictor=PREDICT_SECANT,
                          params=None, tol=1e-10, max_newton=20, forcing=0.0, max_krylov=1000, precision=None,
                          verbose=0):
        """One natural continuation step to ``mu_new`` (LOCA stepper);
        ``x`` (state at ``mu_cur``) becomes the state at ``mu_new`` and
        ``x_prev`` (state at ``mu_prev``) becomes the state at ``mu_cur``."""
        p = self._pvec({**(params or {}), "mu": mu_new})
        o = self._options(tol, max_newton, forcing, max_krylov, precision, verbose)
        st = NewtonStats()
        rc = _lib.nosh_continuation_step(self._h, _ptr(x), _ptr(x_prev), _ptr(p), mu_cur, mu_prev, predictor,
                                         C.byref(o), C.byref(st))
        _check(rc, allow=(ERR_NOT_CONVERGED,))
        return self._stats(st)

    def newton(self, x, params, tol=1e-10, max_newton=20, forcing=0.0, max_krylov=1000, precision=None,
               verbose=0, refine=0.0, phase_fix=False):
        """Full-step inexact Newton with AMG-preconditioned MINRES; ``x`` is
        updated in place (numpy array or device tensor).  ``phase_fix``
        keeps every update orthogonal to the gauge direction i*psi (the
        reference's bordered system).  Returns stats."""
        o = self._options(tol, max_newton, forcing, max_krylov, precision, verbose, refine, phase_fix)
        st = NewtonStats()
        rc = _lib.nosh_newton_solve(self._h, _ptr(x), _ptr(self._pvec(params)), C.byref(o), C.byref(st))
        _check(rc, allow=(ERR_NOT_CONVERGED,))
        return self._stats(st)


# ---------------------------------------------------------------------------
class continuation:
    """Device-resident continuation run (LOCA stepper semantics): natural
    steps in mu (``advance``) and pseudo-arclength steps
    (``advance_arclength``); the last converged states stay on the GPU
    between steps."""

    def __init__(self, model: nls, x0, mu0: float):
        self.model = model
        h = C.c_void_p()
        _check(_lib.nosh_continuation_create(model._h, _ptr(_f64(x0)), mu0, C.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            _lib.nosh_continuation_destroy(h)
            self._h = None

    def advance(self, mu_new, predictor=PREDICT_SECANT, tol=1e-10, max_newton=20, forcing=0.0, max_krylov=1000,
                precision=None, verbose=0, refine=0.0):
        """One step to ``mu_new``; ``refine`` (<= tol) is the residual the
        Newton steps aim at, so that the stored states serve high-order
        predictors."""
        o = self.model._options(tol, max_newton, forcing, max_krylov, precision, verbose, refine)
        st = NewtonStats()
        rc = _lib.nosh_continuation_advance(self._h, mu_new, predictor, C.byref(o), C.byref(st))
        _check(rc, allow=(ERR_NOT_CONVERGED,))
        return nls._stats(st)

    def advance_arclength(self, ds, predictor=PREDICT_TANGENT, theta=1.0, tol=1e-10, max_newton=20, forcing=0.0,
                          max_krylov=1000, precision=None, verbose=0):
        """One pseudo-arclength step of length ``ds`` (norm
        ``x.x/(2N) + theta^2 mu^2``) with the TANGENT or SECANT predictor and
        a bordered Newton corrector (FP64 solves at relative tolerance
        ``forcing``, 1e-8 when 0).  A failed step (no convergence, NaN or a
        Krylov breakdown) leaves the current state unchanged and reports its
        status; the new mu is ``stats["mu"]``."""
        o = self.model._options(tol, max_newton, forcing, max_krylov, precision, verbose)
        st = NewtonStats()
        rc = _lib.nosh_continuation_advance_arclength(self._h, ds, predictor, theta, C.byref(o), C.byref(st))
        _check(rc, allow=(ERR_NOT_CONVERGED, ERR_NAN, ERR_BREAKDOWN))
        out = nls._stats(st)
        out["status"] = rc
        out["mu"] = self.mu
        return out

    @property
    def mu(self):
        mu = C.c_double()
        _check(_lib.nosh_continuation_state(self._h, None, C.byref(mu)))
        return mu.value

    def tangent(self):
        """(dmu/ds of the last unit arclength tangent, theta)."""
        t, th = C.c_double(), C.c_double()
        _check(_lib.nosh_continuation_tangent(self._h, C.byref(t), C.byref(th)))
        return t.value, th.value

    def state(self, x=None):
        mu = C.c_double()
        x = np.empty(2 * self.model.n) if x is None else x
        _check(_lib.nosh_continuation_state(self._h, _ptr(x), C.byref(mu)))
        return x, mu.value

    def learning(self, train_steps, iters_per_step=20, learning_rate=1e-3):
        _check(_lib.nosh_continuation_learning(self._h, train_steps, iters_per_step, learning_rate))

    def inference_period(self, period):
        """Re-infer the learned coefficient every ``period``-th learned step
        after training (reused in between)."""
        _check(_lib.nosh_continuation_inference_period(self._h, int(period)))

    def predictor_residuals(self, mu_new):
        """||F|| at mu_new of the secant, quadratic, cubic and learned
        predictions from the current history, without advancing."""
        out = np.empty(4)
        _check(_lib.nosh_continuation_predictor_residuals(self._h, mu_new, _ptr(out)))
        return dict(zip(("secant", "quadratic", "cubic", "learned"), out.tolist()))

    def last_prediction(self):
        u, fl, fs, tl, w = C.c_int(), C.c_double(), C.c_double(), C.c_double(), C.c_double()
        _check(_lib.nosh_continuation_last_prediction(self._h, C.byref(u), C.byref(fl), C.byref(fs), C.byref(tl),
                                                      C.byref(w)))
        return {"used": u.value, "f_learned": fl.value, "f_secant": fs.value, "train_loss": tl.value,
                "coef": w.value}


class mpnn:
    """The learned predictor's message-passing network (inspection and
    gradient checks); flat FP32 parameter layout as in nosh_gb300.h."""

    def __init__(self, model: nls):
        self.model = model
        h = C.c_void_p()
        _check(_lib.nosh_mpnn_create(model._h, C.byref(h)))
        self._h = h
        n = C.c_int64()
        _check(_lib.nosh_mpnn_num_params(h, C.byref(n)))
        self.num_params = n.value

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            _lib.nosh_mpnn_destroy(h)
            self._h = None

    def params(self, new=None):
        out = np.empty(self.num_params, np.float32)
        _check(_lib.nosh_mpnn_params(self._h, _ptr(out), None))
        if new is not None:
            new = np.ascontiguousarray(new, np.float32)
            _check(_lib.nosh_mpnn_params(self._h, None, _ptr(new)))
        return out

    def edge_features(self):
        out = np.empty((2 * self.model.mesh.num_edges, 4), np.float32)
        _check(_lib.nosh_mpnn_edge_features(self._h, _ptr(out)))
        return out

    def forward(self, X):
        """The readout coefficient w for node features X (N x 10)."""
        X = np.ascontiguousarray(X, np.float32)
        w = C.c_double()
        _check(_lib.nosh_mpnn_forward(self._h, _ptr(X), C.byref(w)))
        return w.value

    def loss_grad(self, X, gram):
        """Training loss and parameter gradient for node features X and the
        Gram scalars [cc, cd, dd] of the two error fields (online
        training uses those of Jc and Jd)."""
        X = np.ascontiguousarray(X, np.float32)
        gram = np.ascontiguousarray(gram, np.float64)
        g = np.empty(self.num_params, np.float32)
        loss = C.c_double()
        _check(_lib.nosh_mpnn_loss_grad(self._h, _ptr(X), _ptr(gram), C.byref(loss), _ptr(g)))
        return loss.value, g
