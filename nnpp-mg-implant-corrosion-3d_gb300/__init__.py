"""Python host binding of the GB300 NNPP library (libnnpp_gb300.so, C ABI in
include/nnpp_gb300.h).

The names mirror the reference's interface for the hot path:
  build_clouds_hash(...)            grid.h:43-204
  Simulation.residuals(...)         utils::Residuals, fields F1..F4 and F11 (utils.h:29-842)
  Simulation.solve_potential(...)   K11 solve (utils.h:1794-1848, main.cpp:764-779)
  Simulation.forward(...)           the time loop of main.cpp:547-1025 as an explicit step
Every call goes to the CUDA library; there is no CPU fallback.  Loading fails loudly when
the library has not been built.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libnnpp_gb300.so")

NSPECIES = 4
FP64 = 0
MIXED = 1
ORDER_REFERENCE = 0
ORDER_CANONICAL = 1
PRECOND_JACOBI = 0
PRECOND_TWO_LEVEL = 1
CHECK_BOUNDS = 1
CHECK_WAIT_PROBE = 2

STATUS = {0: "NNPP_OK", 1: "NNPP_ERR_INVALID", 2: "NNPP_ERR_CAPACITY", 3: "NNPP_ERR_NONFINITE",
          4: "NNPP_ERR_CG_NO_CONVERGE", 5: "NNPP_ERR_CUDA", 6: "NNPP_ERR_UNSUPPORTED",
          7: "NNPP_ERR_STATE", 8: "NNPP_ERR_NOMEM"}


class NNPPError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (STATUS.get(status, status), msg))
        self.status = status


class Params(C.Structure):
    _fields_ = [("dt", C.c_double), ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
                ("delta", C.c_double), ("CSolid", C.c_double), ("CSat", C.c_double),
                ("F", C.c_double), ("R", C.c_double), ("T", C.c_double), ("vol_red", C.c_double),
                ("z", C.c_double * 4), ("D_solid", C.c_double * 4), ("D_liquid", C.c_double * 4),
                ("s1", C.c_double * 4), ("s2", C.c_double * 4), ("K1", C.c_double * 4),
                ("K2", C.c_double * 4), ("sigma", C.c_double), ("s_phi", C.c_double),
                ("K_phi", C.c_double), ("k_diss", C.c_double), ("switch_width", C.c_double),
                ("c_floor", C.c_double), ("sub_step_no", C.c_int), ("reserved", C.c_int)]

    def copy(self):
        p = Params()
        C.memmove(C.byref(p), C.byref(self), C.sizeof(Params))
        return p


class Diag(C.Structure):
    _fields_ = [("steps_done", C.c_int64), ("solid_count", C.c_int64), ("voln1rel", C.c_double),
                ("vol0rel", C.c_double), ("mass", C.c_double * 4), ("mg_mass_lost", C.c_double),
                ("dissolved_total", C.c_double), ("cg_iterations_total", C.c_int64),
                ("cg_solves", C.c_int64), ("cg_not_converged", C.c_int64),
                ("last_rel_residual", C.c_double), ("outer_iterations_total", C.c_int64)]

    def as_dict(self):
        d = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            d[name] = list(v) if name == "mass" else v
        return d


_lib = None

# exported symbols and their signatures (restype, argtypes)
_P = C.c_void_p
_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int)
_SIGS = {
    "nnpp_last_error": (C.c_char_p, []),
    "nnpp_abi_version": (C.c_int, []),
    "nnpp_device_count": (C.c_int, []),
    "nnpp_set_device": (C.c_int, [C.c_int]),
    "nnpp_params_from_reference": (C.c_int, [_DP, _DP, _DP, _DP, _DP, _DP, C.c_double, C.c_double,
                                             C.POINTER(Params)]),
    "nnpp_build_clouds_hash": (C.c_int, [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                         C.c_int, _DP, C.c_int, _IP, _IP, _IP]),
    "nnpp_build_clouds_hash_noalloc": (C.c_int, [C.c_int, C.c_double, C.c_double, C.c_double,
                                                 C.c_double, C.c_int, C.c_void_p, C.c_void_p,
                                                 C.c_void_p, _IP, C.c_void_p]),
    "nnpp_implant_mask": (C.c_int, [C.c_int, _DP, C.c_int, _DP, C.c_double, C.c_int, _IP, _IP]),
    "nnpp_create": (C.c_int, [C.POINTER(_P), C.POINTER(Params), C.c_int, _DP, _IP, _DP, _DP, _IP]),
    "nnpp_destroy": (C.c_int, [_P]),
    "nnpp_build_neighbours": (C.c_int, [_P, C.c_int, C.c_double, C.c_double, C.c_double,
                                        C.c_double, C.c_int, _IP, _IP, _IP]),
    "nnpp_get_neighbours_csr": (C.c_int, [_P, _IP, _IP, C.POINTER(C.c_int64)]),
    "nnpp_forward": (C.c_int, [_P, C.c_int, C.c_int]),
    "nnpp_set_solver": (C.c_int, [_P, C.c_double, C.c_int, C.c_int]),
    "nnpp_get_state": (C.c_int, [_P, _DP, _DP, _IP]),
    "nnpp_set_state": (C.c_int, [_P, _DP, _DP, _IP]),
    "nnpp_get_diagnostics": (C.c_int, [_P, C.POINTER(Diag)]),
    "nnpp_get_flip_steps": (C.c_int, [_P, _IP]),
    "nnpp_step_host": (C.c_int, [_P, C.c_int, _DP, _IP, _DP, _DP, _IP]),
    "nnpp_residuals": (C.c_int, [_P, C.c_int, _DP, _DP, _IP, C.c_double, _DP]),
    "nnpp_solve_potential": (C.c_int, [_P, C.c_int, _DP, _IP, _DP, _IP, _DP]),
    "nnpp_forward_timed": (C.c_int, [_P, C.c_int, C.c_int, _DP]),
    "nnpp_time_kernel": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, _DP]),
    "nnpp_get_tuning": (C.c_int, [_P, _IP, _IP, _IP]),
    "nnpp_set_tuning": (C.c_int, [_P, C.c_int, C.c_int, C.c_int]),
    "nnpp_chem_create": (C.c_int, [C.POINTER(_P), C.c_int, _DP, _IP, C.c_int, _IP, _IP, _DP, _DP, _DP, _DP]),
    "nnpp_chem_set_state": (C.c_int, [_P, _DP, _IP, C.c_double, C.c_double]),
    "nnpp_chem_step": (C.c_int, [_P, C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "nnpp_chem_get_state": (C.c_int, [_P, _DP, _IP, C.POINTER(C.c_double)]),
    "nnpp_chem_destroy": (None, [_P]),
    "nnpp_set_transport_variant": (C.c_int, [_P, C.c_int]),
    "nnpp_set_params": (C.c_int, [_P, C.POINTER(Params)]),
    "nnpp_reset": (C.c_int, [_P]),
    "nnpp_set_warm_start": (C.c_int, [_P, C.c_int]),
    "nnpp_set_preconditioner": (C.c_int, [_P, C.c_int, C.c_int]),
    "nnpp_get_preconditioner": (C.c_int, [_P, _IP, _IP, _IP, C.POINTER(C.c_int64)]),
    "nnpp_forward_ckpt": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, C.c_int, _DP]),
    "nnpp_backward": (C.c_int, [_P, _DP, _DP, _DP]),
    "nnpp_set_adjoint_store": (C.c_int, [_P, C.c_int]),
    "nnpp_set_refinement": (C.c_int, [_P, C.c_double, C.c_int]),
    "nnpp_residuals_full": (C.c_int, [C.c_int, _DP, _IP, C.c_int, _IP, _DP, _DP, _IP, C.c_double,
                                      _DP, _DP, _DP, _DP]),
    "nnpp_residuals_full_device": (C.c_int, [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                             C.c_void_p, C.c_void_p, C.c_double, _DP, _DP, _DP,
                                             C.c_void_p, C.c_void_p]),
    "nnpp_set_adjoint_solver": (C.c_int, [_P, C.c_double]),
    "nnpp_get_adjoint_stats": (C.c_int, [_P, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                         C.POINTER(C.c_int64), _IP]),
    "nnpp_set_checks": (C.c_int, [_P, C.c_int]),
    "nnpp_forward_implicit": (C.c_int, [_P, C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "nnpp_get_coarse_stats": (C.c_int, [_P, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                        C.POINTER(C.c_int64), _DP, _IP]),
    "nnpp_ensemble_create": (C.c_int, [C.POINTER(_P), C.POINTER(_P), C.c_int]),
    "nnpp_ensemble_forward": (C.c_int, [_P, C.c_int, C.c_int]),
    "nnpp_ensemble_forward_timed": (C.c_int, [_P, C.c_int, C.c_int, _DP]),
    "nnpp_ensemble_tuning": (C.c_int, [_P, _IP, _IP]),
    "nnpp_ensemble_destroy": (C.c_int, [_P]),
    "nnpp_synth_count": (C.c_int64, [C.c_int, C.c_int]),
    "nnpp_synth_fill": (C.c_int, [C.c_int, C.c_int, C.c_uint64, _DP, _IP, _DP, _DP, _IP,
                                  C.POINTER(Params)]),
}


def lib():
    """The loaded library; raises if it has not been built (no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libnnpp_gb300.so not built: run __graft_entry__.build() "
                              "(or python build.py in the package directory)")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def exported_symbols():
    return list(_SIGS)


def _check(st):
    if st != 0:
        raise NNPPError(st, lib().nnpp_last_error().decode())


def _dp(a):
    return a.ctypes.data_as(_DP) if a is not None else None


def _ip(a):
    return a.ctypes.data_as(_IP) if a is not None else None


def device_count():
    return lib().nnpp_device_count()


def set_device(device):
    _check(lib().nnpp_set_device(device))


# ------------------------------------------------------------------ inputs -------------
def synth(kind, n_side, seed=0):
    """Deterministic synthetic workload in the reference's input layout (see
    nnpp_synth_fill): nodes (3, N) rows x/y/z, bctypes (N,), bcvalues (S+1, N),
    icvalues (S+1, N), phase0 (N,), params."""
    L = lib()
    N = L.nnpp_synth_count(kind, n_side)
    if N <= 0:
        raise ValueError("bad synthetic kind/n_side")
    nodes = np.empty((3, N), dtype=np.float64)
    bct = np.empty(N, dtype=np.int32)
    bcv = np.empty((NSPECIES + 1, N), dtype=np.float64)
    icv = np.empty((NSPECIES + 1, N), dtype=np.float64)
    ph = np.empty(N, dtype=np.int32)
    p = Params()
    _check(L.nnpp_synth_fill(kind, n_side, seed, _dp(nodes), _ip(bct), _dp(bcv), _dp(icv),
                             _ip(ph), C.byref(p)))
    return dict(nodes=nodes, bctypes=bct, bcvalues=bcv, icvalues=icv, phase0=ph, params=p, N=N)


def params_from_reference(data2, datac, datac11, k_diss=0.0, switch_width=0.0):
    """utils::parameter::set_double (utils.h:2343-2484) for the hot path's fields."""
    d2 = np.ascontiguousarray(data2, dtype=np.float64)
    dc = [np.ascontiguousarray(d, dtype=np.float64) for d in datac]
    d11 = np.ascontiguousarray(datac11, dtype=np.float64)
    p = Params()
    _check(lib().nnpp_params_from_reference(_dp(d2), _dp(dc[0]), _dp(dc[1]), _dp(dc[2]),
                                            _dp(dc[3]), _dp(d11), k_diss, switch_width,
                                            C.byref(p)))
    return p


# ------------------------------------------------------------- ten-species residual -----
def residuals_full(nodes, clouds, cloud_lengths, U_n1, U_n, phase, voln1rel, data2, datac, datac11):
    """nnpp_residuals_full: the reference's complete residual utils::Residuals (ten species,
    their reactions, the potential).  nodes (3, N) or (N, 3); clouds (N, M) as
    build_clouds_hash returns them (self in column 0); U_n1, U_n (11, N); phase (N,);
    data2 (51,), datac (10, 7), datac11 (4,) the reference's control vectors.  Returns F
    (11, N)."""
    xyz = _colmajor_nodes(nodes)
    N = xyz.shape[1]
    cl = np.ascontiguousarray(np.asarray(clouds, dtype=np.int32).T)  # (M, N): column-major N x M
    M = cl.shape[0]
    lens = np.ascontiguousarray(cloud_lengths, dtype=np.int32)
    u1 = np.ascontiguousarray(U_n1, dtype=np.float64)
    u0 = np.ascontiguousarray(U_n, dtype=np.float64)
    ph = np.ascontiguousarray(phase, dtype=np.int32)
    if u1.shape != (11, N) or u0.shape != (11, N) or ph.shape != (N,) or lens.shape != (N,):
        raise ValueError("residuals_full: U_n1, U_n (11, N), phase and cloud_lengths (N,)")
    d2 = np.ascontiguousarray(data2, dtype=np.float64)
    dc = np.ascontiguousarray(datac, dtype=np.float64)
    d11 = np.ascontiguousarray(datac11, dtype=np.float64)
    if d2.size != 51 or dc.size != 70 or d11.size != 4:
        raise ValueError("residuals_full: data2 (51), datac (10, 7), datac11 (4)")
    F = np.zeros((11, N))
    _check(lib().nnpp_residuals_full(N, _dp(xyz), _ip(cl), M, _ip(lens), _dp(u1), _dp(u0), _ip(ph),
                                     float(voln1rel), _dp(d2), _dp(dc), _dp(d11), _dp(F)))
    return F


class ChemImplicit:
    """The reference's implicit time step with its complete model (ten species and the
    potential) on the GPU: nnpp_chem_create / set_state / step / get_state.  nodes (3, N) or
    (N, 3); clouds (N, M) as build_clouds_hash returns them; bcvalues (11, N); data2, datac
    (10, 7), datac11 as the reference's data files hold them."""

    def __init__(self, nodes, clouds, cloud_lengths, bctypes, bcvalues, data2, datac, datac11):
        xyz = _colmajor_nodes(nodes)
        self.N = N = xyz.shape[1]
        cl = np.ascontiguousarray(np.asarray(clouds, dtype=np.int32).T)
        lens = np.ascontiguousarray(cloud_lengths, dtype=np.int32)
        bt = np.ascontiguousarray(bctypes, dtype=np.int32)
        bv = np.ascontiguousarray(bcvalues, dtype=np.float64)
        d2 = np.ascontiguousarray(data2, dtype=np.float64)
        dc = np.ascontiguousarray(datac, dtype=np.float64)
        d11 = np.ascontiguousarray(datac11, dtype=np.float64)
        if bv.shape != (11, N) or bt.shape != (N,) or lens.shape != (N,) or cl.shape[1] != N:
            raise ValueError("ChemImplicit: clouds (N, M), cloud_lengths and bctypes (N,), bcvalues (11, N)")
        if d2.size != 51 or dc.size != 70 or d11.size != 4:
            raise ValueError("ChemImplicit: data2 (51), datac (10, 7), datac11 (4)")
        h = _P()
        _check(lib().nnpp_chem_create(C.byref(h), N, _dp(xyz), _ip(cl), cl.shape[0], _ip(lens), _ip(bt), _dp(bv),
                                      _dp(d2), _dp(dc), _dp(d11)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().nnpp_chem_destroy(h)
            self._h = None

    def set_state(self, U, phase, voln1rel=0.0, vol0rel=0.0):
        U = np.ascontiguousarray(U, dtype=np.float64)
        ph = np.ascontiguousarray(phase, dtype=np.int32)
        if U.shape != (11, self.N) or ph.shape != (self.N,):
            raise ValueError("ChemImplicit.set_state: U (11, N), phase (N,)")
        _check(lib().nnpp_chem_set_state(self._h, _dp(U), _ip(ph), float(voln1rel), float(vol0rel)))

    def step(self, n_steps=1):
        """n implicit steps; returns (Newton iterations, GMRES iterations)."""
        nw, kr = C.c_int64(0), C.c_int64(0)
        _check(lib().nnpp_chem_step(self._h, int(n_steps), C.byref(nw), C.byref(kr)))
        return nw.value, kr.value

    def state(self):
        U = np.empty((11, self.N))
        ph = np.empty(self.N, dtype=np.int32)
        v = C.c_double(0.0)
        _check(lib().nnpp_chem_get_state(self._h, _dp(U), _ip(ph), C.byref(v)))
        return U, ph, v.value


# ------------------------------------------------------------------ neighbour build -----
def build_clouds_hash(max_node_no, r, dx, dy, dz, nodes, order_mode=ORDER_REFERENCE,
                      want_clouds=True):
    """Mirror of build_clouds_hash (grid.h:43-44).  nodes: (3, N) or (N, 3) float64.
    Returns (clouds (N, max_node_no) int32, -1 padded, self at column 0; cloud_lengths (N,);
    max_cloud_length).  Raises NNPPError(NNPP_ERR_CAPACITY) where the reference throws."""
    xyz = _colmajor_nodes(nodes)
    N = xyz.shape[1]
    clouds = np.empty((max_node_no, N), dtype=np.int32) if want_clouds else None
    lengths = np.empty(N, dtype=np.int32)
    ml = C.c_int(0)
    _check(lib().nnpp_build_clouds_hash(max_node_no, r, dx, dy, dz, N, _dp(xyz), order_mode,
                                        _ip(clouds), _ip(lengths), C.byref(ml)))
    return (clouds.T if want_clouds else None), lengths, ml.value


def build_clouds_hash_noalloc(max_node_no, r, dx, dy, dz, n_nodes, d_nodes, d_clouds,
                              d_lengths, stream=0):
    """nnpp_build_clouds_hash_noalloc: canonical-order build between caller-owned DEVICE
    buffers given as integer addresses (3*N doubles in, N*max_node_no and N ints out).
    Allocates nothing; returns max_cloud_length."""
    ml = C.c_int(0)
    _check(lib().nnpp_build_clouds_hash_noalloc(max_node_no, r, dx, dy, dz, n_nodes, d_nodes,
                                                d_clouds, d_lengths, C.byref(ml), stream))
    return ml.value


def implant_mask(nodes, points, r, max_node_no=1024):
    """The nodes' phase from an implant point cloud (nnpp_implant_mask; main.cpp:316-325,
    422-457 with kd_tree_interface.h:156-252): (counts of points within r, phase = counts >
    0).  nodes, points: (3, N) / (3, M) or (N, 3) / (M, 3) float64."""
    xyz = _colmajor_nodes(nodes)
    pts = _colmajor_nodes(points) if len(points) else np.zeros((3, 0))
    N, M = xyz.shape[1], pts.shape[1]
    counts = np.empty(N, dtype=np.int32)
    phase = np.empty(N, dtype=np.int32)
    _check(lib().nnpp_implant_mask(N, _dp(xyz), M, _dp(np.ascontiguousarray(pts)), r, max_node_no,
                                   _ip(counts), _ip(phase)))
    return counts, phase


def _colmajor_nodes(nodes):
    a = np.asarray(nodes, dtype=np.float64)
    if a.ndim != 2 or 3 not in a.shape:
        raise ValueError("nodes must be (3, N) or (N, 3)")
    if a.shape[0] != 3:
        a = a.T
    return np.ascontiguousarray(a)


# ------------------------------------------------------------------ simulation ----------
class Simulation:
    """One NNPP instance on the GPU (an nnpp_handle)."""

    def __init__(self, params, nodes, bctypes, bcvalues, icvalues, phase0=None):
        self.params = params.copy()
        xyz = _colmajor_nodes(nodes)
        self.N = xyz.shape[1]
        self._xyz = xyz
        bct = np.ascontiguousarray(bctypes, dtype=np.int32)
        bcv = np.ascontiguousarray(bcvalues, dtype=np.float64).reshape(NSPECIES + 1, self.N)
        icv = np.ascontiguousarray(icvalues, dtype=np.float64).reshape(NSPECIES + 1, self.N)
        ph = None if phase0 is None else np.ascontiguousarray(phase0, dtype=np.int32)
        h = C.c_void_p()
        _check(lib().nnpp_create(C.byref(h), C.byref(self.params), self.N, _dp(xyz), _ip(bct),
                                 _dp(bcv), _dp(icv), _ip(ph)))
        self._h = h

    @classmethod
    def from_synth(cls, inp):
        return cls(inp["params"], inp["nodes"], inp["bctypes"], inp["bcvalues"],
                   inp["icvalues"], inp["phase0"])

    def close(self):
        if getattr(self, "_h", None):
            lib().nnpp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def build_neighbours(self, max_node_no=1024, r=None, cell=None,
                         order_mode=ORDER_REFERENCE, want_clouds=False):
        """main.cpp:304-305 convention by default: r = delta (1 + 1e-5), cells of 10 dx."""
        p = self.params
        if r is None:
            r = p.delta * (1.0 + 1e-5)
        if cell is None:
            cell = (p.dx * 10.0, p.dy * 10.0, p.dz * 10.0)
        clouds = np.empty((max_node_no, self.N), dtype=np.int32) if want_clouds else None
        lengths = np.empty(self.N, dtype=np.int32)
        ml = C.c_int(0)
        _check(lib().nnpp_build_neighbours(self._h, max_node_no, r, cell[0], cell[1], cell[2],
                                           order_mode, _ip(clouds), _ip(lengths), C.byref(ml)))
        self.max_cloud_length = ml.value
        return (clouds.T if want_clouds else None), lengths, ml.value

    def neighbours_csr(self):
        nnz = C.c_int64(0)
        _check(lib().nnpp_get_neighbours_csr(self._h, None, None, C.byref(nnz)))
        ptr = np.empty(self.N + 1, dtype=np.int32)
        cols = np.empty(max(nnz.value, 1), dtype=np.int32)
        _check(lib().nnpp_get_neighbours_csr(self._h, _ip(ptr), _ip(cols), C.byref(nnz)))
        return ptr, cols[:nnz.value]

    def set_warm_start(self, history):
        """Initial guess of the potential solves: 0 previous potential, 1-2 linear
        extrapolation, 3-6 energy-norm-optimal combination of that many past potentials."""
        _check(lib().nnpp_set_warm_start(self._h, history))

    def set_preconditioner(self, kind, refresh_every=64):
        """Preconditioner of the potential CG: PRECOND_JACOBI (diagonal) or
        PRECOND_TWO_LEVEL (diagonal + coarse correction on aggregates of hash bins, rebuilt
        every refresh_every steps when the phases changed; 0: only on set_state/reset)."""
        _check(lib().nnpp_set_preconditioner(self._h, kind, refresh_every))

    def preconditioner(self):
        """(kind, coarse unknowns, refresh period, coarse inverses computed so far) of the
        potential CG's preconditioner."""
        k, n, r, b = C.c_int(), C.c_int(), C.c_int(), C.c_int64()
        _check(lib().nnpp_get_preconditioner(self._h, C.byref(k), C.byref(n), C.byref(r), C.byref(b)))
        return k.value, n.value, r.value, b.value

    def set_checks(self, flags):
        """Device-side checks (nnpp_set_checks): CHECK_BOUNDS, CHECK_WAIT_PROBE."""
        _check(lib().nnpp_set_checks(self._h, int(flags)))

    def coarse_stats(self):
        """Coarse-inverse rebuilds: total, warm-started, triggered during runs, the run
        rebuilds' summed milliseconds, Newton-Schulz steps of the last one."""
        a, b, c = C.c_int64(0), C.c_int64(0), C.c_int64(0)
        ms = C.c_double(0.0)
        ns = C.c_int(0)
        _check(lib().nnpp_get_coarse_stats(self._h, C.byref(a), C.byref(b), C.byref(c), C.byref(ms),
                                           C.byref(ns)))
        return {"rebuilds": a.value, "warm_rebuilds": b.value, "run_rebuilds": c.value,
                "run_rebuild_ms": ms.value, "last_ns_steps": ns.value}

    def reset(self):
        """Back to the initial state of build_neighbours (lists and tuning kept)."""
        _check(lib().nnpp_reset(self._h))

    def set_params(self, params):
        """New model parameters with the same geometry (no neighbour rebuild)."""
        p = params.copy()
        _check(lib().nnpp_set_params(self._h, C.byref(p)))
        self.params = p

    def set_solver(self, tol=1e-10, max_iter=2000, strict=False):
        _check(lib().nnpp_set_solver(self._h, tol, max_iter, 1 if strict else 0))

    def set_refinement(self, inner_rel=1e-4, max_outer=30):
        """Mixed path: relative reduction of each FP32 inner CG sweep, sweep cap."""
        _check(lib().nnpp_set_refinement(self._h, float(inner_rel), int(max_outer)))

    def forward(self, n_steps, precision=MIXED):
        _check(lib().nnpp_forward(self._h, n_steps, precision))

    def forward_implicit(self, n_steps):
        """n steps of the reference's backward-Euler Newton/GMRES integration (FP64,
        nnpp_forward_implicit); returns (Newton iterations, GMRES iterations)."""
        nw, kr = C.c_int64(0), C.c_int64(0)
        _check(lib().nnpp_forward_implicit(self._h, n_steps, C.byref(nw), C.byref(kr)))
        return nw.value, kr.value

    def forward_timed(self, n_steps, precision=MIXED):
        """forward() timed with CUDA events on the handle's stream; returns milliseconds."""
        ms = C.c_double(0.0)
        _check(lib().nnpp_forward_timed(self._h, n_steps, precision, C.byref(ms)))
        return ms.value

    def time_kernel(self, kernel_id, precision=MIXED, reps=20):
        """Average milliseconds per launch of one step kernel (0 transport, 1 CG SpMV,
        2 FP64 refinement residual, 3 CG update; with the two-level preconditioner on one
        instance 4, 5, 6 time the update's restriction, coarse product and z pass alone)."""
        ms = C.c_double(0.0)
        _check(lib().nnpp_time_kernel(self._h, kernel_id, precision, reps, C.byref(ms)))
        return ms.value

    def forward_ckpt(self, n_steps, precision=MIXED, ckpt_every=50, sample_every=20):
        """Forward half of the adjoint pair: returns the cumulative Mg mass-loss curve
        sampled every `sample_every` steps (checkpoints every `ckpt_every` steps)."""
        curve = np.empty(n_steps // sample_every, dtype=np.float64)
        _check(lib().nnpp_forward_ckpt(self._h, n_steps, precision, ckpt_every, sample_every,
                                       _dp(curve)))
        self._fwd_steps = int(n_steps)
        return curve

    def set_adjoint_store(self, mode):
        """Storage of the recorded forward run: 0 automatic, 1 checkpoints and every step's
        solved potential (backward recomputes the segments' bond sums only), 2 every step's
        snapshot, 3 checkpoints only (backward recomputes whole steps)."""
        _check(lib().nnpp_set_adjoint_store(self._h, mode))

    def set_adjoint_solver(self, tol):
        """Relative tolerance of the adjoint potential solves (0, the default: max(tol, 1e-8)
        for mixed runs, tol for FP64 runs, tol being the forward's)."""
        _check(lib().nnpp_set_adjoint_solver(self._h, float(tol)))

    def adjoint_stats(self, per_step=False):
        """{"cg_iterations", "solves", "sweeps"} of the last backward's adjoint potential
        solves, plus "per_step" (each step's inner iterations, int32) if per_step."""
        it, n, sw = C.c_int64(0), C.c_int64(0), C.c_int64(0)
        log = np.zeros(getattr(self, "_fwd_steps", 0) if per_step else 0, dtype=np.int32)
        _check(lib().nnpp_get_adjoint_stats(self._h, C.byref(it), C.byref(n), C.byref(sw),
                                            _ip(log) if per_step else None))
        out = {"cg_iterations": it.value, "solves": n.value, "sweeps": sw.value}
        if per_step:
            out["per_step"] = log
        return out

    def backward(self, dL_dcurve):
        """Backward half: dL/dD_liquid (4,) and dL/dk_diss for dL/d(curve)."""
        g = np.ascontiguousarray(dL_dcurve, dtype=np.float64)
        gD = np.zeros(NSPECIES)
        gk = C.c_double(0.0)
        _check(lib().nnpp_backward(self._h, _dp(g), _dp(gD), C.byref(gk)))
        return gD, gk.value

    def tuning(self):
        """(bins per tile, lanes per node, CG operator variant) of the autotuned engine."""
        t, w, g = C.c_int(0), C.c_int(0), C.c_int(0)
        _check(lib().nnpp_get_tuning(self._h, C.byref(t), C.byref(w), C.byref(g)))
        return t.value, w.value, g.value

    def set_tuning(self, bins_per_tile, lanes_per_node, cg_operator):
        """Pin the execution configuration instead of autotuning it (cg_operator: 0 L1/L2
        gathers, 1 bulk-copy staged, 2 shared-memory windows)."""
        _check(lib().nnpp_set_tuning(self._h, bins_per_tile, lanes_per_node, int(cg_operator)))

    def set_transport_variant(self, variant):
        """FP32 transport: 0 neighbour records gathered from L1/L2 (the default), 1 tile
        halos staged in shared memory; the same sums in the same order."""
        _check(lib().nnpp_set_transport_variant(self._h, int(variant)))

    def state(self):
        c = np.empty((NSPECIES, self.N), dtype=np.float64)
        phi = np.empty(self.N, dtype=np.float64)
        ph = np.empty(self.N, dtype=np.int32)
        _check(lib().nnpp_get_state(self._h, _dp(c), _dp(phi), _ip(ph)))
        return c, phi, ph

    def set_state(self, c, phi=None, phase=None):
        c = np.ascontiguousarray(c, dtype=np.float64).reshape(NSPECIES, self.N)
        phi = None if phi is None else np.ascontiguousarray(phi, dtype=np.float64)
        phase = None if phase is None else np.ascontiguousarray(phase, dtype=np.int32)
        _check(lib().nnpp_set_state(self._h, _dp(c), _dp(phi), _ip(phase)))

    def diagnostics(self):
        d = Diag()
        _check(lib().nnpp_get_diagnostics(self._h, C.byref(d)))
        return d.as_dict()

    def flip_steps(self):
        f = np.empty(self.N, dtype=np.int32)
        _check(lib().nnpp_get_flip_steps(self._h, _ip(f)))
        return f

    def step_host(self, c_in, phase_in=None, precision=MIXED, out=None):
        """One step with host buffers in and out (nnpp_step_host)."""
        c_in = np.ascontiguousarray(c_in, dtype=np.float64).reshape(NSPECIES, self.N)
        if out is None:
            out = (np.empty((NSPECIES, self.N)), np.empty(self.N), np.empty(self.N, dtype=np.int32))
        phase_in = None if phase_in is None else np.ascontiguousarray(phase_in, dtype=np.int32)
        _check(lib().nnpp_step_host(self._h, precision, _dp(c_in), _ip(phase_in), _dp(out[0]),
                                    _dp(out[1]), _ip(out[2])))
        return out

    def residuals(self, c, phi, phase, voln1rel=0.0, precision=FP64):
        """utils::Residuals F1..F4 and F11 with U^{n+1} = U^n; returns (S+1, N)."""
        c = np.ascontiguousarray(c, dtype=np.float64).reshape(NSPECIES, self.N)
        phi = np.ascontiguousarray(phi, dtype=np.float64)
        phase = np.ascontiguousarray(phase, dtype=np.int32)
        F = np.empty((NSPECIES + 1, self.N), dtype=np.float64)
        _check(lib().nnpp_residuals(self._h, precision, _dp(c), _dp(phi), _ip(phase), voln1rel,
                                    _dp(F)))
        return F

    def solve_potential(self, c, phase, phi0=None, precision=MIXED):
        c = np.ascontiguousarray(c, dtype=np.float64).reshape(NSPECIES, self.N)
        phase = np.ascontiguousarray(phase, dtype=np.int32)
        phi = np.zeros(self.N) if phi0 is None else np.array(phi0, dtype=np.float64)
        it = C.c_int(0)
        rel = C.c_double(0.0)
        _check(lib().nnpp_solve_potential(self._h, precision, _dp(c), _ip(phase), _dp(phi),
                                          C.byref(it), C.byref(rel)))
        return phi, it.value, rel.value


class Ensemble:
    """Many Simulations stepped together in batched launches (nnpp_ensemble_*)."""

    def __init__(self, sims):
        self.sims = list(sims)
        arr = (C.c_void_p * len(self.sims))(*[s.handle for s in self.sims])
        e = C.c_void_p()
        _check(lib().nnpp_ensemble_create(C.byref(e), arr, len(self.sims)))
        self._e = e

    def forward(self, n_steps, precision=MIXED):
        _check(lib().nnpp_ensemble_forward(self._e, n_steps, precision))

    def forward_timed(self, n_steps, precision=MIXED):
        ms = C.c_double(0.0)
        _check(lib().nnpp_ensemble_forward_timed(self._e, n_steps, precision, C.byref(ms)))
        return ms.value

    def tuning(self):
        t, w = C.c_int(0), C.c_int(0)
        _check(lib().nnpp_ensemble_tuning(self._e, C.byref(t), C.byref(w)))
        return t.value, w.value

    def close(self):
        if getattr(self, "_e", None):
            lib().nnpp_ensemble_destroy(self._e)
            self._e = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------------ result errors ---------
def compare_states(params, c, phi, phase, c_ref, phi_ref, phase_ref, mg_lost=None,
                   mg_lost_ref=None):
    """The error of a run against a reference run of the same workload, in the four
    quantities every result states: relative L2 of the concentrations and of the potential,
    the front position in lattice spacings and the Mg mass lost.

    The front position is the radius of the sphere of the solid volume,
    (3 V_solid / 4 pi)^(1/3) with V_solid = solid nodes x dV (the solid/liquid mask of
    main.cpp:914-922); front_dx is the difference of the two radii in units of dx.
    mask_mismatch counts the nodes whose phase differs."""
    dV = params.dx * params.dy * params.dz

    def r_eq(ph):
        return (3.0 * float(np.sum(ph)) * dV / (4.0 * np.pi)) ** (1.0 / 3.0)

    def rel(a, b):
        return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) /
                     max(float(np.linalg.norm(b)), 1e-300))

    out = {"rel_l2_c": rel(c, c_ref), "rel_l2_phi": rel(phi, phi_ref),
           "mask_mismatch": int(np.sum(np.asarray(phase) != np.asarray(phase_ref))),
           "front_dx": abs(r_eq(phase) - r_eq(phase_ref)) / params.dx,
           "front_radius_dx": r_eq(phase_ref) / params.dx,
           "solid_nodes": int(np.sum(phase_ref))}
    if mg_lost is not None and mg_lost_ref is not None:
        out["mg_mass_lost"] = float(mg_lost_ref)
        out["mg_mass_lost_rel"] = abs(mg_lost - mg_lost_ref) / max(abs(mg_lost_ref), 1e-300)
    return out
