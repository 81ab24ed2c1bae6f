"""ctypes binding of the oracle (TEST INFRASTRUCTURE ONLY).

liboracle.so is the FP64 CPU restatement of the reference's hot path (nnpp_oracle.cpp);
_ref/libnnpp_ref.so wraps the reference's own grid.h/utils.h (built only where the
reference's sources are present).  Only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg use this module, as the checker.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
NSPECIES = 4

_orc = None
_ref = None
_DP = C.POINTER(C.c_double)
_IP = C.POINTER(C.c_int)
_LP = C.POINTER(C.c_int64)
_P = C.c_void_p


def _dp(a):
    return a.ctypes.data_as(_DP) if a is not None else None


def _ip(a):
    return a.ctypes.data_as(_IP) if a is not None else None


def _lp(a):
    return a.ctypes.data_as(_LP) if a is not None else None


def load_oracle():
    """liboracle.so, or liboracle_native.so (the same sources for the host's instruction set,
    the same bits) when NNPP_ORACLE_NATIVE=1 was set before the first call."""
    global _orc
    if _orc is None:
        from build_oracle import build_oracle  # noqa: E402 (same directory)
        path = None
        if os.environ.get("NNPP_ORACLE_NATIVE") == "1":
            path = build_oracle(native=True)
        if path is None:
            path = build_oracle()
        L = C.CDLL(path)
        sig = {
            "orc_create": (_P, [_P, C.c_int, _DP, _IP, _DP, _DP, _IP]),
            "orc_destroy": (None, [_P]),
            "orc_set_solver": (None, [_P, C.c_double, C.c_int]),
            "orc_set_threads": (C.c_int, [C.c_int]),
            "orc_build_neighbours": (C.c_int, [_P, C.c_int, C.c_double, C.c_double, C.c_double,
                                               C.c_double, _IP]),
            "orc_nnz": (C.c_int64, [_P]),
            "orc_get_clouds": (C.c_int, [_P, _IP, _LP, _IP]),
            "orc_set_clouds": (C.c_int, [_P, _LP, _IP]),
            "orc_residuals": (C.c_int, [_P, _DP, _DP, _IP, C.c_double, _DP]),
            "orc_residuals_full": (C.c_int, [C.c_int, _DP, _LP, _IP, _DP, _DP, _IP, C.c_double, _DP,
                                             _DP, _DP, _DP]),
            "orc_poisson_matrix": (C.c_int, [_P, _IP, _DP, _DP, C.POINTER(C.c_ubyte)]),
            "orc_solve_potential": (C.c_int, [_P, _DP, _IP, _DP, _IP, _DP]),
            "orc_forward": (C.c_int, [_P, C.c_int]),
            "orc_get_state": (C.c_int, [_P, _DP, _DP, _IP, _IP]),
            "orc_set_state": (C.c_int, [_P, _DP, _DP, _IP]),
            "orc_get_diag": (C.c_int, [_P, _DP]),
            "orc_implant_counts": (C.c_int, [C.c_int, _DP, C.c_int, _DP, C.c_double, _IP]),
            "orc_implicit_forward": (C.c_int, [_P, C.c_int, _LP, _LP]),
            "orc_residuals_implicit": (C.c_int, [_P, _DP, _DP, _DP, _DP, _IP, C.c_double, _DP]),
            "orc_chem_implicit_step": (C.c_int, [_P, _DP, _IP, _IP, _DP, C.c_double, _DP, _DP, _DP, _LP]),
            "orc_chem_tangent": (C.c_int, [_P, C.c_int, _DP, _IP, _IP, _DP, C.c_double, _DP, _DP, _DP, _DP,
                                           _DP]),
            "orc_tangent": (C.c_int, [_P, C.c_int, _DP, _DP]),
            "orc_tangent_gmres": (C.c_int, [_P, C.c_int, _DP, _DP, C.c_double, C.c_int, C.c_int]),
            "nnpp_synth_count": (C.c_int64, [C.c_int, C.c_int]),
            "nnpp_synth_fill": (C.c_int, [C.c_int, C.c_int, C.c_uint64, _DP, _IP, _DP, _DP, _IP,
                                          C.c_void_p]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _orc = L
    return _orc


def load_reference():
    """The reference's own code, or None where its sources are absent."""
    global _ref
    if _ref is None:
        from build_oracle import build_reference_shim
        path = build_reference_shim()
        if path is None:
            return None
        L = C.CDLL(path)
        L.ref_build_clouds_hash.restype = C.c_int
        L.ref_build_clouds_hash.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double,
                                            C.c_double, C.c_int, _DP, _IP, _LP]
        L.ref_get_clouds.argtypes = [_IP, _LP, _IP]
        L.ref_residuals.argtypes = [C.c_int, _DP, _LP, _IP, _DP, _IP, _IP, _DP, C.c_double,
                                    _DP, _DP, _DP, _DP]
        L.ref_newton_k11.argtypes = [C.c_int, _DP, _LP, _IP, _DP, _IP, _IP, _DP, C.c_double,
                                     _DP, _DP, _DP, _LP, _IP, _IP, _DP]
        for name in ("ref_newton_k", "ref_gmres"):
            getattr(L, name).restype = C.c_int
        L.ref_newton_k.argtypes = [C.c_int, C.c_int, _DP, _LP, _IP, _DP, _IP, _IP, _DP, C.c_double,
                                   _DP, _DP, _DP, _LP, _IP, _IP, _DP]
        L.ref_gmres.argtypes = [C.c_int, C.c_int, _DP, _LP, _IP, _DP, _IP, _IP, _DP, C.c_double,
                                _DP, _DP, _DP, _DP, _DP]
        L.ref_residuals2.argtypes = [C.c_int, _DP, _LP, _IP, _DP, _DP, _IP, _IP, _DP, C.c_double,
                                     _DP, _DP, _DP, _DP]
        L.ref_implant_counts.restype = C.c_int
        L.ref_implant_counts.argtypes = [C.c_int, _DP, C.c_int, _DP, C.c_double, C.c_int, _IP]
        _ref = L
    return _ref


class Params(C.Structure):
    """nnpp_params of include/nnpp_gb300.h (the oracle takes the product's parameter block)."""
    _fields_ = [("dt", C.c_double), ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
                ("delta", C.c_double), ("CSolid", C.c_double), ("CSat", C.c_double),
                ("F", C.c_double), ("R", C.c_double), ("T", C.c_double), ("vol_red", C.c_double),
                ("z", C.c_double * 4), ("D_solid", C.c_double * 4), ("D_liquid", C.c_double * 4),
                ("s1", C.c_double * 4), ("s2", C.c_double * 4), ("K1", C.c_double * 4),
                ("K2", C.c_double * 4), ("sigma", C.c_double), ("s_phi", C.c_double),
                ("K_phi", C.c_double), ("k_diss", C.c_double), ("switch_width", C.c_double),
                ("c_floor", C.c_double), ("sub_step_no", C.c_int), ("reserved", C.c_int)]

    def copy(self):
        q = Params()
        C.memmove(C.byref(q), C.byref(self), C.sizeof(Params))
        return q


def synth(kind, n_side, seed=0):
    """The seeded workloads of nnpp_synth_fill, generated by the oracle library's copy of the
    generator (the same source file), without the product library."""
    L = load_oracle()
    N = L.nnpp_synth_count(kind, n_side)
    if N <= 0:
        raise ValueError("bad synthetic kind/n_side")
    nodes = np.empty((3, N), dtype=np.float64)
    bct = np.empty(N, dtype=np.int32)
    bcv = np.empty((NSPECIES + 1, N), dtype=np.float64)
    icv = np.empty((NSPECIES + 1, N), dtype=np.float64)
    ph = np.empty(N, dtype=np.int32)
    p = Params()
    if L.nnpp_synth_fill(kind, n_side, seed, _dp(nodes), _ip(bct), _dp(bcv), _dp(icv), _ip(ph),
                         C.cast(C.byref(p), C.c_void_p)) != 0:
        raise RuntimeError("synthetic workload generation failed")
    return dict(nodes=nodes, bctypes=bct, bcvalues=bcv, icvalues=icv, phase0=ph, params=p, N=N)


def implant_counts(nodes, points, r):
    """Implant points within r of every node (the oracle's restatement of the reference's
    kd-tree query, kd_tree_interface.h:156-252); nodes (3, N), points (3, M)."""
    nodes = np.ascontiguousarray(nodes, dtype=np.float64)
    points = np.ascontiguousarray(points, dtype=np.float64)
    counts = np.empty(nodes.shape[1], dtype=np.int32)
    load_oracle().orc_implant_counts(nodes.shape[1], _dp(nodes), points.shape[1], _dp(points), r,
                                     _ip(counts))
    return counts


def synth_implant_points(n_side, seed, shape="sphere"):
    """A seeded implant point cloud (the reference's implant meshes are not available): the
    points of a jittered lattice of spacing 0.4 / n_side (0.4 of the node spacing of an
    n_side^3 node lattice on the unit cube) that fall inside a sphere of radius 0.3 at the
    centre ("sphere") or inside the sphere's shell of thickness 0.05 ("shell"), from numpy's
    PCG64 (the same points on every machine)."""
    rng = np.random.default_rng(seed)
    h = 0.4 / n_side
    m = int(round(1.0 / h))
    g = (np.arange(m) + 0.5) * h
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    P = np.stack([X.ravel(), Y.ravel(), Z.ravel()]) + rng.uniform(-0.25 * h, 0.25 * h, (3, m ** 3))
    rr = np.sqrt(((P - 0.5) ** 2).sum(axis=0))
    keep = rr <= 0.3 if shape == "sphere" else (rr <= 0.3) & (rr >= 0.25)
    return np.ascontiguousarray(P[:, keep])


DIAG_KEYS = ["steps", "solid_count", "voln1rel", "vol0rel", "mass0", "mass1", "mass2", "mass3",
             "mg_mass_lost", "dissolved_total", "cg_iters", "cg_solves", "cg_nc", "last_relres"]


class Oracle:
    """FP64 CPU restatement of the explicit step (nnpp_oracle.cpp)."""

    def __init__(self, params, nodes, bctypes, bcvalues, icvalues, phase0=None):
        L = load_oracle()
        self.params = params
        self.nodes = np.ascontiguousarray(nodes, dtype=np.float64)
        self.N = self.nodes.shape[1]
        self._keep = [np.ascontiguousarray(bctypes, dtype=np.int32),
                      np.ascontiguousarray(bcvalues, dtype=np.float64),
                      np.ascontiguousarray(icvalues, dtype=np.float64),
                      None if phase0 is None else np.ascontiguousarray(phase0, dtype=np.int32)]
        self._h = L.orc_create(C.byref(params), self.N, _dp(self.nodes), _ip(self._keep[0]),
                               _dp(self._keep[1]), _dp(self._keep[2]), _ip(self._keep[3]))

    @classmethod
    def from_synth(cls, inp):
        return cls(inp["params"], inp["nodes"], inp["bctypes"], inp["bcvalues"], inp["icvalues"],
                   inp["phase0"])

    def __del__(self):
        if getattr(self, "_h", None):
            load_oracle().orc_destroy(self._h)
            self._h = None

    def set_solver(self, tol=1e-12, max_iter=20000):
        load_oracle().orc_set_solver(self._h, tol, max_iter)

    def build_neighbours(self, max_node_no=1024, r=None, cell=None):
        p = self.params
        r = p.delta * (1.0 + 1e-5) if r is None else r
        cell = (p.dx * 10.0, p.dy * 10.0, p.dz * 10.0) if cell is None else cell
        ml = C.c_int(0)
        st = load_oracle().orc_build_neighbours(self._h, max_node_no, r, cell[0], cell[1],
                                                cell[2], C.byref(ml))
        if st != 0:
            raise RuntimeError("oracle neighbour build failed with status %d" % st)
        return ml.value

    def clouds(self):
        """(lengths incl. self, row_ptr int64, cols incl. self at slot 0)"""
        L = load_oracle()
        nnz = L.orc_nnz(self._h)
        lengths = np.empty(self.N, dtype=np.int32)
        ptr = np.empty(self.N + 1, dtype=np.int64)
        cols = np.empty(nnz, dtype=np.int32)
        L.orc_get_clouds(self._h, _ip(lengths), _lp(ptr), _ip(cols))
        return lengths, ptr, cols

    def set_clouds(self, ptr, cols):
        ptr = np.ascontiguousarray(ptr, dtype=np.int64)
        cols = np.ascontiguousarray(cols, dtype=np.int32)
        self._keep += [ptr, cols]
        load_oracle().orc_set_clouds(self._h, _lp(ptr), _ip(cols))

    def residuals(self, c, phi, phase, voln1rel=0.0):
        c = np.ascontiguousarray(c, dtype=np.float64)
        phi = np.ascontiguousarray(phi, dtype=np.float64)
        phase = np.ascontiguousarray(phase, dtype=np.int32)
        F = np.empty((NSPECIES + 1, self.N))
        load_oracle().orc_residuals(self._h, _dp(c), _dp(phi), _ip(phase), voln1rel, _dp(F))
        return F

    def residuals_implicit(self, c1, phi1, c0, phi0, phase, voln1rel=0.0):
        """The implicit step's residual (5, N) at U^{n+1} = (c1, phi1) from U^n = (c0, phi0)."""
        a = [np.ascontiguousarray(x, dtype=np.float64) for x in (c1, phi1, c0, phi0)]
        phase = np.ascontiguousarray(phase, dtype=np.int32)
        F = np.empty((NSPECIES + 1, self.N))
        load_oracle().orc_residuals_implicit(self._h, _dp(a[0]), _dp(a[1]), _dp(a[2]), _dp(a[3]), _ip(phase),
                                             voln1rel, _dp(F))
        return F

    def chem_implicit_step(self, U, phase, bctypes, bcvalues, voln1rel, data2, datac, datac11):
        """One step of the reference's complete model (ten species and the potential) from
        U (11, N) and phase: returns (U^{n+1}, phase after the flip, Newton iterations,
        GMRES iterations)."""
        U = np.array(U, dtype=np.float64, order="C").reshape(11, self.N)
        ph = np.array(phase, dtype=np.int32)
        bt = np.ascontiguousarray(bctypes, dtype=np.int32)
        bv = np.ascontiguousarray(bcvalues, dtype=np.float64).reshape(11, self.N)
        arr = [np.ascontiguousarray(a, dtype=np.float64) for a in (data2, datac, datac11)]
        kr = C.c_int64(0)
        it = load_oracle().orc_chem_implicit_step(self._h, _dp(U), _ip(ph), _ip(bt), _dp(bv), float(voln1rel),
                                                  _dp(arr[0]), _dp(arr[1]), _dp(arr[2]), C.byref(kr))
        if it < 0:
            raise ValueError("chem_implicit_step: bad argument")
        return U, ph, it, kr.value

    def chem_tangent(self, f, U, phase, bctypes, bcvalues, voln1rel, data2, datac, datac11):
        """The complete model's tangent of field f (0..10): (diag (N,), off per bond slot)."""
        U = np.ascontiguousarray(U, dtype=np.float64).reshape(11, self.N)
        ph = np.ascontiguousarray(phase, dtype=np.int32)
        bt = np.ascontiguousarray(bctypes, dtype=np.int32)
        bv = np.ascontiguousarray(bcvalues, dtype=np.float64).reshape(11, self.N)
        arr = [np.ascontiguousarray(a, dtype=np.float64) for a in (data2, datac, datac11)]
        nnz = load_oracle().orc_nnz(self._h)
        diag = np.empty(self.N)
        off = np.empty(nnz)
        load_oracle().orc_chem_tangent(self._h, f, _dp(U), _ip(ph), _ip(bt), _dp(bv), float(voln1rel),
                                       _dp(arr[0]), _dp(arr[1]), _dp(arr[2]), _dp(diag), _dp(off))
        return diag, off

    def poisson_matrix(self, phase):
        phase = np.ascontiguousarray(phase, dtype=np.int32)
        nnz = load_oracle().orc_nnz(self._h)
        diag = np.empty(self.N)
        off = np.empty(nnz)
        free = np.empty(self.N, dtype=np.uint8)
        load_oracle().orc_poisson_matrix(self._h, _ip(phase), _dp(diag), _dp(off),
                                         free.ctypes.data_as(C.POINTER(C.c_ubyte)))
        return diag, off, free

    def solve_potential(self, c, phase, phi0=None):
        c = np.ascontiguousarray(c, dtype=np.float64)
        phase = np.ascontiguousarray(phase, dtype=np.int32)
        phi = np.zeros(self.N) if phi0 is None else np.array(phi0, dtype=np.float64)
        it = C.c_int(0)
        rel = C.c_double(0)
        load_oracle().orc_solve_potential(self._h, _dp(c), _ip(phase), _dp(phi), C.byref(it),
                                          C.byref(rel))
        return phi, it.value, rel.value

    def forward(self, n_steps):
        return load_oracle().orc_forward(self._h, n_steps)

    def state(self):
        c = np.empty((NSPECIES, self.N))
        phi = np.empty(self.N)
        ph = np.empty(self.N, dtype=np.int32)
        fs = np.empty(self.N, dtype=np.int32)
        load_oracle().orc_get_state(self._h, _dp(c), _dp(phi), _ip(ph), _ip(fs))
        return c, phi, ph, fs

    def set_state(self, c, phi=None, phase=None):
        c = np.ascontiguousarray(c, dtype=np.float64)
        phi = None if phi is None else np.ascontiguousarray(phi, dtype=np.float64)
        phase = None if phase is None else np.ascontiguousarray(phase, dtype=np.int32)
        load_oracle().orc_set_state(self._h, _dp(c), _dp(phi), _ip(phase))

    def implicit_forward(self, n_steps):
        """n implicit steps of the reference's Newton/GMRES loop (main.cpp:640-922); returns
        (Newton iterations, GMRES iterations) summed over the steps."""
        nw, kr = C.c_int64(0), C.c_int64(0)
        st = load_oracle().orc_implicit_forward(self._h, n_steps, C.byref(nw), C.byref(kr))
        if st != 0:
            raise RuntimeError("oracle implicit step failed with status %d" % st)
        return nw.value, kr.value

    def tangent(self, field):
        """(diag (N,), off (nnz incl. self slots,)) of the implicit step's tangent of field
        0..3 (species) or 4 (potential) at the current state, in the layout of clouds()."""
        L = load_oracle()
        diag = np.empty(self.N)
        off = np.empty(L.orc_nnz(self._h))
        L.orc_tangent(self._h, field, _dp(diag), _dp(off))
        return diag, off

    def tangent_gmres(self, field, b, tol=10e-6, restart=30, maxit=200):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.empty(self.N)
        it = load_oracle().orc_tangent_gmres(self._h, field, _dp(b), _dp(x), tol, restart, maxit)
        return x, it

    def diagnostics(self):
        out = np.empty(len(DIAG_KEYS))
        load_oracle().orc_get_diag(self._h, _dp(out))
        return dict(zip(DIAG_KEYS, out.tolist()))


def set_threads(n):
    return load_oracle().orc_set_threads(n)


def library_path():
    """File name of the loaded oracle library."""
    L = load_oracle()
    return os.path.basename(L._name)


# ---------------------------------------------------------------- reference shim --------
def reference_params_vectors(p):
    """data2 (51), datac (10x7), datac11 (4) for the reference's parameter object, from an
    nnpp Params: the hot-path fields, every reaction constant zero (utils.h:2343-2484)."""
    d2 = np.zeros(51)
    d2[2], d2[3], d2[4], d2[5], d2[6] = p.dt, p.dx, p.dy, p.dz, p.delta
    d2[7], d2[8] = p.CSolid, p.CSat
    d2[47], d2[48], d2[49], d2[50] = p.T, p.R, p.F, p.vol_red
    dc = np.zeros((10, 7))
    for k in range(NSPECIES):
        dc[k] = [p.z[k], p.D_solid[k], p.D_liquid[k], p.s1[k], p.s2[k], p.K1[k], p.K2[k]]
    d11 = np.array([p.sigma, p.sigma, p.s_phi, p.K_phi])
    return d2, dc, d11


def ref_build_clouds_hash(max_node_no, r, dx, dy, dz, nodes):
    """(lengths incl. self, row_ptr int64, cols incl. self, max_len) from the reference."""
    L = load_reference()
    if L is None:
        return None
    nodes = np.ascontiguousarray(nodes, dtype=np.float64)
    N = nodes.shape[1]
    ml = C.c_int(0)
    nnz = C.c_int64(0)
    st = L.ref_build_clouds_hash(max_node_no, r, dx, dy, dz, N, _dp(nodes), C.byref(ml),
                                 C.byref(nnz))
    if st != 0:
        raise RuntimeError("reference build_clouds_hash failed (status %d)" % st)
    lengths = np.empty(N, dtype=np.int32)
    ptr = np.empty(N + 1, dtype=np.int64)
    cols = np.empty(nnz.value, dtype=np.int32)
    L.ref_get_clouds(_ip(lengths), _lp(ptr), _ip(cols))
    return lengths, ptr, cols, ml.value


def _u11(c, phi, N):
    U = np.zeros((11, N))
    U[:NSPECIES] = c
    U[10] = phi
    return U


def _bc11(bctypes, bcvalues, N):
    B = -np.ones((11, N))
    B[:NSPECIES] = bcvalues[:NSPECIES]
    B[10] = bcvalues[NSPECIES]
    return B


def ref_residuals(p, nodes, ptr, cols, c, phi, phase, bctypes, bcvalues, voln1rel=0.0):
    """utils::Residuals of the reference; returns F (11, N)."""
    L = load_reference()
    if L is None:
        return None
    N = nodes.shape[1]
    d2, dc, d11 = reference_params_vectors(p)
    U = _u11(c, phi, N)
    B = _bc11(bctypes, bcvalues, N)
    F = np.zeros((11, N))
    L.ref_residuals(N, _dp(np.ascontiguousarray(nodes)), _lp(np.ascontiguousarray(ptr, dtype=np.int64)),
                    _ip(np.ascontiguousarray(cols, dtype=np.int32)), _dp(U),
                    _ip(np.ascontiguousarray(phase, dtype=np.int32)),
                    _ip(np.ascontiguousarray(bctypes, dtype=np.int32)), _dp(B), voln1rel,
                    _dp(d2), _dp(np.ascontiguousarray(dc)), _dp(d11), _dp(F))
    return F


def residuals_full(nodes, ptr, cols, Un1, Un, phase, voln1rel, data2, datac, datac11):
    """The oracle's restatement of the reference's complete residual (ten species, their
    reactions, the potential; utils.h:29-842): clouds in the reference format (ptr int64,
    cols with the node itself first), Un1, Un (11, N).  Returns F (11, N)."""
    N = nodes.shape[1]
    F = np.zeros((11, N))
    load_oracle().orc_residuals_full(N, _dp(np.ascontiguousarray(nodes, dtype=np.float64)),
                                     _lp(np.ascontiguousarray(ptr, dtype=np.int64)),
                                     _ip(np.ascontiguousarray(cols, dtype=np.int32)),
                                     _dp(np.ascontiguousarray(Un1, dtype=np.float64)),
                                     _dp(np.ascontiguousarray(Un, dtype=np.float64)),
                                     _ip(np.ascontiguousarray(phase, dtype=np.int32)), float(voln1rel),
                                     _dp(np.ascontiguousarray(data2, dtype=np.float64)),
                                     _dp(np.ascontiguousarray(datac, dtype=np.float64)),
                                     _dp(np.ascontiguousarray(datac11, dtype=np.float64)), _dp(F))
    return F


def ref_residuals_full(nodes, ptr, cols, Un1, Un, phase, voln1rel, data2, datac, datac11):
    """utils::Residuals of the reference with all ten species, their reactions and the given
    parameter arrays (data2 51, datac (10, 7), datac11 4); Un1, Un (11, N).  Returns F (11, N).
    No Dirichlet values are passed (the residual does not read them)."""
    L = load_reference()
    if L is None:
        return None
    N = nodes.shape[1]
    F = np.zeros((11, N))
    bct = np.ones(N, dtype=np.int32)
    B = -np.ones((11, N))
    L.ref_residuals2(N, _dp(np.ascontiguousarray(nodes)), _lp(np.ascontiguousarray(ptr, dtype=np.int64)),
                     _ip(np.ascontiguousarray(cols, dtype=np.int32)), _dp(np.ascontiguousarray(Un1)),
                     _dp(np.ascontiguousarray(Un)), _ip(np.ascontiguousarray(phase, dtype=np.int32)),
                     _ip(bct), _dp(B), voln1rel, _dp(np.ascontiguousarray(data2, dtype=np.float64)),
                     _dp(np.ascontiguousarray(datac, dtype=np.float64)),
                     _dp(np.ascontiguousarray(datac11, dtype=np.float64)), _dp(F))
    return F


def ref_k11(p, nodes, ptr, cols, c, phi, phase, bctypes, bcvalues, voln1rel=0.0):
    """K11 of utils::NewtonMatrices as COO (rows, cols, values)."""
    L = load_reference()
    if L is None:
        return None
    N = nodes.shape[1]
    d2, dc, d11 = reference_params_vectors(p)
    U = _u11(c, phi, N)
    B = _bc11(bctypes, bcvalues, N)
    args = [N, _dp(np.ascontiguousarray(nodes)), _lp(np.ascontiguousarray(ptr, dtype=np.int64)),
            _ip(np.ascontiguousarray(cols, dtype=np.int32)), _dp(U),
            _ip(np.ascontiguousarray(phase, dtype=np.int32)),
            _ip(np.ascontiguousarray(bctypes, dtype=np.int32)), _dp(B), voln1rel, _dp(d2),
            _dp(np.ascontiguousarray(dc)), _dp(d11)]
    nnz = C.c_int64(0)
    L.ref_newton_k11(*args, C.byref(nnz), None, None, None)
    ri = np.empty(nnz.value, dtype=np.int32)
    ci = np.empty(nnz.value, dtype=np.int32)
    val = np.empty(nnz.value)
    L.ref_newton_k11(*args, C.byref(nnz), _ip(ri), _ip(ci), _dp(val))
    return ri, ci, val


def _ref_tangent_args(p, nodes, ptr, cols, c, phi, phase, bctypes, bcvalues, voln1rel):
    N = nodes.shape[1]
    d2, dc, d11 = reference_params_vectors(p)
    U = _u11(c, phi, N)
    B = _bc11(bctypes, bcvalues, N)
    keep = [np.ascontiguousarray(nodes), np.ascontiguousarray(ptr, dtype=np.int64),
            np.ascontiguousarray(cols, dtype=np.int32), U, np.ascontiguousarray(phase, dtype=np.int32),
            np.ascontiguousarray(bctypes, dtype=np.int32), B, d2, np.ascontiguousarray(dc), d11]
    args = [N, _dp(keep[0]), _lp(keep[1]), _ip(keep[2]), _dp(keep[3]), _ip(keep[4]), _ip(keep[5]),
            _dp(keep[6]), voln1rel, _dp(keep[7]), _dp(keep[8]), _dp(keep[9])]
    return args, keep


def ref_newton_k(which, p, nodes, ptr, cols, c, phi, phase, bctypes, bcvalues, voln1rel=0.0):
    """K_(which+1) of the reference's utils::NewtonMatrices as COO (rows, cols, values)."""
    L = load_reference()
    if L is None:
        return None
    args, keep = _ref_tangent_args(p, nodes, ptr, cols, c, phi, phase, bctypes, bcvalues, voln1rel)
    nnz = C.c_int64(0)
    L.ref_newton_k(which, *args, C.byref(nnz), None, None, None)
    ri = np.empty(nnz.value, dtype=np.int32)
    ci = np.empty(nnz.value, dtype=np.int32)
    val = np.empty(nnz.value)
    L.ref_newton_k(which, *args, C.byref(nnz), _ip(ri), _ip(ci), _dp(val))
    return ri, ci, val


def ref_newton_k_full(which, nodes, ptr, cols, U, phase, bctypes, bcvalues, voln1rel, data2, datac, datac11):
    """K_(which+1) of the reference's utils::NewtonMatrices at U (11, N) with the data files'
    parameter arrays, as COO (rows, cols, values)."""
    L = load_reference()
    if L is None:
        return None
    N = nodes.shape[1]
    keep = [np.ascontiguousarray(nodes, dtype=np.float64), np.ascontiguousarray(ptr, dtype=np.int64),
            np.ascontiguousarray(cols, dtype=np.int32), np.ascontiguousarray(U, dtype=np.float64),
            np.ascontiguousarray(phase, dtype=np.int32), np.ascontiguousarray(bctypes, dtype=np.int32),
            np.ascontiguousarray(bcvalues, dtype=np.float64), np.ascontiguousarray(data2, dtype=np.float64),
            np.ascontiguousarray(datac, dtype=np.float64), np.ascontiguousarray(datac11, dtype=np.float64)]
    args = [N, _dp(keep[0]), _lp(keep[1]), _ip(keep[2]), _dp(keep[3]), _ip(keep[4]), _ip(keep[5]),
            _dp(keep[6]), float(voln1rel), _dp(keep[7]), _dp(keep[8]), _dp(keep[9])]
    nnz = C.c_int64(0)
    L.ref_newton_k(which, *args, C.byref(nnz), None, None, None)
    ri = np.empty(nnz.value, dtype=np.int32)
    ci = np.empty(nnz.value, dtype=np.int32)
    val = np.empty(nnz.value)
    L.ref_newton_k(which, *args, C.byref(nnz), _ip(ri), _ip(ci), _dp(val))
    return ri, ci, val


def ref_gmres_full(which, nodes, ptr, cols, U, phase, bctypes, bcvalues, voln1rel, data2, datac, datac11, b):
    """The reference's Eigen::GMRES solve of K_(which+1) x = b (main.cpp:714-779), the
    tangent at U (11, N) with the data files' parameter arrays; returns (x, iterations)."""
    L = load_reference()
    if L is None:
        return None
    N = nodes.shape[1]
    keep = [np.ascontiguousarray(nodes, dtype=np.float64), np.ascontiguousarray(ptr, dtype=np.int64),
            np.ascontiguousarray(cols, dtype=np.int32), np.ascontiguousarray(U, dtype=np.float64),
            np.ascontiguousarray(phase, dtype=np.int32), np.ascontiguousarray(bctypes, dtype=np.int32),
            np.ascontiguousarray(bcvalues, dtype=np.float64), np.ascontiguousarray(data2, dtype=np.float64),
            np.ascontiguousarray(datac, dtype=np.float64), np.ascontiguousarray(datac11, dtype=np.float64),
            np.ascontiguousarray(b, dtype=np.float64)]
    x = np.empty(N)
    it = L.ref_gmres(which, N, _dp(keep[0]), _lp(keep[1]), _ip(keep[2]), _dp(keep[3]), _ip(keep[4]),
                     _ip(keep[5]), _dp(keep[6]), float(voln1rel), _dp(keep[7]), _dp(keep[8]), _dp(keep[9]),
                     _dp(keep[10]), _dp(x))
    return x, it


def ref_gmres(which, p, nodes, ptr, cols, c, phi, phase, bctypes, bcvalues, b, voln1rel=0.0):
    """The reference's Eigen::GMRES solve of K_(which+1) x = b (main.cpp:714-779)."""
    L = load_reference()
    if L is None:
        return None
    args, keep = _ref_tangent_args(p, nodes, ptr, cols, c, phi, phase, bctypes, bcvalues, voln1rel)
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.empty(nodes.shape[1])
    it = L.ref_gmres(which, *args, _dp(b), _dp(x))
    return x, it


def _adjoint_sigs():
    L = load_oracle()
    if not getattr(L, "_adj", False):
        L.orc_forward_record.restype = C.c_int
        L.orc_forward_record.argtypes = [_P, C.c_int, C.c_int, _DP]
        L.orc_backward.restype = C.c_int
        L.orc_backward.argtypes = [_P, _DP, _DP, _DP]
        L._adj = True
    return L


def oracle_forward_record(o, n_steps, sample_every):
    """FP64 forward recording every step; returns the mass-loss curve."""
    L = _adjoint_sigs()
    curve = np.zeros(n_steps // sample_every)
    st = L.orc_forward_record(o._h, n_steps, sample_every, _dp(curve))
    if st not in (0, 4):
        raise RuntimeError("oracle forward_record failed (%d)" % st)
    return curve


def oracle_backward(o, dL_dcurve):
    """Adjoint of the last recorded run: (dL/dD_liquid (4,), dL/dk_diss)."""
    L = _adjoint_sigs()
    g = np.ascontiguousarray(dL_dcurve, dtype=np.float64)
    gD = np.zeros(NSPECIES)
    gk = np.zeros(1)
    L.orc_backward(o._h, _dp(g), _dp(gD), _dp(gk))
    return gD, float(gk[0])
