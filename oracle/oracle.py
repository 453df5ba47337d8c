"""ctypes bindings of the CPU checkers.  TEST INFRASTRUCTURE ONLY.

  Oracle()     oracle/liboracle.so, the C restatement (peec_oracle.c)
  Reference()  oracle/_ref/libpeec_ref.so, the reference's own sources
               (only where they were compiled, i.e. not on the GPU host)

Only tests/, the smoke check and the bench's CPU-baseline leg import this.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from peeeeeeeeeeeeeeeeeeec_gb300 import abi  # noqa: E402  (struct layouts)

ORACLE_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libpeec_ref.so")

D = abi.c_double_p
S = abi.c_size_t_p
P = C.POINTER


def _dp(a):
    return a.ctypes.data_as(D)


class Oracle:
    def __init__(self, path=ORACLE_PATH):
        if not os.path.exists(path):
            raise RuntimeError("oracle library missing: run __graft_entry__.build()")
        lib = C.CDLL(path)
        sig = [
            ("oracle_gauss_legendre_rule", C.c_int, [C.c_int, D, D]),
            ("oracle_classify_pair", C.c_int, [P(abi.QuadPatch), P(abi.QuadPatch), C.c_double]),
            ("oracle_patch_kernel", C.c_double,
             [P(abi.QuadPatch), P(abi.QuadPatch), C.c_int, C.c_int, C.c_int, C.c_int, C.c_double]),
            ("oracle_potential_evaluations", C.c_ulonglong, [C.c_int]),
            ("oracle_inductance_matrix", C.c_int,
             [P(abi.Mesh), P(abi.DualMesh), P(C.c_int), C.c_double, C.c_double, C.c_int, D]),
            ("oracle_inductance_rows", C.c_int,
             [P(abi.Mesh), P(abi.DualMesh), P(C.c_int), C.c_double, C.c_double, C.c_int,
              C.c_size_t, C.c_size_t, D]),
            ("oracle_potential_matrix", C.c_int,
             [P(abi.Mesh), P(abi.DualMesh), P(C.c_int), C.c_double, C.c_int, D]),
            ("oracle_potential_rows", C.c_int,
             [P(abi.Mesh), P(abi.DualMesh), P(C.c_int), C.c_double, C.c_int, C.c_size_t,
              C.c_size_t, D]),
            ("oracle_lu_factorize", C.c_int,
             [D, C.c_size_t, C.c_double, C.c_int, D, S, S, D]),
            ("oracle_lu_solve", C.c_int, [D, S, C.c_size_t, D, D]),
            ("oracle_complex_lu_factorize", C.c_int,
             [D, C.c_size_t, C.c_double, C.c_int, D, S, S, D, D, D]),
            ("oracle_complex_lu_solve", C.c_int, [D, S, D, D, C.c_size_t, D, D]),
            ("oracle_retarded_matrix", C.c_int,
             [P(abi.Mesh), P(abi.DualMesh), C.c_int, P(C.c_int), C.c_double, C.c_double, C.c_double,
              C.c_int, D]),
            ("oracle_transient_stage1_matrix", C.c_int,
             [D, D, P(C.c_int), D, C.c_size_t, C.c_size_t, C.c_int, C.c_double, D, D, D]),
            ("oracle_transient_rhs_stage1", C.c_int,
             [D, D, D, D, P(C.c_int), C.c_size_t, C.c_size_t, C.c_int, C.c_double, D, D, D, D, D]),
            ("oracle_rcs_radiation_vector", C.c_int,
             [P(abi.Mesh), P(abi.DualMesh), P(abi.Complex), C.c_double, D, C.c_int, P(abi.Complex)]),
            ("oracle_lightning_current", C.c_double,
             [C.c_double, C.c_double, C.c_double, C.c_double, C.c_double]),
            ("oracle_transient_lightning", C.c_int,
             [D, D, P(C.c_int), D, C.c_size_t, C.c_size_t, C.c_int, C.c_double, C.c_double,
              C.c_double, C.c_double, C.c_double, C.c_size_t, C.c_size_t, C.c_size_t, D, D,
              P(C.c_int), C.c_size_t, P(C.c_int), C.c_size_t, D]),
            ("oracle_incidence_apat", None, [D, P(C.c_int), C.c_size_t, C.c_size_t, D]),
            ("oracle_incidence_pat", C.c_int, [D, P(C.c_int), C.c_size_t, C.c_size_t, D, P(C.c_longlong)]),
            ("oracle_incidence_as", C.c_int, [D, P(C.c_int), C.c_size_t, C.c_size_t, D]),
        ]
        for name, res, args in sig:
            f = getattr(lib, name)
            f.restype, f.argtypes = res, args
        self.lib = lib

    @staticmethod
    def _orders(o):
        return (C.c_int * 4)(*o)

    def gauss_legendre(self, order):
        x, w = np.zeros(16), np.zeros(16)
        if self.lib.oracle_gauss_legendre_rule(order, _dp(x), _dp(w)) != 0:
            return None
        return x[:order], w[:order]

    def patch_kernel(self, a, b, orders=(4, 10, 12, 8), near_factor=0.5):
        return self.lib.oracle_patch_kernel(C.byref(a), C.byref(b), *orders, near_factor)

    def classify(self, a, b, near_factor=0.5):
        return self.lib.oracle_classify_pair(C.byref(a), C.byref(b), near_factor)

    def inductance(self, m, orders=(4, 10, 12, 8), near_factor=0.5, tol=1e-10, threads=None,
                   rows=None):
        n = m.n_edges
        out = np.zeros((n, n))
        threads = threads or os.cpu_count()
        if rows is None:
            s = self.lib.oracle_inductance_matrix(C.byref(m.mesh), C.byref(m.dual), self._orders(orders),
                                                  near_factor, tol, threads, _dp(out))
        else:
            s = self.lib.oracle_inductance_rows(C.byref(m.mesh), C.byref(m.dual), self._orders(orders),
                                                near_factor, tol, threads, rows[0], rows[1], _dp(out))
        return s, out

    def potential(self, m, orders=(4, 10, 12, 8), near_factor=0.5, threads=None, rows=None):
        n = m.n_nodes
        out = np.zeros((n, n))
        threads = threads or os.cpu_count()
        if rows is None:
            s = self.lib.oracle_potential_matrix(C.byref(m.mesh), C.byref(m.dual), self._orders(orders),
                                                 near_factor, threads, _dp(out))
        else:
            s = self.lib.oracle_potential_rows(C.byref(m.mesh), C.byref(m.dual), self._orders(orders),
                                               near_factor, threads, rows[0], rows[1], _dp(out))
        return s, out

    def lu_factorize(self, a, tol=1e-14, threads=None):
        a = np.ascontiguousarray(a, dtype=np.float64)
        n = a.shape[0]
        lu = np.zeros_like(a)
        piv = np.zeros(n, dtype=np.uintp)
        sc, scale = C.c_size_t(0), C.c_double(0)
        s = self.lib.oracle_lu_factorize(_dp(a), n, tol, threads or os.cpu_count(), _dp(lu),
                                         piv.ctypes.data_as(S), C.byref(sc), C.byref(scale))
        return s, lu, piv, sc.value, scale.value

    def lu_solve(self, lu, piv, b):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros_like(b)
        s = self.lib.oracle_lu_solve(_dp(lu), piv.ctypes.data_as(S), lu.shape[0], _dp(b), _dp(x))
        return s, x

    def complex_lu_factorize(self, a, tol=1e-14, threads=None):
        a = np.ascontiguousarray(a, dtype=np.complex128)
        n = a.shape[0]
        lu = np.zeros_like(a)
        piv = np.zeros(n, dtype=np.uintp)
        rs, cs = np.zeros(n), np.zeros(n)
        sc, scale = C.c_size_t(0), C.c_double(0)
        s = self.lib.oracle_complex_lu_factorize(
            a.ctypes.data_as(D), n, tol, threads or os.cpu_count(), lu.ctypes.data_as(D),
            piv.ctypes.data_as(S), C.byref(sc), C.byref(scale), _dp(rs), _dp(cs))
        return s, lu, piv, sc.value, scale.value, rs, cs

    def complex_lu_solve(self, lu, piv, rs, cs, b):
        b = np.ascontiguousarray(b, dtype=np.complex128)
        x = np.zeros_like(b)
        s = self.lib.oracle_complex_lu_solve(lu.ctypes.data_as(D), piv.ctypes.data_as(S), _dp(rs), _dp(cs),
                                             lu.shape[0], b.ctypes.data_as(D), x.ctypes.data_as(D))
        return s, x

    def incidence_apat(self, P_, edges):
        Pc, e, K = _incidence_oracle(P_, edges, (len(edges), len(edges)))
        self.lib.oracle_incidence_apat(Pc.ctypes.data_as(D), e.ctypes.data_as(P(C.c_int)), Pc.shape[0], len(e),
                                       K.ctypes.data_as(D))
        return K

    def incidence_pat(self, P_, edges):
        """(status, PAT, first non-finite row-major index or -1)"""
        Pc, e, out = _incidence_oracle(P_, edges, (P_.shape[0], len(edges)))
        bad = C.c_longlong()
        s = self.lib.oracle_incidence_pat(Pc.ctypes.data_as(D), e.ctypes.data_as(P(C.c_int)), Pc.shape[0], len(e),
                                          out.ctypes.data_as(D), C.byref(bad))
        return s, out, bad.value

    def incidence_as(self, P_, edges):
        """(status, AS)"""
        Pc, e, out = _incidence_oracle(P_, edges, (len(edges), P_.shape[0]))
        s = self.lib.oracle_incidence_as(Pc.ctypes.data_as(D), e.ctypes.data_as(P(C.c_int)), Pc.shape[0], len(e),
                                         out.ctypes.data_as(D))
        return s, out

    def retarded(self, m, kind, wave_number, orders=(4, 10, 12, 8), near_factor=0.5, tol=1e-10,
                 threads=None):
        """kind 0: Lp, 1: P with the exp(-jkR)/R kernel (complex n x n)."""
        n = m.n_edges if kind == 0 else m.n_nodes
        out = np.zeros((n, n), dtype=np.complex128)
        s = self.lib.oracle_retarded_matrix(C.byref(m.mesh), C.byref(m.dual), kind, self._orders(orders),
                                            near_factor, tol, wave_number, threads or os.cpu_count(),
                                            out.ctypes.data_as(D))
        return s, out

    def rcs_radiation(self, m, current, wave_number, directions, order=6):
        """[n_dir][3] complex radiation vectors of one edge current vector."""
        return _rcs(self.lib.oracle_rcs_radiation_vector, m, current, wave_number, directions,
                    lambda f, cur, d, out: f(C.byref(m.mesh), C.byref(m.dual), cur, wave_number, d, order, out))

    def transient_matrix(self, L, P_, edges, R, scheme, dt):
        ne, nv = L.shape[0], P_.shape[0]
        nt = ne + nv
        M, F, AS = np.zeros((nt, nt)), np.zeros(nv), np.zeros((ne, nv))
        s = self.lib.oracle_transient_stage1_matrix(
            _dp(L), _dp(P_), _ip(edges), None if R is None else _dp(R), ne, nv, scheme, dt,
            _dp(M), _dp(F), _dp(AS))
        return s, M, F, AS

    def transient_lightning(self, L, P_, edges, R, scheme, dt, source, n_steps, I=None, V=None,
                            probe_nodes=(), probe_edges=()):
        return _transient_lightning(self.lib.oracle_transient_lightning, L, P_, edges, R, scheme,
                                    dt, source, n_steps, I, V, probe_nodes, probe_edges)


def _ip(a):
    return a.ctypes.data_as(P(C.c_int))


def _transient_lightning(fn, L, P_, edges, R, scheme, dt, source, n_steps, I, V, probe_nodes,
                         probe_edges):
    """source = (K, alpha, beta, delay, strike_node, return_node).  Returns
    (status, I, V, probes [n_steps][len(probe_nodes) + len(probe_edges)])."""
    L = np.ascontiguousarray(L, dtype=np.float64)
    P_ = np.ascontiguousarray(P_, dtype=np.float64)
    edges = np.ascontiguousarray(edges, dtype=np.int32)
    ne, nv = L.shape[0], P_.shape[0]
    I = np.zeros(ne) if I is None else np.array(I, dtype=np.float64)
    V = np.zeros(nv) if V is None else np.array(V, dtype=np.float64)
    pn = np.ascontiguousarray(probe_nodes, dtype=np.int32)
    pe = np.ascontiguousarray(probe_edges, dtype=np.int32)
    probes = np.zeros((n_steps, len(pn) + len(pe)))
    Rp = None if R is None else _dp(np.ascontiguousarray(R, dtype=np.float64))
    K, alpha, beta, delay, strike, ret = source
    s = fn(_dp(L), _dp(P_), _ip(edges), Rp, ne, nv, scheme, dt, K, alpha, beta, delay, strike, ret,
           n_steps, _dp(I), _dp(V), _ip(pn), len(pn), _ip(pe), len(pe), _dp(probes))
    return s, I, V, probes


def _rcs(fn, m, current, wave_number, directions, call):
    cur = np.ascontiguousarray(current, dtype=np.complex128)
    dirs = np.ascontiguousarray(directions, dtype=np.float64).reshape(-1, 3)
    out = np.zeros((dirs.shape[0], 3), dtype=np.complex128)
    cp = cur.ctypes.data_as(P(abi.Complex))
    for q in range(dirs.shape[0]):
        d = np.ascontiguousarray(dirs[q])
        o = (abi.Complex * 3)()
        s = call(fn, cp, _dp(d), o)
        if s != 0:
            return s, out
        out[q] = [complex(o[c].re, o[c].im) for c in range(3)]
    return 0, out


class RcsOptions(C.Structure):
    """rcs.h RcsOptions (integration 1 = dual-patch quadrature)."""
    _fields_ = [("integration", C.c_int), ("surface_order", C.c_int), ("parallel_threads", C.c_int)]


def _incidence_oracle(P_, edges, shape):
    Pc = np.ascontiguousarray(P_, dtype=np.float64)
    e = np.ascontiguousarray(np.asarray(edges).reshape(-1, 2), dtype=np.int32)
    return Pc, e, np.zeros(shape)


def incidence_products(lib, mesh, P_, threads=1):
    """Call the incidence.h functions of a library with the drop-in ABI (the
    reference's own, or the GB300 one) on a Mesh struct and a dense P:
    {"A", "APAT", "PAT", "AS"} as numpy arrays, or the int status of the
    first call that failed under that key."""
    libc = C.CDLL(None)
    libc.free.argtypes = [C.c_void_p]
    nv = P_.shape[0]
    Pc = np.ascontiguousarray(P_, dtype=np.float64)
    Pm = abi.PotentialMatrix(nv, Pc.ctypes.data_as(D))
    out = {}
    A = abi.IncidenceMatrix()
    s = lib.incidence_build(C.byref(mesh), C.byref(A))
    if s != 0:
        return {"A": s}
    out["A"] = np.ctypeslib.as_array(A.data, shape=(A.rows, A.cols)).copy()
    for name, call in (("APAT", lambda M: lib.incidence_build_APAT(C.byref(mesh), C.byref(Pm), C.byref(M), threads)),
                       ("PAT", lambda M: lib.incidence_build_PAT(C.byref(mesh), C.byref(Pm), C.byref(M), threads)),
                       ("AS", lambda M: lib.incidence_build_AS(C.byref(A), C.byref(Pm), C.byref(M), threads))):
        M = abi.Matrix()
        s = call(M)
        if s != 0:
            out[name] = s
            continue
        out[name] = np.ctypeslib.as_array(M.data, shape=(M.rows, M.cols)).copy()
        libc.free(C.cast(M.data, C.c_void_p))
    libc.free(C.cast(A.data, C.c_void_p))
    return out


def reference_available():
    return os.path.exists(REF_PATH)


class Reference:
    """The reference's own hot-path functions (same ABI as the drop-in)."""

    def __init__(self, path=REF_PATH):
        lib = C.CDLL(path)
        abi._bind(lib, abi.DROP_IN_SYMBOLS)
        extra = [
            ("mesh_init", None, [P(abi.Mesh)]),
            ("mesh_free", None, [P(abi.Mesh)]),
            ("mesh_load_gmsh", C.c_int, [C.c_char_p, P(abi.Mesh)]),
            ("mesh_build_topology", C.c_int, [P(abi.Mesh)]),
            ("dual_mesh_init", None, [P(abi.DualMesh)]),
            ("dual_mesh_free", None, [P(abi.DualMesh)]),
            ("dual_mesh_build", C.c_int, [P(abi.Mesh), P(abi.DualMesh)]),
        ]
        abi._bind(lib, extra)
        f = lib.rcs_compute_radiation_vector
        f.restype, f.argtypes = C.c_int, [P(abi.Mesh), P(abi.DualMesh), P(abi.Complex), C.c_double, D,
                                          P(RcsOptions), P(abi.Complex)]
        f = lib.ref_transient_lightning
        f.restype, f.argtypes = C.c_int, [D, D, P(C.c_int), D, C.c_size_t, C.c_size_t, C.c_int, C.c_double, C.c_double,
              C.c_double, C.c_double, C.c_double, C.c_size_t, C.c_size_t, C.c_size_t, D, D,
              P(C.c_int), C.c_size_t, P(C.c_int), C.c_size_t, D]
        self.lib = lib

    def rcs_radiation(self, m, current, wave_number, directions, order=6):
        """The reference's rcs_compute_radiation_vector (one thread: its
        edge reduction is then sequential)."""
        opt = RcsOptions(1, order, 1)
        return _rcs(self.lib.rcs_compute_radiation_vector, m, current, wave_number, directions,
                    lambda f, cur, d, out: f(C.byref(m.mesh), C.byref(m.dual), cur, wave_number, d,
                                             C.byref(opt), out))

    def transient_lightning(self, L, P_, edges, R, scheme, dt, source, n_steps, I=None, V=None,
                            probe_nodes=(), probe_edges=()):
        return _transient_lightning(self.lib.ref_transient_lightning, L, P_, edges, R, scheme, dt,
                                    source, n_steps, I, V, probe_nodes, probe_edges)
