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
# the same sources built with the reference's own release flags (CPU baseline)
REF_NATIVE_PATH = os.path.join(HERE, "_ref", "libpeec_ref_native.so")

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


def _cp(a):
    return a.ctypes.data_as(P(abi.Complex))


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


# ---------------------------------------------------------------------
# synthetic mesh arrays (the same numbering as the library's mesher)
# ---------------------------------------------------------------------
def plate_arrays(lx, ly, nx, ny):
    xyz = np.zeros(((nx + 1) * (ny + 1), 3))
    for j in range(ny + 1):
        for i in range(nx + 1):
            xyz[j * (nx + 1) + i] = (lx * i / nx, ly * j / ny, 0.0)
    quads = []
    for j in range(ny):
        for i in range(nx):
            v = j * (nx + 1) + i
            quads.append((v, v + 1, v + 1 + nx + 1, v + nx + 1))
    return xyz, np.array(quads, dtype=np.int32)


def box_arrays(lx, ly, lz, nx, ny, nz):
    # same construction as the library's peec_synth_box (outward winding,
    # first-seen vertex numbering over the faces -z, +z, -y, +y, -x, +x)
    ids, xyz, quads = {}, [], []

    def v(i, j, k):
        if (i, j, k) not in ids:
            ids[(i, j, k)] = len(xyz)
            xyz.append((lx * i / nx, ly * j / ny, lz * k / nz))
        return ids[(i, j, k)]

    for j in range(ny):
        for i in range(nx):
            quads.append((v(i, j, 0), v(i, j + 1, 0), v(i + 1, j + 1, 0), v(i + 1, j, 0)))
    for j in range(ny):
        for i in range(nx):
            quads.append((v(i, j, nz), v(i + 1, j, nz), v(i + 1, j + 1, nz), v(i, j + 1, nz)))
    for k in range(nz):
        for i in range(nx):
            quads.append((v(i, 0, k), v(i + 1, 0, k), v(i + 1, 0, k + 1), v(i, 0, k + 1)))
    for k in range(nz):
        for i in range(nx):
            quads.append((v(i, ny, k), v(i, ny, k + 1), v(i + 1, ny, k + 1), v(i + 1, ny, k)))
    for k in range(nz):
        for j in range(ny):
            quads.append((v(0, j, k), v(0, j, k + 1), v(0, j + 1, k + 1), v(0, j + 1, k)))
    for k in range(nz):
        for j in range(ny):
            quads.append((v(nx, j, k), v(nx, j + 1, k), v(nx, j + 1, k + 1), v(nx, j, k + 1)))
    return np.array(xyz), np.array(quads, dtype=np.int32)


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
        Cp = P(abi.Complex)
        harmonic = [
            ("ref_plane_wave_excitation", C.c_int,
             [P(abi.Mesh), C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, C.c_int, Cp, D, D]),
            ("ref_harmonic_build", C.c_int, [P(abi.Mesh), D, D, D, C.c_double, C.c_int, Cp]),
            ("ref_harmonic_residual", C.c_int,
             [Cp, C.c_size_t, C.c_size_t, C.c_double, D, Cp, Cp, C.c_int, D]),
            ("ref_harmonic_pipeline", C.c_int,
             [P(abi.Mesh), P(abi.DualMesh), C.c_double, C.c_double, C.c_double, C.c_int, C.c_double, C.c_int,
              D, D, D, Cp, Cp, Cp, S, D, D, D, D]),
        ]
        abi._bind(lib, harmonic)
        self.lib = lib

    # ---- harmonic scattering chain (oracle/ref_harmonic.c) ----
    def plane_wave_excitation(self, m, frequency, theta_deg=0.0, phi_deg=0.0, polarization=1, analytic=True,
                              threads=1):
        """(U_inc [Ne] complex, k_hat [3], E0 [3]) of a unit COMPLEX plane
        wave (polarization 1 vertical, 0 horizontal)."""
        U = np.zeros(m.n_edges, dtype=np.complex128)
        kh, e0 = np.zeros(3), np.zeros(3)
        s = self.lib.ref_plane_wave_excitation(C.byref(m.mesh), frequency, theta_deg, phi_deg, polarization,
                                               1 if analytic else 0, threads, _cp(U), _dp(kh), _dp(e0))
        if s != 0:
            raise RuntimeError("reference excitation failed: %d" % s)
        return U, kh, e0

    def harmonic_build(self, m, L, P_, R, frequency, threads=1):
        """Z of the reference's harmonic_build_system from given Lp, P, R."""
        n = m.n_edges + m.n_nodes
        Z = np.zeros((n, n), dtype=np.complex128)
        L = np.ascontiguousarray(L, dtype=np.float64)
        P_ = np.ascontiguousarray(P_, dtype=np.float64)
        Rp = None if R is None else _dp(np.ascontiguousarray(R, dtype=np.float64))
        s = self.lib.ref_harmonic_build(C.byref(m.mesh), _dp(L), _dp(P_), Rp, frequency, threads, _cp(Z))
        if s != 0:
            raise RuntimeError("reference harmonic_build_system failed: %d" % s)
        return Z

    def harmonic_residual(self, Z, ne, nv, frequency, P_, U, x, threads=1):
        """The 7 fields of the reference's harmonic_compute_residual."""
        out = np.zeros(7)
        Z = np.ascontiguousarray(Z, dtype=np.complex128)
        P_ = np.ascontiguousarray(P_, dtype=np.float64)
        U = np.ascontiguousarray(U, dtype=np.complex128)
        x = np.ascontiguousarray(x, dtype=np.complex128)
        s = self.lib.ref_harmonic_residual(_cp(Z), ne, nv, frequency, _dp(P_), _cp(U), _cp(x), threads, _dp(out))
        if s != 0:
            raise RuntimeError("reference harmonic_compute_residual failed: %d" % s)
        return out

    def harmonic_pipeline(self, m, frequency, theta_deg=0.0, phi_deg=0.0, polarization=1, sheet_resistance=0.0,
                          threads=1, matrices=True):
        """The reference's whole harmonic scattering chain on one mesh: a dict
        with x, U, R, pivots, row / column scales, residual[7], times[8] and,
        with matrices=True, L, P and Z."""
        ne, nv = m.n_edges, m.n_nodes
        n = ne + nv
        out = {"x": np.zeros(n, dtype=np.complex128), "U": np.zeros(ne, dtype=np.complex128), "R": np.zeros(ne),
               "pivots": np.zeros(n, dtype=np.uintp), "row_scale": np.zeros(n), "column_scale": np.zeros(n),
               "residual": np.zeros(7), "times": np.zeros(8)}
        if matrices:
            out.update(L=np.zeros((ne, ne)), P=np.zeros((nv, nv)), Z=np.zeros((n, n), dtype=np.complex128))
        g = out.get
        s = self.lib.ref_harmonic_pipeline(
            C.byref(m.mesh), C.byref(m.dual), frequency, theta_deg, phi_deg, polarization, sheet_resistance,
            threads, _dp(g("L")) if matrices else None, _dp(g("P")) if matrices else None, _dp(out["R"]),
            _cp(g("Z")) if matrices else None, _cp(out["U"]), _cp(out["x"]), out["pivots"].ctypes.data_as(S),
            _dp(out["row_scale"]), _dp(out["column_scale"]), _dp(out["residual"]), _dp(out["times"]))
        if s != 0:
            raise RuntimeError("reference harmonic chain failed: %d" % s)
        out["pivots"] = out["pivots"].astype(np.int64)
        return out

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


# ---------------------------------------------------------------------
# harmonic system around the hot path (numpy restatement)
# ---------------------------------------------------------------------
def harmonic_system(L, P_, edges, R, frequency):
    """Z = [R + j w L, A; -P A^T, j w I] as harmonic_build_system
    (src/solver/harmonic.c:175-372) writes it: re = R_ii on the diagonal of
    the top-left block, im = w L_ij; A[e, a] = -1, A[e, b] = +1
    (incidence.c:34-110); -(P[i, b] - P[i, a]) from incidence_build_PAT
    (incidence.c:417-592); j w on the diagonal of the bottom-right block.
    Elementwise, so bit-identical to the reference."""
    L = np.asarray(L, dtype=np.float64)
    P_ = np.asarray(P_, dtype=np.float64)
    e = np.asarray(edges).reshape(-1, 2)
    ne, nv = L.shape[0], P_.shape[0]
    n = ne + nv
    w = 2.0 * np.pi * frequency
    Z = np.zeros((n, n), dtype=np.complex128)
    zr, zi = Z.real, Z.imag          # views into Z
    zi[:ne, :ne] = w * L
    if R is not None:
        zr[np.arange(ne), np.arange(ne)] = np.asarray(R, dtype=np.float64)
    A = np.zeros((ne, nv))
    A[np.arange(ne), e[:, 0]] = -1.0
    A[np.arange(ne), e[:, 1]] = 1.0
    zr[:ne, ne:] = A
    zr[ne:, :ne] = -(P_[:, e[:, 1]] - P_[:, e[:, 0]])
    zi[np.arange(ne, n), np.arange(ne, n)] = w
    return Z


def plane_wave_field(frequency, theta_deg, phi_deg, polarization, amplitude=1.0):
    """(k_hat, E0, wave number) of a harmonic plane wave, as
    incident_field_configure_harmonic builds them (incident_field.c:110-230,
    312-423): k_hat = -(sin t cos p, sin t sin p, cos t); E0 = amplitude *
    e_theta (polarization 1, vertical) or e_phi (0, horizontal); each
    vector normalised by its Euclidean norm; k0 = 2 pi f / c0."""
    c0 = 299792458.0
    t = theta_deg * np.pi / 180.0
    p = phi_deg * np.pi / 180.0
    k_hat = np.array([-np.sin(t) * np.cos(p), -np.sin(t) * np.sin(p), -np.cos(t)])
    e_theta = np.array([np.cos(t) * np.cos(p), np.cos(t) * np.sin(p), -np.sin(t)])
    e_phi = np.array([-np.sin(p), np.cos(p), 0.0])

    def unit(v):
        return v / np.sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2])

    k_hat, e_theta, e_phi = unit(k_hat), unit(e_theta), unit(e_phi)
    E0 = amplitude * (e_theta if polarization == 1 else e_phi)
    return k_hat, E0, 2.0 * np.pi * frequency / c0


def plane_wave_excitation(centers, vectors, k_hat, E0, wave_number, analytic=True):
    """U_inc per edge (scattering.c:140-336): E(r_c) = E0 exp(-j k0 k_hat.r_c)
    (incident_field.c:754-830, zero phase), projected on the edge vector; the
    analytic edge integral multiplies by sinc(k0 k_hat.l / 2), with the
    reference's series 1 - x^2/6 + x^4/120 below |x| = 1e-4."""
    c = np.asarray(centers, dtype=np.float64).reshape(-1, 3)
    v = np.asarray(vectors, dtype=np.float64).reshape(-1, 3)
    kr = k_hat[0] * c[:, 0] + k_hat[1] * c[:, 1] + k_hat[2] * c[:, 2]
    gamma = -wave_number * kr + 0.0
    cs, sn = np.cos(gamma), np.sin(gamma)
    re = (E0[0] * cs) * v[:, 0] + (E0[1] * cs) * v[:, 1] + (E0[2] * cs) * v[:, 2]
    im = (E0[0] * sn) * v[:, 0] + (E0[1] * sn) * v[:, 1] + (E0[2] * sn) * v[:, 2]
    if analytic:
        x = 0.5 * (wave_number * (k_hat[0] * v[:, 0] + k_hat[1] * v[:, 1] + k_hat[2] * v[:, 2]))
        x2 = x * x
        small = np.abs(x) < 1.0e-4
        f = np.where(small, 1.0 - x2 / 6.0 + (x2 * x2) / 120.0, np.sin(x) / np.where(small, 1.0, x))
        re, im = re * f, im * f
    return re + 1j * im


def harmonic_rhs(U, nv):
    """b = [-U_e ; 0] (harmonic_build_rhs, harmonic.c:436-552, no node current)."""
    U = np.asarray(U, dtype=np.complex128)
    return np.concatenate([-U, np.zeros(nv, dtype=np.complex128)])


def harmonic_residual(Z, ne, U, x):
    """The fields of harmonic_compute_residual (harmonic.c:720-1080) as
    [absolute, rhs-relative, backward error, edge absolute, node absolute,
    edge backward error, node backward error]; backward error =
    max_i |r_i| / (sum_j |Z_ij||x_j| + |b_i|).  Summation order differs from
    the reference's, so values agree to rounding, not bit for bit."""
    Z = np.asarray(Z, dtype=np.complex128)
    n = Z.shape[0]
    b = harmonic_rhs(U, n - ne)
    r = Z @ x - b
    ra, ba = np.hypot(r.real, r.imag), np.hypot(b.real, b.imag)
    den = np.hypot(Z.real, Z.imag) @ np.hypot(x.real, x.imag) + ba
    eta = np.where(den > 0, ra / np.where(den > 0, den, 1.0), ra)
    bmax = ba.max()
    return np.array([ra.max(), ra.max() / bmax if bmax > 0 else ra.max(), eta.max(), ra[:ne].max(),
                     ra[ne:].max(), eta[:ne].max(), eta[ne:].max()])
