"""The reference's CPU path on the host cores, timed on a bounded sample and
extrapolated to one full harmonic solve.  TEST / BASELINE INFRASTRUCTURE
ONLY: bench.py's CPU-baseline leg and its reference arm use it; nothing in
the product imports it.

Which code runs:
  "reference"  oracle/_ref/libpeec_ref_native.so: the reference's own
               sources (staged into baseline/_ref/ and built on this host by
               `make -C oracle ref` with its release flags -O3 -march=native
               -fopenmp), driven by oracle/ref_harmonic.c.  The meshes get
               the reference's own mesh_build_topology / dual_mesh_build.
  "port"       oracle/liboracle.so (the C restatement, bit-exact with the
               reference) where the reference's sources are not here.

Sample of one step (the work the reference's harmonic driver does for one
solve, main.c:700-830 and 1266-1480):
  Lp, P        S rows of the upper triangle each, evenly spaced with an
               offset that moves every step (stratified), all pairs of the
               sampled rows over all threads; scaled by the number of pairs
               of the whole upper triangle over the sampled pairs
  solve chain  a real PEEC system of n = 2102 unknowns (the 1.0 x 0.5 x 0.25 m
               PEC box at 5 cm, 30 MHz, its Lp / P assembled once at set-up
               by the same library): P A^T, excitation + MNA fill, complex LU
               factorisation, solve, residual; the factorisation scaled by
               (N / n)^3, the O(n^2) stages by (N / n)^2
"""
import ctypes as C
import os
import statistics
import time

import numpy as np

from oracle import REF_NATIVE_PATH, ORACLE_PATH, box_arrays, harmonic_residual, harmonic_system, \
    plane_wave_excitation, plane_wave_field
from peeeeeeeeeeeeeeeeeeec_gb300 import abi

P = C.POINTER
D = abi.c_double_p
S = abi.c_size_t_p
GOLDEN_RATIO_FRAC = 0.6180339887498949
LU_BOX = (1.0, 0.5, 0.25, 20, 10, 5)

_libc = C.CDLL(None)
_libc.malloc.restype = C.c_void_p
_libc.malloc.argtypes = [C.c_size_t]


def _c_copy(arr, ctype):
    """malloc'ed copy (the reference's mesh_free releases it with free)."""
    p = _libc.malloc(max(1, arr.nbytes))
    C.memmove(p, arr.ctypes.data, arr.nbytes)
    return C.cast(p, P(ctype))


class _Mesh:
    def __init__(self, impl, box):
        self.impl = impl
        self.mesh, self.dual = abi.Mesh(), abi.DualMesh()
        lib = impl.lib
        if impl.kind == "reference":
            xyz, quads = box_arrays(*box)
            lib.mesh_init(C.byref(self.mesh))
            self.mesh.n_nodes, self.mesh.n_quads = xyz.shape[0], quads.shape[0]
            self.mesh.xyz = _c_copy(np.ascontiguousarray(xyz, np.float64), C.c_double)
            self.mesh.quads = _c_copy(np.ascontiguousarray(quads, np.int32), C.c_int)
            assert lib.mesh_build_topology(C.byref(self.mesh)) == 0
            lib.dual_mesh_init(C.byref(self.dual))
            assert lib.dual_mesh_build(C.byref(self.mesh), C.byref(self.dual)) == 0
        else:
            assert lib.peec_synth_box(*box, C.byref(self.mesh)) == 0
            assert lib.peec_synth_topology(C.byref(self.mesh)) == 0
            assert lib.peec_synth_dual(C.byref(self.mesh), C.byref(self.dual)) == 0
        self.n_edges, self.n_nodes = self.mesh.n_edges, self.mesh.n_nodes

    def edges(self):
        return np.ctypeslib.as_array(self.mesh.edges, shape=(self.n_edges, 2)).copy()

    def array(self, name, shape):
        return np.ctypeslib.as_array(getattr(self.mesh, name), shape=shape).copy()


class CpuReference:
    def __init__(self, prefer="reference"):
        if prefer == "reference" and os.path.exists(REF_NATIVE_PATH):
            self.kind, self.path = "reference", REF_NATIVE_PATH
            lib = C.CDLL(REF_NATIVE_PATH)
            abi._bind(lib, [
                ("mesh_init", None, [P(abi.Mesh)]),
                ("mesh_build_topology", C.c_int, [P(abi.Mesh)]),
                ("dual_mesh_init", None, [P(abi.DualMesh)]),
                ("dual_mesh_build", C.c_int, [P(abi.Mesh), P(abi.DualMesh)]),
                ("inductance_options_default", None, [P(abi.InductanceOptions), C.c_int]),
                ("inductance_compute_matrix", C.c_int,
                 [P(abi.Mesh), P(abi.DualMesh), P(abi.InductanceOptions), P(abi.InductanceMatrix)]),
                ("potential_options_default", None, [P(abi.PotentialOptions), C.c_int]),
                ("potential_compute_matrix", C.c_int,
                 [P(abi.Mesh), P(abi.DualMesh), P(abi.PotentialOptions), P(abi.PotentialMatrix)]),
                ("ref_sample_rows", C.c_int, [P(abi.Mesh), P(abi.DualMesh), C.c_int, S, C.c_size_t, C.c_int, D]),
                ("ref_harmonic_from_matrices", C.c_int,
                 [P(abi.Mesh), D, D, D, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, P(abi.Complex), D, D]),
            ])
        else:
            self.kind, self.path = "port", ORACLE_PATH
            lib = C.CDLL(ORACLE_PATH)
            abi._bind(lib, abi.MESH_SYMBOLS)
            abi._bind(lib, [
                ("oracle_sample_rows", C.c_int, [P(abi.Mesh), P(abi.DualMesh), C.c_int, S, C.c_size_t, C.c_int, D]),
                ("oracle_inductance_matrix", C.c_int,
                 [P(abi.Mesh), P(abi.DualMesh), P(C.c_int), C.c_double, C.c_double, C.c_int, D]),
                ("oracle_potential_matrix", C.c_int,
                 [P(abi.Mesh), P(abi.DualMesh), P(C.c_int), C.c_double, C.c_int, D]),
                ("oracle_complex_lu_factorize", C.c_int, [D, C.c_size_t, C.c_double, C.c_int, D, S, S, D, D, D]),
                ("oracle_complex_lu_solve", C.c_int, [D, S, D, D, C.c_size_t, D, D]),
            ])
        self.lib = lib
        self.meshes = {}
        self.lu_case = None

    def mesh(self, box):
        if box not in self.meshes:
            self.meshes[box] = _Mesh(self, box)
        return self.meshes[box]

    # ---- set-up: the n = 2102 system's Lp / P (untimed) ----
    def _lu_system(self, threads):
        if self.lu_case is None:
            m = self.mesh(LU_BOX)
            ne, nv = m.n_edges, m.n_nodes
            L, Pm = np.zeros((ne, ne)), np.zeros((nv, nv))
            if self.kind == "reference":
                lo, po = abi.InductanceOptions(), abi.PotentialOptions()
                self.lib.inductance_options_default(C.byref(lo), threads)
                self.lib.potential_options_default(C.byref(po), threads)
                Lr, Pr = abi.InductanceMatrix(), abi.PotentialMatrix()
                assert self.lib.inductance_compute_matrix(C.byref(m.mesh), C.byref(m.dual), C.byref(lo),
                                                          C.byref(Lr)) == 0
                assert self.lib.potential_compute_matrix(C.byref(m.mesh), C.byref(m.dual), C.byref(po),
                                                         C.byref(Pr)) == 0
                L[:] = np.ctypeslib.as_array(Lr.data, shape=(ne, ne))
                Pm[:] = np.ctypeslib.as_array(Pr.data, shape=(nv, nv))
            else:
                orders = (C.c_int * 4)(4, 10, 12, 8)
                assert self.lib.oracle_inductance_matrix(C.byref(m.mesh), C.byref(m.dual), orders, 0.5, 1e-10,
                                                         threads, L.ctypes.data_as(D)) == 0
                assert self.lib.oracle_potential_matrix(C.byref(m.mesh), C.byref(m.dual), orders, 0.5, threads,
                                                        Pm.ctypes.data_as(D)) == 0
            self.lu_case = (m, L, Pm)
        return self.lu_case

    # ---- timed pieces ----
    def sample_rows(self, m, kind, rows, threads):
        n = m.n_edges if kind == 0 else m.n_nodes
        r = np.ascontiguousarray(rows, dtype=np.uintp)
        out = np.zeros((len(r), n))
        fn = self.lib.ref_sample_rows if self.kind == "reference" else self.lib.oracle_sample_rows
        t = time.perf_counter()
        s = fn(C.byref(m.mesh), C.byref(m.dual), kind, r.ctypes.data_as(S), len(r), threads, out.ctypes.data_as(D))
        dt = time.perf_counter() - t
        assert s == 0, "sampled rows failed"
        return dt, out

    def solve_chain(self, frequency, threads):
        """(seconds per stage, backward error) of the n = 2102 system."""
        m, L, Pm = self._lu_system(threads)
        ne, nv = m.n_edges, m.n_nodes
        n = ne + nv
        if self.kind == "reference":
            x = np.zeros(n, dtype=np.complex128)
            res, tm = np.zeros(7), np.zeros(5)
            s = self.lib.ref_harmonic_from_matrices(C.byref(m.mesh), L.ctypes.data_as(D), Pm.ctypes.data_as(D), None,
                                                    frequency, 0.0, 0.0, 1, threads,
                                                    x.ctypes.data_as(P(abi.Complex)), res.ctypes.data_as(D),
                                                    tm.ctypes.data_as(D))
            assert s == 0, "reference harmonic chain failed"
            stages = dict(zip(["pat", "fill", "factor", "solve", "residual"], tm.tolist()))
            return stages, float(res[2])
        # port: the C restatement for the factor and solve, numpy for the rest
        t0 = time.perf_counter()
        Z = harmonic_system(L, Pm, m.edges(), None, frequency)
        kh, e0, k0 = plane_wave_field(frequency, 0.0, 0.0, 1)
        U = plane_wave_excitation(m.array("edge_centers", (ne, 3)), m.array("edge_vectors", (ne, 3)), kh, e0, k0)
        b = np.concatenate([-U, np.zeros(nv, dtype=np.complex128)])
        t1 = time.perf_counter()
        lu, piv = np.zeros_like(Z), np.zeros(n, dtype=np.uintp)
        rs, cs = np.zeros(n), np.zeros(n)
        sc, scale = C.c_size_t(0), C.c_double(0)
        assert self.lib.oracle_complex_lu_factorize(Z.ctypes.data_as(D), n, 1e-14, threads, lu.ctypes.data_as(D),
                                                    piv.ctypes.data_as(S), C.byref(sc), C.byref(scale),
                                                    rs.ctypes.data_as(D), cs.ctypes.data_as(D)) == 0
        t2 = time.perf_counter()
        x = np.zeros(n, dtype=np.complex128)
        assert self.lib.oracle_complex_lu_solve(lu.ctypes.data_as(D), piv.ctypes.data_as(S), rs.ctypes.data_as(D),
                                                cs.ctypes.data_as(D), n, b.ctypes.data_as(D),
                                                x.ctypes.data_as(D)) == 0
        t3 = time.perf_counter()
        be = harmonic_residual(Z, ne, U, x)[2]
        t4 = time.perf_counter()
        return {"pat": 0.0, "fill": t1 - t0, "factor": t2 - t1, "solve": t3 - t2, "residual": t4 - t3}, float(be)

    def sample_solve(self, box, frequency, threads, rows=(32, 32), step=0):
        """One bounded sample, extrapolated: (seconds per full solve, phase
        seconds (extrapolated), sample seconds (measured), description)."""
        m = self.mesh(box)
        ne, nv = m.n_edges, m.n_nodes
        N = ne + nv
        u = (0.5 + step * GOLDEN_RATIO_FRAC) % 1.0
        parts, measured = {}, 0.0
        for kind, count, name in ((0, ne, "Lp"), (1, nv, "P")):
            S_ = rows[kind]
            sel = np.minimum((np.arange(S_) + u) * count / S_, count - 1).astype(np.int64)
            dt, _ = self.sample_rows(m, kind, sel, threads)
            measured += dt
            pairs = float(np.sum(count - sel))
            parts[name] = dt * (count * (count + 1) / 2.0) / pairs
        stages, be = self.solve_chain(frequency, threads)
        n = self._lu_system(threads)[0]
        n = n.n_edges + n.n_nodes
        measured += sum(stages.values())
        q2, q3 = (N / n) ** 2, (N / n) ** 3
        parts["mna_fill_pat_rhs"] = (stages["pat"] + stages["fill"]) * q2
        parts["complex_lu"] = stages["factor"] * q3
        parts["solve"] = stages["solve"] * q2
        parts["backward_error"] = stages["residual"] * q2
        desc = ("%s code, %d threads: Lp and P each %d / %d evenly spaced rows of the upper triangle (stratified, "
                "offset moving per step), all their pairs, scaled by pair count; harmonic chain (P A^T, excitation + "
                "MNA fill, complex LU, solve, residual) of a real %d-unknown PEEC system (1.0 x 0.5 x 0.25 m PEC box, "
                "5 cm, %g MHz), factorisation scaled by (N/n)^3 = %.1f, O(n^2) stages by (N/n)^2 = %.1f; "
                "backward error of the sampled solve %.2g"
                % ("the reference's own" if self.kind == "reference" else "oracle restatement of the reference",
                   threads, rows[0], rows[1], n, frequency / 1e6, q3, q2, be))
        return sum(parts.values()), parts, measured, desc


def run_steps(impl, box, frequency, threads, steps, warmup, rows=(32, 32)):
    """Median of `steps` extrapolated solve times after `warmup` samples."""
    times, last, measured = [], None, []
    for i in range(warmup + steps):
        sec, parts, meas, desc = impl.sample_solve(box, frequency, threads, rows, step=i)
        if i >= warmup:
            times.append(sec)
            measured.append(meas)
        last = (parts, desc)
    return statistics.median(times), last[0], statistics.median(measured), last[1]
