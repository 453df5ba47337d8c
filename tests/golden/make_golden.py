"""Generate the golden fixtures in this folder from the reference itself.

Runs the reference's own hot-path sources, compiled unchanged into
oracle/_ref/libpeec_ref.so (`make -C oracle ref`), on small seeded inputs and
stores inputs and outputs as .npz files.  The GPU machine has no copy of the
reference, so the tests there compare against these files.

    python tests/golden/make_golden.py            (needs oracle/_ref/libpeec_ref.so)
    python tests/golden/make_golden.py harmonic   (only the harmonic chain)
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "oracle"))

from peeeeeeeeeeeeeeeeeeec_gb300 import abi  # noqa: E402
from oracle import Reference, box_arrays, plate_arrays  # noqa: E402

# the reference's meshes, from the copy `make -C oracle stage` keeps
REF_MESH_DIR = os.path.join(REPO, "baseline", "_ref", "meshes")

_libc = C.CDLL(None)
_libc.malloc.restype = C.c_void_p
_libc.malloc.argtypes = [C.c_size_t]


def _c_copy(arr, ctype):
    p = _libc.malloc(max(1, arr.nbytes))
    C.memmove(p, arr.ctypes.data, arr.nbytes)
    return C.cast(p, C.POINTER(ctype))


def _arr(ptr, shape, dtype):
    n = int(np.prod(shape))
    ctype = C.c_double if dtype == np.float64 else C.c_int
    return np.frombuffer(C.cast(ptr, C.POINTER(ctype * n)).contents, dtype=dtype).reshape(shape).copy()


def reference_case(R, xyz, quads, name, with_matrices=True):
    m = abi.Mesh()
    R.lib.mesh_init(C.byref(m))
    m.n_nodes, m.n_quads = xyz.shape[0], quads.shape[0]
    m.xyz = _c_copy(np.ascontiguousarray(xyz, np.float64), C.c_double)
    m.quads = _c_copy(np.ascontiguousarray(quads, np.int32), C.c_int)
    assert R.lib.mesh_build_topology(C.byref(m)) == 0
    d = abi.DualMesh()
    assert R.lib.dual_mesh_build(C.byref(m), C.byref(d)) == 0
    ne, nv, nq = m.n_edges, m.n_nodes, m.n_quads
    out = dict(
        xyz=xyz, quads=quads,
        edges=_arr(m.edges, (ne, 2), np.int32),
        cell_edges=_arr(m.cell_edges, (nq, 4), np.int32),
        cell_edge_signs=_arr(m.cell_edge_signs, (nq, 4), np.int32),
        edge_lengths=_arr(m.edge_lengths, (ne,), np.float64),
        edge_directions=_arr(m.edge_directions, (ne, 3), np.float64),
        edge_region_areas=np.ctypeslib.as_array(d.edge_region_areas, shape=(ne,)).copy(),
        node_region_areas=np.ctypeslib.as_array(d.node_region_areas, shape=(nv,)).copy(),
        edge_patch_counts=np.array([d.edge_patches[r].count for r in range(ne)]),
        node_patch_counts=np.array([d.node_patches[r].count for r in range(nv)]),
    )
    out["edge_patches"] = np.concatenate([
        np.array([list(d.edge_patches[r].patches[k].points) for k in range(d.edge_patches[r].count)])
        for r in range(ne)])
    out["node_patches"] = np.concatenate([
        np.array([list(d.node_patches[r].patches[k].points) for k in range(d.node_patches[r].count)])
        for r in range(nv)])
    if with_matrices:
        lo = abi.InductanceOptions()
        R.lib.inductance_options_default(C.byref(lo), os.cpu_count())
        L = abi.InductanceMatrix()
        assert R.lib.inductance_compute_matrix(C.byref(m), C.byref(d), C.byref(lo), C.byref(L)) == 0
        out["L"] = np.ctypeslib.as_array(L.data, shape=(ne, ne)).copy()
        po = abi.PotentialOptions()
        R.lib.potential_options_default(C.byref(po), os.cpu_count())
        Pm = abi.PotentialMatrix()
        assert R.lib.potential_compute_matrix(C.byref(m), C.byref(d), C.byref(po), C.byref(Pm)) == 0
        out["P"] = np.ctypeslib.as_array(Pm.data, shape=(nv, nv)).copy()
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print("wrote", name, "Ne=%d Nv=%d" % (ne, nv))


def gmsh_case(R, path, name):
    m = abi.Mesh()
    R.lib.mesh_init(C.byref(m))
    assert R.lib.mesh_load_gmsh(path.encode(), C.byref(m)) == 0
    xyz = _arr(m.xyz, (m.n_nodes, 3), np.float64)
    quads = _arr(m.quads, (m.n_quads, 4), np.int32)
    reference_case(R, xyz, quads, name)


def lu_cases(R):
    rng = np.random.default_rng(20261203)
    out = {}
    for n in (1, 7, 40, 97):
        a = rng.standard_normal((n, n))
        if n == 40:
            a[:, 3] *= 1e-3   # forces pivoting decisions away from the diagonal
        b = rng.standard_normal(n)
        o = abi.LUOptions()
        R.lib.lu_options_default(C.byref(o), 1)
        lu = abi.LUFactorization()
        assert R.lib.lu_factorize(a.ctypes.data_as(abi.c_double_p), n, C.byref(o), C.byref(lu)) == 0
        x = np.zeros(n)
        assert R.lib.lu_solve(C.byref(lu), b.ctypes.data_as(abi.c_double_p), x.ctypes.data_as(abi.c_double_p)) == 0
        out["real%d_a" % n] = a
        out["real%d_b" % n] = b
        out["real%d_lu" % n] = np.ctypeslib.as_array(lu.data, shape=(n, n)).copy()
        out["real%d_piv" % n] = np.ctypeslib.as_array(lu.pivots, shape=(n,)).astype(np.int64)
        out["real%d_x" % n] = x
        out["real%d_det" % n] = np.array(R.lib.lu_determinant(C.byref(lu)))
        R.lib.lu_free(C.byref(lu))
    for n in (1, 5, 33, 80):
        a = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
        a[0, :] *= 1e6  # unequal row scales exercise the equilibration
        b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        o = abi.ComplexLUOptions()
        R.lib.complex_lu_options_default(C.byref(o), 1)
        lu = abi.ComplexLUFactorization()
        ac = np.ascontiguousarray(a)
        assert R.lib.complex_lu_factorize(C.cast(ac.ctypes.data, C.POINTER(abi.Complex)), n, C.byref(o),
                                          C.byref(lu)) == 0
        x = np.zeros(n, dtype=np.complex128)
        bc = np.ascontiguousarray(b)
        assert R.lib.complex_lu_solve(C.byref(lu), C.cast(bc.ctypes.data, C.POINTER(abi.Complex)),
                                      C.cast(x.ctypes.data, C.POINTER(abi.Complex))) == 0
        raw = np.ctypeslib.as_array(C.cast(lu.data, abi.c_double_p), shape=(n * n * 2,)).copy()
        out["cplx%d_a" % n] = a
        out["cplx%d_b" % n] = b
        out["cplx%d_lu" % n] = raw.view(np.complex128).reshape(n, n)
        out["cplx%d_piv" % n] = np.ctypeslib.as_array(lu.pivots, shape=(n,)).astype(np.int64)
        out["cplx%d_rs" % n] = np.ctypeslib.as_array(lu.row_scale, shape=(n,)).copy()
        out["cplx%d_cs" % n] = np.ctypeslib.as_array(lu.column_scale, shape=(n,)).copy()
        out["cplx%d_x" % n] = x
        R.lib.complex_lu_free(C.byref(lu))
    np.savez_compressed(os.path.join(HERE, "lu_cases.npz"), **out)
    print("wrote lu_cases")


def quadrature_cases(R):
    """Single patch pairs in every class, including the reference tests'
    rectangles and partitions, with the reference's K values."""
    rng = np.random.default_rng(7)
    pairs = []
    sq = np.array([0, 0, 0, 1, 0, 0, 1, 1, 0, 0, 1, 0], float)
    for aspect in (1.0, 10.0, 100.0):
        p = np.array([0, 0, 0, aspect, 0, 0, aspect, 1, 0, 0, 1, 0], float)
        pairs.append((p, p, 1))                 # same object (SELF by pointer)
    pairs.append((sq, sq.copy(), 0))            # SELF by geometry
    b = sq.copy()
    b[0::3] += 1
    pairs.append((sq, b, 0))                    # TOUCHING along an edge
    pairs.append((b, sq, 0))
    c = sq.copy()
    c[0::3] += 1
    c[1::3] += 1
    pairs.append((sq, c, 0))                    # TOUCHING at a corner
    d = sq.copy()
    d[2::3] = 1e-7
    pairs.append((sq, d, 0))                    # NEAR (stacked, tiny gap)
    e = sq.copy()
    e[0::3] += 1.3
    pairs.append((sq, e, 0))                    # NEAR (gap 0.3 < 0.5)
    f = sq.copy()
    f[2::3] = 100.0
    pairs.append((sq, f, 0))                    # FAR
    for _ in range(12):                         # random skewed quads at random offsets
        base = rng.uniform(-1, 1, 3)
        q1 = (base + rng.uniform(0, 0.5, (4, 3)) * np.array([1, 1, 0.2])
              + np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]])).ravel()
        off = rng.uniform(-3, 3, 3)
        q2 = (q1.reshape(4, 3) + off).ravel()
        pairs.append((q1, q2, 0))
    rot = np.array([0, 0, 0, 2, 0, 0, 2, 1, 0, 0, 1, 0], float)
    e1, f1 = np.array([0.6, 0.8, 0]), np.array([-0.48, 0.36, 0.8])
    rr = np.array([3.7 * (rot[3 * i] * e1 + rot[3 * i + 1] * f1) + np.array([1, 2, 3]) for i in range(4)]).ravel()
    pairs.append((rr, rr, 1))
    A, B, SAME, K, CLS = [], [], [], [], []
    for pa, pb, same in pairs:
        qa = abi.QuadPatch()
        qb = abi.QuadPatch()
        for t in range(12):
            qa.points[t] = pa[t]
            qb.points[t] = pb[t]
        b_ref = qa if same else qb
        K.append(R.lib.quad_patch_kernel_1_over_r(C.byref(qa), C.byref(b_ref), 4, 10, 12, 8, 0.5))
        CLS.append(R.lib.quad_patch_classify_pair(C.byref(qa), C.byref(b_ref), 0.5))
        A.append(pa)
        B.append(pb)
        SAME.append(same)
    np.savez_compressed(os.path.join(HERE, "quadrature_cases.npz"), a=np.array(A), b=np.array(B),
                        same=np.array(SAME), K=np.array(K), cls=np.array(CLS))
    gl = {}
    for q in (2, 3, 4, 5, 6, 8, 10, 12, 16):
        x, w = np.zeros(16), np.zeros(16)
        R.lib.gauss_legendre_rule(q, x.ctypes.data_as(abi.c_double_p), w.ctypes.data_as(abi.c_double_p))
        gl["x%d" % q] = x[:q]
        gl["w%d" % q] = w[:q]
    np.savez_compressed(os.path.join(HERE, "gauss_legendre.npz"), **gl)
    print("wrote quadrature_cases, gauss_legendre")


# Stage-1 lightning transient on the fixtures' own Lp / P (the reference's
# transient.c / lightning.c driven by oracle/ref_transient.c): every step's
# node self-voltages and edge currents, for backward Euler and trapezoidal.
TRANSIENT_SOURCE = (102900.0, 1500.0, 1.0e6, 0.0)  # the reference's default waveform
TRANSIENT_DT = 1.0e-7


def transient_case(R, name, n_steps, strike, ret, r_edge=1.0e-3):
    f = np.load(os.path.join(HERE, name + ".npz"))
    L, P, edges = f["L"], f["P"], f["edges"].astype(np.int32)
    ne, nv = L.shape[0], P.shape[0]
    Rd = np.full(ne, r_edge)
    out = dict(R=Rd, strike=strike, ret=ret, dt=TRANSIENT_DT, source=np.array(TRANSIENT_SOURCE),
               n_steps=n_steps)
    for scheme in (1, 2):
        s, I, V, probes = R.transient_lightning(L, P, edges, Rd, scheme, TRANSIENT_DT,
                                                TRANSIENT_SOURCE + (strike, ret), n_steps,
                                                probe_nodes=range(nv), probe_edges=range(ne))
        assert s == 0
        out["V%d" % scheme] = probes[:, :nv]
        out["I%d" % scheme] = probes[:, nv:]
    np.savez_compressed(os.path.join(HERE, "transient_" + name + ".npz"), **out)
    print("wrote transient_" + name, n_steps, "steps")


# RCS radiation vectors (rcs.c:701-1000, dual-patch quadrature, one thread so
# that the reference's edge reduction is sequential) of a seeded complex edge
# current on the fixture's own mesh, for a few directions, wave numbers and
# surface orders.
RCS_K = (0.63, 6.3)
RCS_ORDERS = (6, 4)


def rcs_case(R, name):
    from peeeeeeeeeeeeeeeeeeec_gb300.mesh import SynthMesh
    f = np.load(os.path.join(HERE, name + ".npz"))
    rng = np.random.default_rng(11)
    with SynthMesh.from_arrays(f["xyz"], f["quads"]) as m:
        ne = m.n_edges
        cur = rng.standard_normal(ne) + 1j * rng.standard_normal(ne)
        th, ph = np.arccos(rng.uniform(-1, 1, 6)), rng.uniform(0, 2 * np.pi, 6)
        dirs = np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], 1)
        dirs[0] = (0.0, 0.0, 1.0)
        out = dict(current=cur, directions=dirs, k=np.array(RCS_K), orders=np.array(RCS_ORDERS))
        for k in RCS_K:
            for order in RCS_ORDERS:
                s, F = R.rcs_radiation(m, cur, k, dirs, order)
                assert s == 0
                out["F_%g_%d" % (k, order)] = F
    np.savez_compressed(os.path.join(HERE, "rcs_" + name + ".npz"), **out)
    print("wrote rcs_" + name)


# incidence.c:34-741: A, A P A^T, P A^T and A S of the fixture's mesh and
# its reference P, from the reference's own functions.
def incidence_case(R, name):
    from oracle import incidence_products
    from peeeeeeeeeeeeeeeeeeec_gb300.mesh import SynthMesh
    f = np.load(os.path.join(HERE, name + ".npz"))
    with SynthMesh.from_arrays(f["xyz"], f["quads"]) as m:
        assert np.array_equal(m.edges(), f["edges"])
        out = incidence_products(R.lib, m.mesh, f["P"])
    for k, v in out.items():
        assert not isinstance(v, int), (k, v)
    np.savez_compressed(os.path.join(HERE, "incidence_" + name + ".npz"), **out)
    print("wrote incidence_" + name)


# The reference's harmonic scattering chain (oracle/ref_harmonic.c, the calls
# of main.c's solve_harmonic_scattering): Lp, P, P A^T, R, the analytic
# plane-wave excitation, harmonic_build_system, harmonic_factorize,
# harmonic_solve and harmonic_compute_residual, at 30 MHz with a unit
# x-polarised wave from +z (theta 0, phi 0, vertical).  Small cases keep
# every matrix; the 2102-unknown box keeps the solution, pivots, scales and
# residual.  Also: an oblique wave's excitation (theta 60, phi 30,
# horizontal) and the residual of a perturbed solution, whose backward error
# is far above rounding so that implementations can be compared on it.
SIGMA_SHEET = 1.0 / (5.8e7 * 1.0e-3)   # 1 mm copper sheet, ohms per square
HARMONIC_FREQ = 30.0e6


def harmonic_case(R, xyz, quads, name, sheet_resistance, matrices):
    from peeeeeeeeeeeeeeeeeeec_gb300.mesh import SynthMesh
    threads = os.cpu_count()
    with SynthMesh.from_arrays(xyz, quads) as m:
        ne, nv = m.n_edges, m.n_nodes
        out = R.harmonic_pipeline(m, HARMONIC_FREQ, 0.0, 0.0, 1, sheet_resistance, threads, matrices=True)
        U1, kh1, e01 = R.plane_wave_excitation(m, HARMONIC_FREQ, 0.0, 0.0, 1, True, threads)
        assert np.array_equal(U1, out["U"])
        U2, kh2, e02 = R.plane_wave_excitation(m, HARMONIC_FREQ, 60.0, 30.0, 0, True, threads)
        rng = np.random.default_rng(17)
        x = out["x"]
        xp = x * (1.0 + 1e-6 * (rng.standard_normal(x.size) + 1j * rng.standard_normal(x.size)))
        res_p = R.harmonic_residual(out["Z"], ne, nv, HARMONIC_FREQ, out["P"], out["U"], xp, threads)
        edges = m.edges()
        centers = m.array("edge_centers", (ne, 3))
        vectors = m.array("edge_vectors", (ne, 3))
    keep = dict(xyz=xyz, quads=quads, edges=edges, edge_centers=centers, edge_vectors=vectors,
                frequency=HARMONIC_FREQ, sheet_resistance=sheet_resistance, x=x, U=out["U"], R=out["R"],
                pivots=out["pivots"], row_scale=out["row_scale"], column_scale=out["column_scale"],
                residual=out["residual"], k_hat=kh1, E0=e01, U_oblique=U2, k_hat_oblique=kh2, E0_oblique=e02,
                x_perturbed=xp, residual_perturbed=res_p, cpu_seconds=out["times"], threads=threads)
    if matrices:
        keep.update(L=out["L"], P=out["P"], Z=out["Z"])
    np.savez_compressed(os.path.join(HERE, "harmonic_" + name + ".npz"), **keep)
    print("wrote harmonic_%s Ne=%d Nv=%d backward error %.3g, %.1f s" % (name, ne, nv, out["residual"][2],
                                                                        out["times"].sum()))


def harmonic_cases(R):
    harmonic_case(R, *plate_arrays(1.0, 1.0, 4, 4), "plate4", SIGMA_SHEET, True)
    harmonic_case(R, *box_arrays(0.4, 0.2, 0.1, 4, 2, 1), "box421", 0.0, True)
    harmonic_case(R, *box_arrays(1.0, 0.5, 0.25, 20, 10, 5), "box1m_5cm", 0.0, False)


def main():
    if sys.argv[1:] == ["harmonic"]:
        harmonic_cases(Reference())
        return
    if sys.argv[1:] == ["incidence"]:
        R = Reference()
        incidence_case(R, "plate4")
        incidence_case(R, "box421")
        return
    R = Reference()
    quadrature_cases(R)
    lu_cases(R)
    reference_case(R, *plate_arrays(1.0, 1.0, 4, 4), "plate4")
    reference_case(R, *plate_arrays(1.0, 1.0, 8, 8), "plate8")
    reference_case(R, *box_arrays(0.4, 0.2, 0.1, 4, 2, 1), "box421")
    reference_case(R, *box_arrays(2.0, 1.0, 0.5, 40, 20, 10), "box_5cm_topology", with_matrices=False)
    transient_case(R, "plate4", 300, 0, 24)
    transient_case(R, "box421", 200, 0, 5)
    rcs_case(R, "plate4")
    rcs_case(R, "box421")
    incidence_case(R, "plate4")
    incidence_case(R, "box421")
    plate_msh = os.path.join(REF_MESH_DIR, "plate.msh")
    if os.path.exists(plate_msh):
        gmsh_case(R, plate_msh, "plate_msh")
    harmonic_cases(R)


if __name__ == "__main__":
    main()
