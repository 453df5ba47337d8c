"""The harmonic system that feeds every solve, pinned to the reference's own
harmonic chain.  The fixtures were written by the reference
(tests/golden/make_golden.py harmonic, via oracle/ref_harmonic.c):
harmonic_build_system (harmonic.c:175-372), incident_field_configure_harmonic +
scattering_build_harmonic_excitation with the analytic edge integral
(incident_field.c:312-423, scattering.c:263-336), harmonic_factorize /
harmonic_solve (complex_lu.c) and harmonic_compute_residual
(harmonic.c:720-1080), on a resistive plate, a small PEC box and the
1.0 x 0.5 x 0.25 m PEC box at 5 cm (N = 2102), 30 MHz, unit x-polarised
plane wave from +z.

Bars:
  MNA fill                bit-identical to the reference's Z
  plane-wave RHS          within 1e-14 of its largest entry (the device sin /
                          cos may differ from the host's by an ulp)
  backward error          within 1e-6 relative (the device sums the
                          denominator sum_j |Z_ij||x_j| in FP32)
  LU on identical inputs  pivots and equilibration scales identical (the
                          reference's Z; the oracle's restatement of
                          complex_lu_factorize on the GPU-built Z at N = 2102)
  solution                branch currents and node potentials within 1e-10
                          relative, normwise per block (max |dI| / max |I|,
                          max |dV| / max |V|), for the reference's Z and for
                          the whole GPU chain (GPU Lp / P -> device fill ->
                          drop-in complex_lu_factorize / complex_lu_solve);
                          backward error <= 1e-10
"""
import ctypes as C

import numpy as np
import pytest

from conftest import golden
from helpers import ComplexLU, DeviceBuffers, inductance, potential
from peeeeeeeeeeeeeeeeeeec_gb300 import abi
from peeeeeeeeeeeeeeeeeeec_gb300.mesh import SynthMesh

pytestmark = pytest.mark.gpu
C0 = 299792458.0
SOLUTION_TOL = 1e-10


def device_fill(lib, db, L, P, edges, R, frequency):
    ne, nv = L.shape[0], P.shape[0]
    n = ne + nv
    dZ = db.alloc(n * n * 16)
    dR = None if R is None else db.put(np.asarray(R, dtype=np.float64))
    s = lib.peec_gb300_harmonic_build_device(db.put(L), db.put(P), db.put(np.asarray(edges, dtype=np.int32)), dR,
                                             ne, nv, frequency, dZ)
    assert s == 0
    return dZ


def device_rhs(lib, db, centers, vectors, nv, k_hat, E0, frequency):
    ne = centers.shape[0]
    d = db.alloc((ne + nv) * 16)
    kh = (C.c_double * 3)(*k_hat)
    eh = (C.c_double * 3)(*E0)
    s = lib.peec_gb300_plane_wave_rhs_device(db.put(centers), db.put(vectors), ne, nv, kh, eh,
                                             2.0 * np.pi * frequency / C0, d)
    assert s == 0
    return d


def device_backward_error(lib, db, dZ, n, x, b):
    out = (C.c_double * 3)()
    assert lib.peec_gb300_backward_error_device(dZ, n, db.put(x), db.put(b), 1, out) == 0
    return out[0], out[1], out[2]


@pytest.mark.parametrize("name", ["plate4", "box421"])
def test_mna_fill_bit_identical_to_reference(gpu_lib, name):
    g = golden("harmonic_" + name)
    n = g["Z"].shape[0]
    with DeviceBuffers(gpu_lib) as db:
        dZ = device_fill(gpu_lib, db, g["L"], g["P"], g["edges"], g["R"], float(g["frequency"]))
        Z = db.get(dZ, (n, n), np.complex128)
    assert np.array_equal(Z.view(np.uint64), g["Z"].view(np.uint64))


def test_mna_fill_bit_identical_at_size(gpu_lib):
    """At N = 2102, from the GPU's own Lp / P and a resistive diagonal: the
    device fill equals the oracle's fill (itself bit-identical to the
    reference's harmonic_build_system on the fixtures) of the same inputs."""
    from oracle import harmonic_system
    g = golden("harmonic_box1m_5cm")
    with SynthMesh.from_arrays(g["xyz"], g["quads"]) as m:
        assert np.array_equal(m.edges(), g["edges"])
        s, L = inductance(gpu_lib, m)
        assert s == 0
        s, P = potential(gpu_lib, m)
        assert s == 0
    R = np.random.default_rng(3).uniform(1e-5, 1e-3, L.shape[0])
    n = L.shape[0] + P.shape[0]
    with DeviceBuffers(gpu_lib) as db:
        for Rd in (None, R):
            dZ = device_fill(gpu_lib, db, L, P, g["edges"], Rd, 30e6)
            Z = db.get(dZ, (n, n), np.complex128)
            ref = harmonic_system(L, P, g["edges"], Rd, 30e6)
            assert np.array_equal(Z.view(np.uint64), ref.view(np.uint64))


@pytest.mark.parametrize("name", ["plate4", "box421", "box1m_5cm"])
@pytest.mark.parametrize("wave", ["", "_oblique"])
def test_plane_wave_rhs_matches_reference(gpu_lib, name, wave):
    g = golden("harmonic_" + name)
    ne = g["edges"].shape[0]
    nv = g["x"].shape[0] - ne
    with DeviceBuffers(gpu_lib) as db:
        d = device_rhs(gpu_lib, db, g["edge_centers"], g["edge_vectors"], nv, g["k_hat" + wave], g["E0" + wave],
                       float(g["frequency"]))
        b = db.get(d, (ne + nv,), np.complex128)
    U = g["U" + wave]
    assert np.max(np.abs(b[:ne] + U)) <= 1e-14 * np.max(np.abs(U))
    assert not np.any(b[ne:])


@pytest.mark.parametrize("name", ["plate4", "box421"])
def test_backward_error_matches_reference(gpu_lib, name):
    """On a perturbed solution (backward error ~1e-6, far above rounding)."""
    g = golden("harmonic_" + name)
    ne, n = g["L"].shape[0], g["Z"].shape[0]
    b = np.concatenate([-g["U"], np.zeros(n - ne, dtype=np.complex128)])
    ref = g["residual_perturbed"]
    with DeviceBuffers(gpu_lib) as db:
        dZ = db.put(g["Z"])
        eta, rmax, bmax = device_backward_error(gpu_lib, db, dZ, n, g["x_perturbed"], b)
        eta0, _, _ = device_backward_error(gpu_lib, db, dZ, n, g["x"], b)
    assert abs(eta - ref[2]) <= 1e-6 * ref[2]
    assert abs(rmax - ref[0]) <= 1e-9 * ref[0]
    assert abs(bmax - np.max(np.abs(b))) <= 1e-15 * bmax
    assert eta0 <= 1e-10


def block_errors(x, xr, ne):
    """Normwise errors of the branch currents and node potentials."""
    err_I = np.max(np.abs(x[:ne] - xr[:ne])) / np.max(np.abs(xr[:ne]))
    err_V = np.max(np.abs(x[ne:] - xr[ne:])) / np.max(np.abs(xr[ne:]))
    return err_I, err_V


def device_factor_solve(lib, db, Z, d_b):
    n = Z.shape[0]
    dLU = db.put(Z)
    dpiv, dperm = db.alloc(n * 8), db.alloc(n * 4)
    drs, dcs = db.alloc(n * 8), db.alloc(n * 8)
    scale, col = C.c_double(), C.c_int()
    assert lib.peec_gb300_complex_lu_factor_device(dLU, n, 1e-14, dpiv, dperm, drs, dcs, C.byref(scale),
                                                   C.byref(col)) == 0
    dx = db.alloc(n * 16)
    assert lib.peec_gb300_complex_lu_solve_device(dLU, dperm, drs, dcs, n, d_b, dx, 1) == 0
    return db.get(dx, (n,), np.complex128), db.get(dpiv, (n,), np.int64), db.get(dLU, (n, n), np.complex128)


@pytest.mark.parametrize("name", ["plate4", "box421"])
def test_lu_of_reference_system_matches_reference(gpu_lib, name):
    """The drop-in complex_lu_factorize / complex_lu_solve and the device-
    resident factor / solve on the reference's own Z and b: pivots and
    scales identical, solution within 1e-10 per block.  On these meshes
    several pivot candidates of a column tie to the last bit after the
    equilibration (each is its row's largest entry over that row's scale),
    so this also checks that ties go to the first row, as in the
    reference."""
    g = golden("harmonic_" + name)
    Z, ne = g["Z"], g["L"].shape[0]
    b = np.concatenate([-g["U"], np.zeros(Z.shape[0] - ne, dtype=np.complex128)])
    lu = ComplexLU(gpu_lib, Z)
    assert lu.status == 0
    _, piv, rs, cs = lu.factors()
    s, x = lu.solve(b)
    assert s == 0
    lu.free()
    assert np.array_equal(piv, g["pivots"])
    assert np.array_equal(rs, g["row_scale"]) and np.array_equal(cs, g["column_scale"])
    with DeviceBuffers(gpu_lib) as db:
        x_dev, piv_dev, _ = device_factor_solve(gpu_lib, db, Z, db.put(b))
    assert np.array_equal(piv_dev, g["pivots"])
    for xs in (x, x_dev):
        err_I, err_V = block_errors(xs, g["x"], ne)
        assert err_I < SOLUTION_TOL and err_V < SOLUTION_TOL, (err_I, err_V)


@pytest.mark.parametrize("name", ["plate4", "box421", "box1m_5cm"])
def test_solve_chain_matches_reference(gpu_lib, name):
    """The whole chain on the GPU against the reference's solution: drop-in
    Lp / P (inductance_compute_matrix / potential_compute_matrix), device MNA
    fill and plane-wave RHS, drop-in complex_lu_factorize / complex_lu_solve
    on the host arrays, and the device-resident factor / solve beside it.
    Pivots are compared on identical inputs (above, and against the oracle
    at N = 2102 below), not here: Lp / P within 1e-14 of the reference's
    can move a pivot candidate by an ulp, and candidates that tie to the
    last bit on structured meshes then rank the other way."""
    g = golden("harmonic_" + name)
    f = float(g["frequency"])
    with SynthMesh.from_arrays(g["xyz"], g["quads"]) as m:
        assert np.array_equal(m.edges(), g["edges"])
        s, L = inductance(gpu_lib, m)
        assert s == 0
        s, P = potential(gpu_lib, m)
        assert s == 0
    ne, nv = L.shape[0], P.shape[0]
    n = ne + nv
    R = g["R"] if np.any(g["R"]) else None
    with DeviceBuffers(gpu_lib) as db:
        dZ = device_fill(gpu_lib, db, L, P, g["edges"], R, f)
        d_b = device_rhs(gpu_lib, db, g["edge_centers"], g["edge_vectors"], nv, g["k_hat"], g["E0"], f)
        Z = db.get(dZ, (n, n), np.complex128)
        b = db.get(d_b, (n,), np.complex128)
        lu = ComplexLU(gpu_lib, Z)
        assert lu.status == 0
        s, x = lu.solve(b)
        assert s == 0
        lu.free()
        eta, _, _ = device_backward_error(gpu_lib, db, dZ, n, x, b)
        x_dev, _, _ = device_factor_solve(gpu_lib, db, Z, d_b)
    for xs in (x, x_dev):
        err_I, err_V = block_errors(xs, g["x"], ne)
        assert err_I < SOLUTION_TOL, "branch currents: %g" % err_I
        assert err_V < SOLUTION_TOL, "node potentials: %g" % err_V
    assert eta <= 1e-10
    assert g["residual"][2] <= 1e-10


def test_lu_at_size_matches_oracle(gpu_lib, oracle):
    """N = 2102 (the same panel, update and wavefront-solve kernels as the
    8402-unknown headline): the GPU's complex LU of the GPU-assembled PEEC
    system against the oracle's (the reference's complex_lu_factorize and
    complex_lu_solve restated in C, pinned bit for bit) on the same Z, run
    on the host: pivots and scales identical, packed factors within 1e-12
    of their largest entry, solution within 1e-10 per block."""
    g = golden("harmonic_box1m_5cm")
    f = float(g["frequency"])
    with SynthMesh.from_arrays(g["xyz"], g["quads"]) as m:
        s, L = inductance(gpu_lib, m)
        assert s == 0
        s, P = potential(gpu_lib, m)
        assert s == 0
    ne, nv = L.shape[0], P.shape[0]
    n = ne + nv
    with DeviceBuffers(gpu_lib) as db:
        dZ = device_fill(gpu_lib, db, L, P, g["edges"], None, f)
        d_b = device_rhs(gpu_lib, db, g["edge_centers"], g["edge_vectors"], nv, g["k_hat"], g["E0"], f)
        Z = db.get(dZ, (n, n), np.complex128)
        b = db.get(d_b, (n,), np.complex128)
        x_dev, piv_dev, LU_dev = device_factor_solve(gpu_lib, db, Z, d_b)
    lu = ComplexLU(gpu_lib, Z)
    assert lu.status == 0
    LU, piv, rs, cs = lu.factors()
    s, x = lu.solve(b)
    lu.free()
    import os
    so, LUo, pivo, _, _, rso, cso = oracle.complex_lu_factorize(Z, threads=os.cpu_count())
    assert so == 0
    _, xo = oracle.complex_lu_solve(LUo, pivo, rso, cso, b)
    pivo = pivo.astype(np.int64)
    assert np.array_equal(piv, pivo) and np.array_equal(piv_dev, pivo)
    assert np.array_equal(rs, rso) and np.array_equal(cs, cso)
    scale = np.max(np.abs(LUo))
    assert np.max(np.abs(LU - LUo)) <= 1e-12 * scale
    for xs in (x, x_dev):
        err_I, err_V = block_errors(xs, xo, ne)
        assert err_I < SOLUTION_TOL and err_V < SOLUTION_TOL, (err_I, err_V)
