"""Retarded Lp / P (kernel exp(-jkR)/R; no reference counterpart) on the GPU
against the oracle's FP64 restatement of the same formula.

The static part is the quasi-static pipeline itself (parity 1e-12); the
correction D_k = integral of (exp(-jkR) - 1)/R runs on the FP32 pipes, with
the product rule's order lowered to 3 or 2 for patch pairs far apart
relative to their size and the wavelength; the oracle applies the far order
to every pair.  The tolerance stated here: |GPU - oracle| <= 1e-12 |entry| +
1e-5 max|D_k| per entry.  k = 0 must give the static matrices bit for bit."""
import ctypes as C

import numpy as np
import pytest

from helpers import inductance, potential
from peeeeeeeeeeeeeeeeeeec_gb300 import abi
from peeeeeeeeeeeeeeeeeeec_gb300.mesh import SynthMesh

pytestmark = pytest.mark.gpu


def retarded(lib, m, kind, k):
    n = m.n_edges if kind == 0 else m.n_nodes
    d = lib.peec_gb300_device_alloc(n * n * 16)
    try:
        if kind == 0:
            o = abi.InductanceOptions()
            lib.inductance_options_default(C.byref(o), 1)
            s = lib.peec_gb300_inductance_retarded_device(C.byref(m.mesh), C.byref(m.dual), C.byref(o), k, d, None)
        else:
            o = abi.PotentialOptions()
            lib.potential_options_default(C.byref(o), 1)
            s = lib.peec_gb300_potential_retarded_device(C.byref(m.mesh), C.byref(m.dual), C.byref(o), k, d, None)
        out = np.zeros((n, n), dtype=np.complex128)
        if s == 0:
            assert lib.peec_gb300_copy_to_host(out.ctypes.data, d, out.nbytes) == 0
        return s, out
    finally:
        lib.peec_gb300_device_free(d)


# box_fine: 5 cm cells, so that patch pairs of all three correction orders
# (2, 3 and the far order) occur at 30 and 100 MHz
MESHES = {"plate4": lambda: SynthMesh.plate(1.0, 1.0, 4, 4),
          "box421": lambda: SynthMesh.box(0.4, 0.2, 0.1, 4, 2, 1),
          "box_2m": lambda: SynthMesh.box(2.0, 1.0, 0.5, 8, 4, 2),
          "box_fine": lambda: SynthMesh.box(0.5, 0.25, 0.125, 10, 5, 3)}


@pytest.mark.parametrize("name", list(MESHES))
@pytest.mark.parametrize("k", [0.63, 2.1, 6.3])  # 30 MHz, 100 MHz, 300 MHz
def test_against_oracle(gpu_lib, oracle, name, k):
    with MESHES[name]() as m:
        for kind in (0, 1):
            s, g = retarded(gpu_lib, m, kind, k)
            so, o = oracle.retarded(m, kind, k)
            assert s == 0 and so == 0
            st = (oracle.inductance(m) if kind == 0 else oracle.potential(m))[1]
            D = o - st
            tol = 1e-12 * np.abs(o) + 1e-5 * np.max(np.abs(D))
            assert np.all(np.abs(g - o) <= tol), (name, kind, np.max(np.abs(g - o) / tol))
            assert np.array_equal(g, g.T)  # reciprocity, mirrored exactly
            if kind == 0:
                assert np.array_equal(g == 0, st == 0)  # orthogonal edges stay exact zeros


def test_zero_wave_number_is_the_static_matrix(gpu_lib):
    with SynthMesh.box(0.4, 0.2, 0.1, 4, 2, 1) as m:
        for kind, static in ((0, inductance), (1, potential)):
            s, g = retarded(gpu_lib, m, kind, 0.0)
            s0, st = static(gpu_lib, m)
            assert s == 0 and s0 == 0
            assert np.array_equal(g.real, st) and not g.imag.any()
        assert retarded(gpu_lib, m, 0, -1.0)[0] == -1
        assert retarded(gpu_lib, m, 1, float("nan"))[0] == -1


def test_retarded_harmonic_solve(gpu_lib):
    """Complex MNA fill from retarded Lp / P equals the host construction,
    and a plain FP64 solve of it meets the 1e-10 backward-error gate."""
    from helpers import ComplexLU
    f = 100e6
    k = 2 * np.pi * f / 299792458.0
    with SynthMesh.box(0.4, 0.2, 0.1, 8, 4, 2) as m:
        ne, nv = m.n_edges, m.n_nodes
        n = ne + nv
        s1, L = retarded(gpu_lib, m, 0, k)
        s2, P = retarded(gpu_lib, m, 1, k)
        assert s1 == 0 and s2 == 0
        edges = np.ascontiguousarray(m.edges())
        bufs = []

        def put(a):
            a = np.ascontiguousarray(a)
            p = gpu_lib.peec_gb300_device_alloc(a.nbytes)
            gpu_lib.peec_gb300_copy_to_device(p, a.ctypes.data, a.nbytes)
            bufs.append(p)
            return p

        dL, dP, dE = put(L), put(P), put(edges)
        dZ = gpu_lib.peec_gb300_device_alloc(n * n * 16)
        bufs.append(dZ)
        assert gpu_lib.peec_gb300_harmonic_build_retarded_device(dL, dP, dE, None, ne, nv, f, dZ) == 0
        Z = np.zeros((n, n), dtype=np.complex128)
        gpu_lib.peec_gb300_copy_to_host(Z.ctypes.data, dZ, Z.nbytes)
        for p in bufs:
            gpu_lib.peec_gb300_device_free(p)
    w = 2 * np.pi * f
    A = np.zeros((ne, nv))
    A[np.arange(ne), edges[:, 0]] = -1.0
    A[np.arange(ne), edges[:, 1]] = 1.0
    Zh = np.block([[1j * w * L, A], [-(P @ A.T), 1j * w * np.eye(nv)]])
    assert np.max(np.abs(Z - Zh)) <= 1e-14 * np.max(np.abs(Zh))
    rng = np.random.default_rng(1)
    b = np.concatenate([rng.standard_normal(ne) + 1j * rng.standard_normal(ne), np.zeros(nv)])
    lu = ComplexLU(gpu_lib, Z)
    assert lu.status == 0
    s, x = lu.solve(b)
    lu.free()
    assert s == 0
    be = np.max(np.abs(Z @ x - b) / (np.abs(Z) @ np.abs(x) + np.abs(b)))
    assert be <= 1e-10
