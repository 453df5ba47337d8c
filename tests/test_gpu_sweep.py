"""Batched frequency sweep (peec_gb300_sweep_*): one mesh's harmonic systems
at many frequencies solved by the mixed solve recorded once into a CUDA
graph and replayed per frequency, with the autotuner's choice of split
terms, refinement sweeps and tile width.

Gate: every system's componentwise backward error <= 1e-10, recomputed
independently (peec_gb300_backward_error_device) from the returned solution
against the FP64 Z and b the harmonic fill and plane-wave kernels build; at
the well-conditioned top of the band the solution agrees with the plain FP64
LU's to 1e-8 (normwise per block)."""
import ctypes as C

import numpy as np
import pytest

from helpers import ComplexLU, DeviceBuffers
from peeeeeeeeeeeeeeeeeeec_gb300 import abi
from peeeeeeeeeeeeeeeeeeec_gb300.mesh import SynthMesh
from peeeeeeeeeeeeeeeeeeec_gb300.workloads import plane_waves

pytestmark = pytest.mark.gpu
C0 = 299792458.0


def mesh_on_device(lib, db, m):
    ne, nv = m.n_edges, m.n_nodes
    lo, po = abi.InductanceOptions(), abi.PotentialOptions()
    lib.inductance_options_default(C.byref(lo), 1)
    lib.potential_options_default(C.byref(po), 1)
    dL, dP = db.alloc(ne * ne * 8), db.alloc(nv * nv * 8)
    assert lib.peec_gb300_inductance_device(C.byref(m.mesh), C.byref(m.dual), C.byref(lo), dL, None) == 0
    assert lib.peec_gb300_potential_device(C.byref(m.mesh), C.byref(m.dual), C.byref(po), dP, None) == 0
    de = db.put(np.ascontiguousarray(m.edges(), dtype=np.int32))
    dc = db.put(m.array("edge_centers", (ne, 3)))
    dv = db.put(m.array("edge_vectors", (ne, 3)))
    return dL, dP, de, dc, dv


@pytest.mark.parametrize("tune", [False, True])
def test_sweep_reaches_gate(gpu_lib, tune):
    lib = gpu_lib
    rng = np.random.default_rng(4)
    k_hat, e_hat = plane_waves(rng, 4)
    freqs = np.logspace(3, 8, 8)
    with SynthMesh.box(0.6, 0.4, 0.3, 6, 4, 3) as m, DeviceBuffers(lib) as db:
        ne, nv = m.n_edges, m.n_nodes
        n = ne + nv
        dL, dP, de, dc, dv = mesh_on_device(lib, db, m)
        kh = np.ascontiguousarray(k_hat)
        eh = np.ascontiguousarray(e_hat)
        plan = lib.peec_gb300_sweep_create(dL, dP, de, None, dc, dv, ne, nv, 4, kh.ctypes.data_as(abi.c_double_p),
                                           eh.ctypes.data_as(abi.c_double_p), None)
        assert plan
        try:
            if tune:
                t = abi.PeecSweepTuning()
                ms = C.c_double()
                probes = np.ascontiguousarray(freqs[[0, 4, 7]])
                assert lib.peec_gb300_sweep_tune(plan, probes.ctypes.data_as(abi.c_double_p), 3, C.byref(t),
                                                 C.byref(ms)) == 0
                assert t.split_terms in (3, 6) and t.sweeps >= 1 and t.tile_bn in (64, 128) and ms.value > 0
            dX = db.alloc(len(freqs) * 4 * n * 16)
            be = np.zeros(len(freqs))
            fb = np.zeros(len(freqs), dtype=np.int32)
            f = np.ascontiguousarray(freqs)
            s = lib.peec_gb300_sweep_run(plan, f.ctypes.data_as(abi.c_double_p), len(freqs), 1e-10, dX,
                                         be.ctypes.data_as(abi.c_double_p), fb.ctypes.data_as(abi.c_int_p))
            assert s == 0, (be, fb)
            assert np.all(be <= 1e-10)
            X = db.get(dX, (len(freqs), 4, n), np.complex128)
        finally:
            lib.peec_gb300_sweep_destroy(plan)
        # independent check of every system: rebuild Z and b, recompute eta
        dZ, db_ = db.alloc(n * n * 16), db.alloc(4 * n * 16)
        for fi, fr in enumerate(freqs):
            assert lib.peec_gb300_harmonic_build_device(dL, dP, de, None, ne, nv, fr, dZ) == 0
            for q in range(4):
                kq = (C.c_double * 3)(*k_hat[q])
                eq = (C.c_double * 3)(*e_hat[q])
                assert lib.peec_gb300_plane_wave_rhs_device(dc, dv, ne, nv, kq, eq, 2 * np.pi * fr / C0,
                                                            db_ + q * n * 16) == 0
            out = (C.c_double * 3)()
            assert lib.peec_gb300_backward_error_device(dZ, n, db.put(X[fi]), db_, 4, out) == 0
            assert out[0] <= 1e-10, (fr, out[0])
            if fi == len(freqs) - 1:
                Z = db.get(dZ, (n, n), np.complex128)
                B = db.get(db_, (4, n), np.complex128)
                lu = ComplexLU(lib, Z)
                assert lu.status == 0
                s, Xp = lu.solve_multiple(B)
                assert s == 0
                lu.free()
                for q in range(4):
                    for sl in (slice(0, ne), slice(ne, n)):
                        err = np.max(np.abs(X[fi, q, sl] - Xp[q, sl])) / np.max(np.abs(Xp[q, sl]))
                        assert err < 1e-8, err
