"""Stage-1 lightning transient on the device (peec_gb300_transient_*) against
the reference's own waveforms (golden fixtures made by the reference's
transient.c / lightning.c) and the oracle.

Tolerances, relative to the waveform maximum over every step: edge currents
within 1e-11 and node self-voltages within 2e-9.  The oracle matches the
reference to 1e-13 / 7e-10; the device solve applies explicit inverses of
its 64 x 64 diagonal blocks instead of substituting, which moves currents
by a few 1e-12 (rounding times the blocks' condition), and self-voltages
integrate small differences of edge currents, so any change of summation
order shows there first."""
import ctypes as C

import numpy as np
import pytest

from conftest import golden
from peeeeeeeeeeeeeeeeeeec_gb300.mesh import SynthMesh

pytestmark = pytest.mark.gpu

I_TOL = 1e-11
V_TOL = 2e-9


def werr(got, ref):
    return np.max(np.abs(got - ref)) / np.max(np.abs(ref))


class DeviceTransient:
    def __init__(self, lib, L, P, edges, R, scheme, dt):
        self.lib = lib
        self.ne, self.nv = L.shape[0], P.shape[0]
        self.bufs = []
        self.dL = self.put(L)
        self.dP = self.put(P)
        self.dE = self.put(np.ascontiguousarray(edges, dtype=np.int32))
        self.dR = None if R is None else self.put(R)
        h = C.c_void_p()
        self.status = lib.peec_gb300_transient_create(self.dL, self.dP, self.dE, self.dR, self.ne, self.nv,
                                                      scheme, dt, C.byref(h))
        self.h = h

    def put(self, a):
        a = np.ascontiguousarray(a)
        p = self.lib.peec_gb300_device_alloc(max(a.nbytes, 8))
        assert self.lib.peec_gb300_copy_to_device(p, a.ctypes.data, a.nbytes) == 0
        self.bufs.append(p)
        return p

    def run(self, source, n_steps, step0=0, I=None, V=None, probe_nodes=None, probe_edges=None):
        lib = self.lib
        I = np.zeros(self.ne) if I is None else np.array(I, dtype=np.float64)
        V = np.zeros(self.nv) if V is None else np.array(V, dtype=np.float64)
        pn = np.arange(self.nv, dtype=np.int32) if probe_nodes is None else np.asarray(probe_nodes, np.int32)
        pe = np.arange(self.ne, dtype=np.int32) if probe_edges is None else np.asarray(probe_edges, np.int32)
        dI, dV = self.put(I), self.put(V)
        dpn, dpe = self.put(pn), self.put(pe)
        probes = np.zeros((n_steps, len(pn) + len(pe)))
        dpr = lib.peec_gb300_device_alloc(max(probes.nbytes, 8))
        self.bufs.append(dpr)
        K, alpha, beta, delay, strike, ret = source
        s = lib.peec_gb300_transient_lightning(self.h, K, alpha, beta, delay, strike, ret, step0, n_steps, dI, dV,
                                               dpn, len(pn), dpe, len(pe), dpr)
        if s == 0:
            assert lib.peec_gb300_copy_to_host(I.ctypes.data, dI, I.nbytes) == 0
            assert lib.peec_gb300_copy_to_host(V.ctypes.data, dV, V.nbytes) == 0
            if probes.size:
                assert lib.peec_gb300_copy_to_host(probes.ctypes.data, dpr, probes.nbytes) == 0
        return s, I, V, probes

    def close(self):
        if self.h:
            self.lib.peec_gb300_transient_destroy(self.h)
            self.h = None
        for p in self.bufs:
            self.lib.peec_gb300_device_free(p)
        self.bufs = []


@pytest.mark.parametrize("name", ["plate4", "box421"])
@pytest.mark.parametrize("scheme", [1, 2])
def test_against_reference_waveforms(gpu_lib, name, scheme):
    f, g = golden(name), golden("transient_" + name)
    nv = f["P"].shape[0]
    src = tuple(g["source"]) + (int(g["strike"]), int(g["ret"]))
    t = DeviceTransient(gpu_lib, f["L"], f["P"], f["edges"], g["R"], scheme, float(g["dt"]))
    try:
        assert t.status == 0
        s, I, V, probes = t.run(src, int(g["n_steps"]))
        assert s == 0
        assert werr(probes[:, nv:], g["I%d" % scheme]) < I_TOL
        assert werr(probes[:, :nv], g["V%d" % scheme]) < V_TOL
        assert np.array_equal(probes[-1, :nv], V) and np.array_equal(probes[-1, nv:], I)
    finally:
        t.close()


def test_against_oracle_on_the_16x16_plate(gpu_lib, oracle):
    """The 16 x 16 unit plate (Ne 544, Nv 289, N 833) as a real MNA: Lp and P
    assembled on the GPU, sheet resistance 1/(5.8e7 * 1 mm) per square,
    current injected at node 0 and returned at the opposite corner."""
    from helpers import inductance, potential
    with SynthMesh.plate(1.0, 1.0, 16, 16) as m:
        s1, L = inductance(gpu_lib, m)
        s2, P = potential(gpu_lib, m)
        assert s1 == 0 and s2 == 0
        edges = np.ascontiguousarray(m.edges())
        rs = 1.0 / (5.8e7 * 1e-3)
        w = 1.0 / 16  # every edge of the uniform grid crosses one cell width
        R = rs * m.edge_lengths() / w
        src = (102900.0, 1500.0, 1.0e6, 3e-7, 0, m.n_nodes - 1)
        for scheme in (1, 2):
            t = DeviceTransient(gpu_lib, L, P, edges, R, scheme, 1e-7)
            try:
                assert t.status == 0
                s, I, V, probes = t.run(src, 120)
                assert s == 0
                so, Io, Vo, po = oracle.transient_lightning(L, P, edges, R, scheme, 1e-7, src, 120,
                                                            probe_nodes=range(m.n_nodes),
                                                            probe_edges=range(m.n_edges))
                assert so == 0
                assert werr(probes[:, m.n_nodes:], po[:, m.n_nodes:]) < I_TOL
                assert werr(probes[:, :m.n_nodes], po[:, :m.n_nodes]) < V_TOL
            finally:
                t.close()


def test_continued_runs_match_one_run(gpu_lib):
    """Two runs (steps 0..99, then 100..249 from the returned state) give the
    one-run result bit for bit: the state and the step clock carry over."""
    f, g = golden("plate4"), golden("transient_plate4")
    src = tuple(g["source"]) + (int(g["strike"]), int(g["ret"]))
    t = DeviceTransient(gpu_lib, f["L"], f["P"], f["edges"], g["R"], 2, float(g["dt"]))
    try:
        s, I, V, full = t.run(src, 250)
        s1, I1, V1, p1 = t.run(src, 100)
        s2, I2, V2, p2 = t.run(src, 150, step0=100, I=I1, V=V1)
        assert s == s1 == s2 == 0
        assert np.array_equal(np.vstack([p1, p2]), full)
        assert np.array_equal(I2, I) and np.array_equal(V2, V)
    finally:
        t.close()


def test_invalid_inputs(gpu_lib):
    f = golden("plate4")
    ne = f["L"].shape[0]
    t = DeviceTransient(gpu_lib, f["L"], f["P"], f["edges"], np.zeros(ne), 3, 1e-7)
    assert t.status == -1
    t.close()
    t = DeviceTransient(gpu_lib, f["L"], f["P"], f["edges"], None, 1, 0.0)
    assert t.status == -1
    t.close()
    bad = f["P"].copy()
    bad[4, 4] = -1.0
    t = DeviceTransient(gpu_lib, f["L"], bad, f["edges"], None, 1, 1e-7)
    assert t.status == -1
    t.close()
    t = DeviceTransient(gpu_lib, f["L"], f["P"], f["edges"], None, 1, 1e-7)
    try:
        assert t.status == 0
        assert t.run((1.0, 1e6, 1500.0, 0.0, 0, 3), 5)[0] == -1      # beta <= alpha
        assert t.run((1.0, 1500.0, 1e6, 0.0, 2, 2), 5)[0] == -1      # same node twice
        assert t.run((1.0, 1500.0, 1e6, 0.0, 0, 10 ** 6), 5)[0] == -1  # outside the mesh
        s, I, V, probes = t.run((1.0, 1500.0, 1e6, 0.0, 0, 3), 3, probe_nodes=[0, 10 ** 6], probe_edges=[-1])
        assert s == 0 and np.isfinite(probes[:, 0]).all() and np.isnan(probes[:, 1:]).all()
    finally:
        t.close()


def test_batched_runs_equal_single_runs(gpu_lib):
    """Three runs with different sources stepped together (every matrix of a
    step read once for all) give each run's single-run waveforms bit for
    bit; bad run counts are refused."""
    f, g = golden("box421"), golden("transient_box421")
    ne, nv = f["L"].shape[0], f["P"].shape[0]
    nt = ne + nv
    srcs = [(102900.0, 1500.0, 1.0e6, 0.0, 0, 5), (105139.0, 2127.18, 246066.0, 2e-7, 3, 17),
            (5.0e4, 1000.0, 5.0e5, 0.0, 11, 2)]
    t = DeviceTransient(gpu_lib, f["L"], f["P"], f["edges"], g["R"], 2, 1e-7)
    try:
        single = [t.run(src, 120, probe_nodes=range(nv), probe_edges=range(ne)) for src in srcs]
        n = len(srcs)
        X = np.zeros((n, nt))
        dX = t.put(X)
        pn, pe = t.put(np.arange(nv, dtype=np.int32)), t.put(np.arange(ne, dtype=np.int32))
        dpr = gpu_lib.peec_gb300_device_alloc(120 * n * nt * 8)
        t.bufs.append(dpr)
        col = lambda k: (C.c_double * n)(*[s[k] for s in srcs])
        sz = lambda k: (C.c_size_t * n)(*[s[k] for s in srcs])
        st = gpu_lib.peec_gb300_transient_lightning_batch(t.h, n, col(0), col(1), col(2), col(3), sz(4), sz(5), 0, 120,
                                                          dX, pn, nv, pe, ne, dpr)
        assert st == 0
        probes = np.zeros((120, n, nt))
        gpu_lib.peec_gb300_copy_to_host(probes.ctypes.data, dpr, probes.nbytes)
        gpu_lib.peec_gb300_copy_to_host(X.ctypes.data, dX, X.nbytes)
        for r, (s, I, V, p1) in enumerate(single):
            assert s == 0
            assert np.array_equal(probes[:, r, :], p1)
            assert np.array_equal(X[r, :ne], I) and np.array_equal(X[r, ne:], V)
        # more runs than a batch takes (8): refused before any array is read
        big = 9
        colb = lambda k: (C.c_double * big)(*([s[k] for s in srcs] * 6)[:big])
        szb = lambda k: (C.c_size_t * big)(*([s[k] for s in srcs] * 6)[:big])
        bad = gpu_lib.peec_gb300_transient_lightning_batch(t.h, big, colb(0), colb(1), colb(2), colb(3), szb(4),
                                                           szb(5), 0, 5, dX, None, 0, None, 0, None)
        assert bad == -1
    finally:
        t.close()
