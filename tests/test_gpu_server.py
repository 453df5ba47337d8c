"""Serving loop (peec_gb300_server_*): every result is the same alone and in
the mix.

Each request is solved once alone (a fresh one-worker server, nothing else on
the GPU) and once inside a mix of requests on several meshes, frequencies and
both precisions that four workers run concurrently on their own streams,
sharing the device-resident Lp / P cache.  The kernels are deterministic
(integer atomics only), so the tolerance stated here is zero: the mixed-in
result must be bit-identical to the alone result.  A tight memory budget
(admission one request at a time, cache evictions) must not change results
either, and every solve meets the 1e-10 backward-error gate, checked on the
host against the MNA matrix."""
import ctypes as C

import numpy as np
import pytest

from peeeeeeeeeeeeeeeeeeec_gb300 import abi
from peeeeeeeeeeeeeeeeeeec_gb300.mesh import SynthMesh
from peeeeeeeeeeeeeeeeeeec_gb300.server import Server

pytestmark = pytest.mark.gpu

GB = 1 << 30


@pytest.fixture(scope="module")
def meshes():
    ms = [SynthMesh.box(0.4, 0.2, 0.1, 8, 4, 2), SynthMesh.plate(0.5, 0.5, 10, 10),
          SynthMesh.box(0.3, 0.3, 0.2, 6, 6, 4)]
    yield ms
    for m in ms:
        m.close()


def requests():
    rng = np.random.default_rng(11)
    out = []
    for i in range(12):
        mesh = i % 3
        q = int(rng.integers(1, 4))
        th = rng.uniform(0, np.pi, q)
        ph = rng.uniform(0, 2 * np.pi, q)
        k = np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], 1)
        e = np.cross(k, [0.3, 0.5, 0.81])
        e /= np.linalg.norm(e, axis=1)[:, None]
        out.append(dict(mesh=mesh, frequency=float(10 ** rng.uniform(6, 8)), k_hat=k, e_hat=e,
                        mixed=bool(i % 2)))
    return out


def run(meshes, reqs, budget, workers, one_at_a_time=False):
    res = []
    with Server(budget, workers) as s:
        if one_at_a_time:
            for r in reqs:
                t = s.submit(meshes[r["mesh"]], r["mesh"], r["frequency"], r["k_hat"], r["e_hat"],
                             mixed=r["mixed"])
                res.append(s.wait(t))
        else:
            ts = [s.submit(meshes[r["mesh"]], r["mesh"], r["frequency"], r["k_hat"], r["e_hat"],
                           mixed=r["mixed"]) for r in reqs]
            res = [s.wait(t) for t in ts]
    return res


def host_mna(lib, m, freq):
    ne, nv = m.n_edges, m.n_nodes
    n = ne + nv
    lo = abi.InductanceOptions()
    lib.inductance_options_default(C.byref(lo), 1)
    po = abi.PotentialOptions()
    lib.potential_options_default(C.byref(po), 1)
    dL = lib.peec_gb300_device_alloc(ne * ne * 8)
    dP = lib.peec_gb300_device_alloc(nv * nv * 8)
    dZ = lib.peec_gb300_device_alloc(n * n * 16)
    edges = np.ascontiguousarray(m.edges())
    dE = lib.peec_gb300_device_alloc(edges.nbytes)
    try:
        assert lib.peec_gb300_copy_to_device(dE, edges.ctypes.data, edges.nbytes) == 0
        assert lib.peec_gb300_inductance_device(C.byref(m.mesh), C.byref(m.dual), C.byref(lo), dL, None) == 0
        assert lib.peec_gb300_potential_device(C.byref(m.mesh), C.byref(m.dual), C.byref(po), dP, None) == 0
        assert lib.peec_gb300_harmonic_build_device(dL, dP, dE, None, ne, nv, freq, dZ) == 0
        Z = np.zeros((n, n), dtype=np.complex128)
        assert lib.peec_gb300_copy_to_host(Z.ctypes.data, dZ, Z.nbytes) == 0
        return Z
    finally:
        for p in (dL, dP, dZ, dE):
            lib.peec_gb300_device_free(p)


def plane_wave_rhs(m, freq, k, e):
    """[-U_e; 0]: the incident field at each edge centre along the edge vector
    times sinc(k0 k.l / 2)."""
    k0 = 2 * np.pi * freq / 299792458.0
    ctr = m.array("edge_centers", (m.n_edges, 3))
    vec = m.array("edge_vectors", (m.n_edges, 3))
    h = 0.5 * k0 * (vec @ k)
    sinc = np.where(np.abs(h) < 1e-8, 1 - h * h / 6, np.sin(h) / np.where(h == 0, 1, h))
    u = (vec @ e) * np.exp(-1j * k0 * (ctr @ k)) * sinc
    return np.concatenate([-u, np.zeros(m.n_nodes)])


def test_same_alone_and_in_the_mix(gpu_lib, meshes):
    reqs = requests()
    alone = [run(meshes, [r], 8 * GB, 1)[0] for r in reqs]
    mix = run(meshes, reqs, 8 * GB, 4)
    for r, (xa, ra), (xm, rm) in zip(reqs, alone, mix):
        assert ra["status"] == 0 and rm["status"] == 0, (ra, rm)
        assert ra["backward_error"] <= 1e-10 and rm["backward_error"] <= 1e-10
        assert np.array_equal(xa, xm), r
        assert rm["t_submit"] <= rm["t_start"] <= rm["t_end"]
    # the mix really overlapped: some requests were on the GPU at the same time
    iv = sorted((rm["t_start"], rm["t_end"]) for _, rm in mix)
    assert any(iv[i + 1][0] < iv[i][1] for i in range(len(iv) - 1))


def test_tight_budget_admits_one_at_a_time(gpu_lib, meshes):
    reqs = requests()[:6]
    ref = run(meshes, reqs, 8 * GB, 1, one_at_a_time=True)
    # a budget that holds one request (its estimate is 64 MiB of library
    # scratch + 32 N^2 bytes of matrices + ~10 kB per unknown of splits and
    # vectors) and one cached mesh, never two requests: admission waits,
    # meshes are evicted and re-assembled
    n = max(m.n_edges + m.n_nodes for m in meshes)
    budget = (64 << 20) + 48 * n * n + 10000 * n + (1 << 20)
    tight = run(meshes, reqs, budget, 4)
    for (xa, _), (xb, rb) in zip(ref, tight):
        assert rb["status"] == 0
        assert np.array_equal(xa, xb)


def test_results_meet_the_backward_error_gate(gpu_lib, meshes):
    reqs = [r for r in requests()[:4]]
    res = run(meshes, reqs, 8 * GB, 2)
    for r, (x, info) in zip(reqs, res):
        m = meshes[r["mesh"]]
        Z = host_mna(gpu_lib, m, r["frequency"])
        for q in range(x.shape[0]):
            b = plane_wave_rhs(m, r["frequency"], r["k_hat"][q], r["e_hat"][q])
            res_ = Z @ x[q] - b
            be = np.max(np.abs(res_) / (np.abs(Z) @ np.abs(x[q]) + np.abs(b)))
            assert be <= 1e-10, (r, be, info)


def test_refused_requests(gpu_lib, meshes):
    with Server(64 << 20, 1) as s:  # smaller than any request
        with pytest.raises(ValueError, match="budget"):
            s.submit(meshes[0], 0, 1e6, [0, 0, 1], [1, 0, 0])
    with Server(GB, 1) as s:
        with pytest.raises(ValueError, match="invalid"):
            s.submit(meshes[0], 0, -1.0, [0, 0, 1], [1, 0, 0])


def test_transient_requests_alone_and_in_the_mix(gpu_lib, meshes):
    """Lightning runs through the server (the factorised transient system
    cached per mesh, scheme and dt) equal a direct device run bit for bit,
    alone and mixed with harmonic requests."""
    from test_gpu_transient import DeviceTransient
    from helpers import inductance, potential
    m = meshes[0]
    src = (102900.0, 1500.0, 1.0e6, 0.0, 3, 20)
    pn, pe = [0, 3, 20], [1, 5]
    s1, L = inductance(gpu_lib, m)
    s2, P = potential(gpu_lib, m)
    direct = DeviceTransient(gpu_lib, L, P, m.edges(), None, 2, 1e-7)
    try:
        assert direct.status == 0
        s, I, V, probes = direct.run(src, 300, probe_nodes=pn, probe_edges=pe)
        assert s == 0
    finally:
        direct.close()
    with Server(8 * GB, 1) as srv:
        (pa, Ia, Va), ra = srv.wait(srv.submit_transient(m, 0, 300, src, probe_nodes=pn, probe_edges=pe))
    assert ra["status"] == 0 and ra["iterations"] == 300
    assert np.array_equal(pa, probes) and np.array_equal(Ia, I) and np.array_equal(Va, V)
    reqs = requests()[:6]
    with Server(8 * GB, 4) as srv:
        tt = [srv.submit_transient(m, 0, 300, src, probe_nodes=pn, probe_edges=pe) for _ in range(2)]
        th = [srv.submit(meshes[r["mesh"]], r["mesh"], r["frequency"], r["k_hat"], r["e_hat"], mixed=r["mixed"])
              for r in reqs]
        outs = [srv.wait(t) for t in tt]
        hs = [srv.wait(t) for t in th]
    for (pb, Ib, Vb), rb in outs:
        assert rb["status"] == 0
        assert np.array_equal(pb, probes) and np.array_equal(Ib, I)
    assert all(h[1]["status"] == 0 for h in hs)


def test_queued_transient_runs_are_batched(gpu_lib, meshes):
    """Lightning runs that queue up behind other work on the same system are
    stepped together by one worker; each still equals its own direct run."""
    from test_gpu_transient import DeviceTransient
    from helpers import inductance, potential
    m = meshes[0]
    srcs = [(102900.0, 1500.0, 1.0e6, 0.0, 3, 20), (105139.0, 2127.18, 246066.0, 0.0, 7, 0),
            (6.0e4, 1800.0, 4.0e5, 1e-7, 12, 25)]
    pn, pe = [0, 3, 20], [1, 5]
    s1, L = inductance(gpu_lib, m)
    s2, P = potential(gpu_lib, m)
    direct = DeviceTransient(gpu_lib, L, P, m.edges(), None, 2, 1e-7)
    try:
        ref = [direct.run(src, 200, probe_nodes=pn, probe_edges=pe) for src in srcs]
    finally:
        direct.close()
    r = requests()[0]
    with Server(8 * GB, 1) as srv:
        busy = srv.submit(meshes[r["mesh"]], r["mesh"], r["frequency"], r["k_hat"], r["e_hat"], mixed=r["mixed"])
        tt = [srv.submit_transient(m, 0, 200, src, probe_nodes=pn, probe_edges=pe) for src in srcs]
        outs = [srv.wait(t) for t in tt]
        srv.wait(busy)
    starts = {o[1]["t_start"] for o in outs}
    assert len(starts) <= 2  # the queued runs started together with the first or right after it
    for (pb, Ib, Vb), rb in outs:
        assert rb["status"] == 0
    for ((pb, Ib, Vb), rb), (s, I, V, p) in zip(outs, ref):
        assert np.array_equal(pb, p) and np.array_equal(Ib, I) and np.array_equal(Vb, V)


def test_lightning_runs_join_a_running_batch(gpu_lib, meshes):
    """A lightning run submitted while another run on the same system is
    stepping joins that batch at a chunk boundary (one worker: it starts
    before the first run ends), with its own probe lists, and both equal
    their direct runs bit for bit."""
    import time
    from test_gpu_transient import DeviceTransient
    from helpers import inductance, potential
    m = meshes[0]
    runs = [((102900.0, 1500.0, 1.0e6, 0.0, 3, 20), 20000, [0, 3, 20], [1, 5]),
            ((6.0e4, 1800.0, 4.0e5, 1e-7, 12, 25), 700, [12], [2, 7, 9])]
    s1, L = inductance(gpu_lib, m)
    s2, P = potential(gpu_lib, m)
    direct = DeviceTransient(gpu_lib, L, P, m.edges(), None, 2, 1e-7)
    try:
        ref = [direct.run(src, n, probe_nodes=pn, probe_edges=pe) for src, n, pn, pe in runs]
    finally:
        direct.close()
    with Server(8 * GB, 1) as srv:
        src, n, pn, pe = runs[0]
        ta = srv.submit_transient(m, 0, n, src, probe_nodes=pn, probe_edges=pe)
        time.sleep(0.05)
        src, n, pn, pe = runs[1]
        tb = srv.submit_transient(m, 0, n, src, probe_nodes=pn, probe_edges=pe)
        (pa, Ia, Va), ra = srv.wait(ta)
        (pb, Ib, Vb), rb = srv.wait(tb)
    assert ra["status"] == 0 and rb["status"] == 0
    assert rb["t_start"] < ra["t_end"]  # it joined, not queued behind the first run
    for (p, I, V), (s, Ir, Vr, pr) in zip(((pa, Ia, Va), (pb, Ib, Vb)), ref):
        assert s == 0
        assert np.array_equal(p, pr) and np.array_equal(I, Ir) and np.array_equal(V, Vr)
