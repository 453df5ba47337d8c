"""Python handle on the library's serving loop (peec_gb300_server_* in
include/peec_gb300.h).

A Server owns worker threads inside the library; a request is one harmonic
solve (mesh, frequency, plane-wave right-hand sides, plain FP64 LU or the
mixed-precision solve) or one lightning transient run.  The handle keeps
every array a pending request points at alive until it has been waited for.
"""
import ctypes as C

import numpy as np

from . import abi


class Server:
    def __init__(self, hbm_budget_bytes, workers=4, lib=None):
        self.lib = lib or abi.load_gpu_lib()
        self.handle = self.lib.peec_gb300_server_create(int(hbm_budget_bytes), int(workers))
        if not self.handle:
            raise RuntimeError("peec_gb300_server_create failed: %s" % self.lib.peec_gb300_last_error())
        self._pending = {}

    def submit(self, mesh, key, frequency, k_hat, e_hat, mixed=False, tolerance=0.0):
        """mesh: a SynthMesh (kept alive until wait); k_hat, e_hat: (nrhs, 3)."""
        k_hat = np.ascontiguousarray(np.atleast_2d(k_hat), dtype=np.float64)
        e_hat = np.ascontiguousarray(np.atleast_2d(e_hat), dtype=np.float64)
        assert k_hat.shape == e_hat.shape and k_hat.shape[1] == 3
        nrhs = k_hat.shape[0]
        x = np.zeros((nrhs, mesh.n_edges + mesh.n_nodes), dtype=np.complex128)
        req = abi.PeecHarmonicRequest(
            mesh=C.pointer(mesh.mesh), dual=C.pointer(mesh.dual), mesh_key=int(key),
            frequency=float(frequency), nrhs=nrhs,
            k_hat=k_hat.ctypes.data_as(abi.c_double_p), e_hat=e_hat.ctypes.data_as(abi.c_double_p),
            mixed=1 if mixed else 0, tolerance=float(tolerance),
            x=x.ctypes.data_as(C.POINTER(abi.Complex)))
        t = self.lib.peec_gb300_server_submit(self.handle, C.byref(req))
        if t < 0:
            raise ValueError("request refused: %s" % self.lib.peec_gb300_last_error().decode())
        self._pending[t] = (x, mesh, req, k_hat, e_hat)
        return t

    def submit_transient(self, mesh, key, n_steps, source, scheme=2, dt=1e-7, probe_nodes=(), probe_edges=()):
        """Lightning run on a PEC mesh; source = (K, alpha, beta, delay,
        strike_node, return_node).  wait() returns ((probes [n_steps][np],
        I, V), result dict)."""
        pn = np.ascontiguousarray(probe_nodes, dtype=np.int32)
        pe = np.ascontiguousarray(probe_edges, dtype=np.int32)
        probes = np.zeros((n_steps, len(pn) + len(pe)))
        I, V = np.zeros(mesh.n_edges), np.zeros(mesh.n_nodes)
        K, alpha, beta, delay, strike, ret = source
        req = abi.PeecTransientRequest(
            mesh=C.pointer(mesh.mesh), dual=C.pointer(mesh.dual), mesh_key=int(key), scheme=int(scheme),
            dt=float(dt), n_steps=int(n_steps), K=float(K), alpha=float(alpha), beta=float(beta),
            delay=float(delay), strike_node=int(strike), return_node=int(ret),
            probe_nodes=pn.ctypes.data_as(C.POINTER(C.c_int)), n_probe_nodes=len(pn),
            probe_edges=pe.ctypes.data_as(C.POINTER(C.c_int)), n_probe_edges=len(pe),
            probes=probes.ctypes.data_as(abi.c_double_p), I=I.ctypes.data_as(abi.c_double_p),
            V=V.ctypes.data_as(abi.c_double_p))
        t = self.lib.peec_gb300_server_submit_transient(self.handle, C.byref(req))
        if t < 0:
            raise ValueError("request refused: %s" % self.lib.peec_gb300_last_error().decode())
        self._pending[t] = ((probes, I, V), mesh, req, pn, pe)
        return t

    def wait(self, ticket):
        """Returns (x [nrhs][Ne+Nv] complex128, result dict) for a harmonic
        request, ((probes, I, V), result dict) for a transient one."""
        r = abi.PeecRequestResult()
        if self.lib.peec_gb300_server_wait(self.handle, ticket, C.byref(r)) != 0:
            raise KeyError(ticket)
        x = self._pending.pop(ticket)[0]
        return x, {"status": r.status, "iterations": r.iterations, "fallback": r.fallback,
                   "backward_error": r.backward_error, "t_submit": r.t_submit,
                   "t_start": r.t_start, "t_end": r.t_end}

    def clock(self):
        return self.lib.peec_gb300_server_clock(self.handle)

    def close(self):
        if self.handle:
            for t in list(self._pending):
                self.wait(t)
            self.lib.peec_gb300_server_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
