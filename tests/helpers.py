"""Call helpers shared by the tests: numpy in, numpy out, through the C ABI."""
import ctypes as C

import numpy as np

from peeeeeeeeeeeeeeeeeeec_gb300 import abi


def dp(a):
    return a.ctypes.data_as(abi.c_double_p)


def cp(a):
    return C.cast(a.ctypes.data, C.POINTER(abi.Complex))


def quad_patch(points):
    q = abi.QuadPatch()
    for t in range(12):
        q.points[t] = float(points[t])
    return q


def inductance(lib, m, **over):
    o = abi.InductanceOptions()
    lib.inductance_options_default(C.byref(o), 1)
    for k, v in over.items():
        setattr(o, k, v)
    L = abi.InductanceMatrix()
    s = lib.inductance_compute_matrix(C.byref(m.mesh), C.byref(m.dual), C.byref(o), C.byref(L))
    if s != 0:
        return s, None
    out = np.ctypeslib.as_array(L.data, shape=(L.n, L.n)).copy()
    lib.inductance_free(C.byref(L))
    return s, out


def potential(lib, m, **over):
    o = abi.PotentialOptions()
    lib.potential_options_default(C.byref(o), 1)
    for k, v in over.items():
        setattr(o, k, v)
    P = abi.PotentialMatrix()
    s = lib.potential_compute_matrix(C.byref(m.mesh), C.byref(m.dual), C.byref(o), C.byref(P))
    if s != 0:
        return s, None
    out = np.ctypeslib.as_array(P.data, shape=(P.n, P.n)).copy()
    lib.potential_free(C.byref(P))
    return s, out


class RealLU:
    def __init__(self, lib, a, tol=None):
        self.lib = lib
        self.a = np.ascontiguousarray(a, dtype=np.float64)
        self.n = self.a.shape[0]
        o = abi.LUOptions()
        lib.lu_options_default(C.byref(o), 1)
        if tol is not None:
            o.pivot_tolerance = tol
        self.f = abi.LUFactorization()
        self.status = lib.lu_factorize(dp(self.a), self.n, C.byref(o), C.byref(self.f))

    def factors(self):
        n = self.n
        return (np.ctypeslib.as_array(self.f.data, shape=(n, n)).copy(),
                np.ctypeslib.as_array(self.f.pivots, shape=(n,)).astype(np.int64))

    def solve(self, b):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros_like(b)
        s = self.lib.lu_solve(C.byref(self.f), dp(b), dp(x))
        return s, x

    def solve_multiple(self, B):
        B = np.ascontiguousarray(B, dtype=np.float64)
        X = np.zeros_like(B)
        s = self.lib.lu_solve_multiple(C.byref(self.f), dp(B), dp(X), B.shape[0], 1)
        return s, X

    def free(self):
        self.lib.lu_free(C.byref(self.f))


class ComplexLU:
    def __init__(self, lib, a, tol=None):
        self.lib = lib
        self.a = np.ascontiguousarray(a, dtype=np.complex128)
        self.n = self.a.shape[0]
        o = abi.ComplexLUOptions()
        lib.complex_lu_options_default(C.byref(o), 1)
        if tol is not None:
            o.pivot_tolerance = tol
        self.f = abi.ComplexLUFactorization()
        self.status = lib.complex_lu_factorize(cp(self.a), self.n, C.byref(o), C.byref(self.f))

    def factors(self):
        n = self.n
        raw = np.ctypeslib.as_array(C.cast(self.f.data, abi.c_double_p), shape=(2 * n * n,)).copy()
        return (raw.view(np.complex128).reshape(n, n),
                np.ctypeslib.as_array(self.f.pivots, shape=(n,)).astype(np.int64),
                np.ctypeslib.as_array(self.f.row_scale, shape=(n,)).copy(),
                np.ctypeslib.as_array(self.f.column_scale, shape=(n,)).copy())

    def solve(self, b):
        b = np.ascontiguousarray(b, dtype=np.complex128)
        x = np.zeros_like(b)
        s = self.lib.complex_lu_solve(C.byref(self.f), cp(b), cp(x))
        return s, x

    def solve_multiple(self, B):
        B = np.ascontiguousarray(B, dtype=np.complex128)
        X = np.zeros_like(B)
        s = self.lib.complex_lu_solve_multiple(C.byref(self.f), cp(B), cp(X), B.shape[0], 1)
        return s, X

    def free(self):
        self.lib.complex_lu_free(C.byref(self.f))


def rel_err(a, b):
    """max |a-b| / max |b| (matrix-relative)."""
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def elem_rel_err(a, b):
    """max over nonzero entries of b of |a-b| / |b|; zeros of b must be zeros of a."""
    nz = b != 0
    if np.any(a[~nz] != 0):
        return float("inf")
    return float(np.max(np.abs(a[nz] - b[nz]) / np.abs(b[nz]))) if nz.any() else 0.0


class DeviceBuffers:
    """Device copies of numpy arrays for the extension API; freed on exit."""

    def __init__(self, lib):
        self.lib, self.ptrs = lib, []

    def put(self, arr):
        arr = np.ascontiguousarray(arr)
        p = self.alloc(arr.nbytes)
        assert self.lib.peec_gb300_copy_to_device(p, arr.ctypes.data, arr.nbytes) == 0
        return p

    def alloc(self, nbytes):
        p = self.lib.peec_gb300_device_alloc(max(int(nbytes), 16))
        assert p, "device allocation failed"
        self.ptrs.append(p)
        return p

    def get(self, p, shape, dtype):
        out = np.zeros(shape, dtype=dtype)
        assert self.lib.peec_gb300_copy_to_host(out.ctypes.data, p, out.nbytes) == 0
        return out

    def __enter__(self):
        return self

    def __exit__(self, *a):
        for p in self.ptrs:
            self.lib.peec_gb300_device_free(p)
        self.ptrs = []
