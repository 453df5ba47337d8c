"""The allocation-free LU entry point (peec_gb300_lu_factor_device_noalloc).

It exists for callers that cannot let the library allocate device memory --
applications that own all GPU memory through their own pool or hard budget,
and solver loops that must not let cudaMalloc / cudaFree synchronise the
device -- and keeps its scratch in a fixed static device array instead.  This
file checks, through the C ABI, that two calls in a row give the same factor,
pivots, permutation and scale as the allocating entry point
peec_gb300_lu_factor_device, and that sizes above its limit are refused.  It
is collected last so a failure here cannot hide another test's result.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import rel_err

pytestmark = pytest.mark.gpu


def _factor(lib, entry, a):
    n = a.shape[0]
    a = np.ascontiguousarray(a, dtype=np.float64)
    d_a = lib.peec_gb300_device_alloc(n * n * 8)
    d_piv = lib.peec_gb300_device_alloc(n * 8)
    d_perm = lib.peec_gb300_device_alloc(n * 4)
    try:
        assert lib.peec_gb300_copy_to_device(d_a, a.ctypes.data, a.nbytes) == 0
        scale, col = C.c_double(), C.c_int()
        status = entry(d_a, n, 1e-14, d_piv, d_perm, C.byref(scale), C.byref(col))
        assert lib.peec_gb300_synchronize() == 0
        lu = np.zeros((n, n))
        piv = np.zeros(n, dtype=np.int64)
        perm = np.zeros(n, dtype=np.int32)
        assert lib.peec_gb300_copy_to_host(lu.ctypes.data, d_a, lu.nbytes) == 0
        assert lib.peec_gb300_copy_to_host(piv.ctypes.data, d_piv, piv.nbytes) == 0
        assert lib.peec_gb300_copy_to_host(perm.ctypes.data, d_perm, perm.nbytes) == 0
        return status, lu, piv, perm, scale.value
    finally:
        for p in (d_a, d_piv, d_perm):
            lib.peec_gb300_device_free(p)


def test_no_alloc_matches_allocating_entry_point(gpu_lib):
    rng = np.random.default_rng(2024)
    # 300: cooperative multi-CTA panels; 97: single-CTA panels
    mats = [rng.standard_normal((300, 300)), rng.standard_normal((97, 97))]
    mats[1][:, 5] *= 1e-3  # pivots away from the diagonal
    expected = [_factor(gpu_lib, gpu_lib.peec_gb300_lu_factor_device, a) for a in mats]
    got = [_factor(gpu_lib, gpu_lib.peec_gb300_lu_factor_device_noalloc, a) for a in mats]  # two calls in a row
    for (s0, lu0, piv0, perm0, sc0), (s1, lu1, piv1, perm1, sc1) in zip(expected, got):
        assert s0 == 0 and s1 == 0
        assert np.array_equal(piv1, piv0)
        assert np.array_equal(perm1, perm0)
        assert sc1 == sc0
        assert rel_err(lu1, lu0) < 1e-12


def test_no_alloc_rejects_sizes_beyond_its_limit(gpu_lib):
    dummy = C.c_void_p(1)  # never dereferenced: the size check comes first
    s = gpu_lib.peec_gb300_lu_factor_device_noalloc(dummy, 50001, 1e-14, dummy, dummy, None, None)
    assert s == -1
    assert b"exceeds the maximum" in gpu_lib.peec_gb300_last_error()
