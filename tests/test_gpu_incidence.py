"""Incidence matrix and its products with P (incidence.h) on the GPU against
the reference's own outputs (golden fixtures) and the oracle, bit for bit:
every entry is the reference's expression in the same order."""
import ctypes as C

import numpy as np
import pytest

from conftest import golden
from oracle import incidence_products
from peeeeeeeeeeeeeeeeeeec_gb300 import abi
from peeeeeeeeeeeeeeeeeeec_gb300.mesh import SynthMesh

pytestmark = pytest.mark.gpu


def dev_put(lib, arr):
    p = lib.peec_gb300_device_alloc(max(arr.nbytes, 8))
    assert lib.peec_gb300_copy_to_device(p, arr.ctypes.data, arr.nbytes) == 0
    return p


def dev_get(lib, p, shape):
    out = np.zeros(shape)
    lib.peec_gb300_copy_to_host(out.ctypes.data, p, out.nbytes)
    return out


@pytest.mark.parametrize("name", ["plate4", "box421"])
def test_drop_in_matches_reference_fixtures(gpu_lib, name):
    f, g = golden(name), golden("incidence_" + name)
    with SynthMesh.from_arrays(f["xyz"], f["quads"]) as m:
        out = incidence_products(gpu_lib, m.mesh, f["P"])
        A = abi.IncidenceMatrix()
        assert gpu_lib.incidence_build(C.byref(m.mesh), C.byref(A)) == 0
        assert gpu_lib.incidence_check_row_sum(C.byref(A)) == 0.0
        gpu_lib.incidence_free(C.byref(A))
    for k in ("A", "APAT", "PAT", "AS"):
        assert np.array_equal(out[k], g[k]), k


def random_system(nx=12, ny=6, nz=3, seed=5):
    rng = np.random.default_rng(seed)
    with SynthMesh.box(1.2, 0.6, 0.3, nx, ny, nz) as m:
        edges = np.ascontiguousarray(m.edges())
        nv = m.n_nodes
    X = rng.standard_normal((nv, nv))
    return X @ X.T + nv * np.eye(nv), edges


def test_device_forms_match_oracle(gpu_lib, oracle):
    P_, edges = random_system()
    nv, ne = P_.shape[0], edges.shape[0]
    dP, dE = dev_put(gpu_lib, P_), dev_put(gpu_lib, edges)
    dO = gpu_lib.peec_gb300_device_alloc(max(ne * ne, nv * ne) * 8)
    bad = C.c_longlong()
    assert gpu_lib.peec_gb300_pat_device(dP, dE, nv, ne, dO, C.byref(bad)) == 0 and bad.value == -1
    assert np.array_equal(dev_get(gpu_lib, dO, (nv, ne)), oracle.incidence_pat(P_, edges)[1])
    assert gpu_lib.peec_gb300_apat_device(dP, dE, nv, ne, dO) == 0
    K = dev_get(gpu_lib, dO, (ne, ne))
    assert np.array_equal(K, oracle.incidence_apat(P_, edges)) and np.array_equal(K, K.T)
    assert gpu_lib.peec_gb300_as_device(dP, dE, nv, ne, dO) == 0
    assert np.array_equal(dev_get(gpu_lib, dO, (ne, nv)), oracle.incidence_as(P_, edges)[1])
    for p in (dP, dE, dO):
        gpu_lib.peec_gb300_device_free(p)


def test_failures_match_the_reference_rules(gpu_lib, oracle):
    P_, edges = random_system(4, 3, 2)
    nv, ne = P_.shape[0], edges.shape[0]
    # a non-finite P entry: P A^T fails at the first bad entry in row-major order
    Pn = P_.copy()
    Pn[3, edges[5, 1]] = np.nan
    s, _, first = oracle.incidence_pat(Pn, edges)
    dP, dE = dev_put(gpu_lib, Pn), dev_put(gpu_lib, edges)
    dO = gpu_lib.peec_gb300_device_alloc(max(ne * ne, nv * ne) * 8)
    bad = C.c_longlong()
    assert s == -1 and gpu_lib.peec_gb300_pat_device(dP, dE, nv, ne, dO, C.byref(bad)) == 1 and bad.value == first
    # a non-positive diagonal: A S fails
    Pd = P_.copy()
    Pd[2, 2] = 0.0
    gpu_lib.peec_gb300_copy_to_device(dP, Pd.ctypes.data, Pd.nbytes)
    assert gpu_lib.peec_gb300_as_device(dP, dE, nv, ne, dO) == 1
    # an edge out of range: A P A^T refuses it
    eb = edges.copy()
    eb[1, 0] = nv
    gpu_lib.peec_gb300_copy_to_device(dE, eb.ctypes.data, eb.nbytes)
    assert gpu_lib.peec_gb300_apat_device(dP, dE, nv, ne, dO) == -1
    for p in (dP, dE, dO):
        gpu_lib.peec_gb300_device_free(p)
    # drop-in: an incidence row with another value fails A S; P A^T frees its output
    with SynthMesh.box(0.4, 0.3, 0.2, 4, 3, 2) as m:
        A = abi.IncidenceMatrix()
        assert gpu_lib.incidence_build(C.byref(m.mesh), C.byref(A)) == 0
        Pm = abi.PotentialMatrix(nv, np.ascontiguousarray(P_).ctypes.data_as(abi.c_double_p))
        A.data[3] = 0.5 if A.data[3] == 0.0 else A.data[3]
        A.data[A.cols + 1] = 0.5 if A.data[A.cols + 1] == 0.0 else 2.0
        M = abi.Matrix()
        assert gpu_lib.incidence_build_AS(C.byref(A), C.byref(Pm), C.byref(M), 1) == -1
        assert not M.data and M.rows == 0
        Pn_m = abi.PotentialMatrix(nv, np.ascontiguousarray(Pn).ctypes.data_as(abi.c_double_p))
        assert gpu_lib.incidence_build_PAT(C.byref(m.mesh), C.byref(Pn_m), C.byref(M), 1) == -1
        assert not M.data
        assert gpu_lib.incidence_build_PAT(C.byref(m.mesh), C.byref(Pm), C.byref(M), 0) == -1
        gpu_lib.incidence_free(C.byref(A))
