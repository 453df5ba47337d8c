"""Matrix Market export (matrix_export.h): files byte-identical to the
reference's own writer, and values that read back exactly."""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import golden
from oracle import Oracle, reference_available
from peeeeeeeeeeeeeeeeeeec_gb300 import abi
from peeeeeeeeeeeeeeeeeeec_gb300.mesh import SynthMesh


def export_set(lib, directory, m, L, P_, PAT, Rd):
    ne, nv = L.shape[0], P_.shape[0]
    Lc, Pc, Tc, Rc = (np.ascontiguousarray(a, dtype=np.float64) for a in (L, P_, PAT, Rd))
    Lm = abi.InductanceMatrix(ne, Lc.ctypes.data_as(abi.c_double_p))
    Pm = abi.PotentialMatrix(nv, Pc.ctypes.data_as(abi.c_double_p))
    Tm = abi.Matrix(PAT.shape[0], PAT.shape[1], Tc.ctypes.data_as(abi.c_double_p))
    Rm = abi.ResistanceMatrix(ne, Rc.ctypes.data_as(abi.c_double_p))
    return lib.matrix_export_peec_set(directory.encode(), C.byref(m.mesh), C.byref(Lm), C.byref(Pm), C.byref(Tm),
                                      C.byref(Rm))


def case(name):
    f = golden(name)
    L, P_, edges = f["L"], f["P"], f["edges"]
    _, PAT, _ = Oracle().incidence_pat(P_, edges)
    Rd = np.linspace(1e-3, 2e-3, L.shape[0])
    return f, L, P_, PAT, Rd


@pytest.mark.skipif(not reference_available(), reason="reference library not built here")
@pytest.mark.parametrize("name", ["plate4", "box421"])
def test_files_identical_to_reference(tmp_path, name):
    from oracle import Reference
    f, L, P_, PAT, Rd = case(name)
    lib, ref = abi.load_gpu_lib(), Reference().lib
    with SynthMesh.from_arrays(f["xyz"], f["quads"]) as m:
        assert export_set(lib, str(tmp_path / "ours" / "set"), m, L, P_, PAT, Rd) == 0
        assert export_set(ref, str(tmp_path / "ref" / "set"), m, L, P_, PAT, Rd) == 0
    for fn in ("L.mtx", "A.mtx", "P.mtx", "PAT.mtx", "R.mtx"):
        a = (tmp_path / "ours" / "set" / fn).read_bytes()
        b = (tmp_path / "ref" / "set" / fn).read_bytes()
        assert a == b, fn


def test_dense_values_read_back_exactly(tmp_path):
    lib = abi.load_gpu_lib()
    rng = np.random.default_rng(2)
    X = rng.standard_normal((37, 53)) * 10.0 ** rng.uniform(-300, 300, (37, 53))
    X[0, 0], X[1, 2] = 0.0, -0.0
    path = str(tmp_path / "x.mtx")
    assert lib.matrix_export_dense_mtx(path.encode(), np.ascontiguousarray(X).ctypes.data_as(abi.c_double_p),
                                       37, 53) == 0
    lines = open(path).read().splitlines()
    assert lines[0] == "%%MatrixMarket matrix array real general" and lines[2] == "37 53"
    vals = np.array([float(v) for v in lines[3:]])
    assert np.array_equal(vals.reshape(53, 37).T, X)  # column-major


def test_bad_arguments(tmp_path):
    lib = abi.load_gpu_lib()
    one = np.ones(1)
    assert lib.matrix_export_dense_mtx(None, one.ctypes.data_as(abi.c_double_p), 1, 1) == -1
    assert lib.matrix_export_dense_mtx(str(tmp_path / "a.mtx").encode(), one.ctypes.data_as(abi.c_double_p),
                                       0, 1) == -1
    missing = str(tmp_path / "no" / "such" / "dir" / "a.mtx").encode()
    assert lib.matrix_export_dense_mtx(missing, one.ctypes.data_as(abi.c_double_p), 1, 1) == -1
