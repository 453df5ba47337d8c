"""RCS radiation vectors on the GPU (rcs.c:701-1000, dual-patch quadrature)
against the reference's own outputs (golden fixtures) and the oracle.

Tolerance: the device sums the quadrature points over warp lanes and the
edges over lanes, the reference left to right, so entries agree to
rounding: |F_gpu - F_ref| <= 1e-12 max |F| per direction set."""
import ctypes as C

import numpy as np
import pytest

from conftest import golden
from peeeeeeeeeeeeeeeeeeec_gb300 import abi
from peeeeeeeeeeeeeeeeeeec_gb300.mesh import SynthMesh

pytestmark = pytest.mark.gpu


def gpu_rcs(lib, m, currents, k, dirs, order, stride=None):
    cur = np.atleast_2d(np.asarray(currents, dtype=np.complex128))
    n_rhs, ne = cur.shape
    stride = stride or ne
    buf = np.zeros((n_rhs, stride), dtype=np.complex128)
    buf[:, :ne] = cur
    d = lib.peec_gb300_device_alloc(buf.nbytes)
    lib.peec_gb300_copy_to_device(d, buf.ctypes.data, buf.nbytes)
    dirs = np.ascontiguousarray(dirs, dtype=np.float64).reshape(-1, 3)
    out = np.zeros((dirs.shape[0], n_rhs, 3), dtype=np.complex128)
    s = lib.peec_gb300_rcs_radiation_device(C.byref(m.mesh), C.byref(m.dual), d, n_rhs, stride, k,
                                            dirs.ctypes.data_as(abi.c_double_p), dirs.shape[0], order,
                                            out.ctypes.data)
    lib.peec_gb300_device_free(d)
    return s, out


@pytest.mark.parametrize("name", ["plate4", "box421"])
def test_against_reference_fixtures(gpu_lib, name):
    f, g = golden(name), golden("rcs_" + name)
    with SynthMesh.from_arrays(f["xyz"], f["quads"]) as m:
        for k in g["k"]:
            for order in g["orders"]:
                s, F = gpu_rcs(gpu_lib, m, g["current"], float(k), g["directions"], int(order))
                assert s == 0
                ref = g["F_%g_%d" % (k, order)]
                assert np.max(np.abs(F[:, 0, :] - ref)) <= 1e-12 * np.max(np.abs(ref)), (k, order)


def test_many_solutions_and_directions(gpu_lib, oracle):
    """Several solutions with a padded stride and a bistatic sweep equal the
    oracle's one-at-a-time results."""
    rng = np.random.default_rng(4)
    with SynthMesh.box(2.0, 1.0, 0.5, 8, 4, 2) as m:
        ne = m.n_edges
        cur = rng.standard_normal((3, ne)) + 1j * rng.standard_normal((3, ne))
        ph = np.radians(np.arange(0, 360, 15))
        dirs = np.stack([np.cos(ph), np.sin(ph), np.zeros_like(ph)], 1)
        k = 2 * np.pi * 100e6 / 299792458.0
        s, F = gpu_rcs(gpu_lib, m, cur, k, dirs, 6, stride=ne + 7)
        assert s == 0
        for q in range(3):
            so, Fo = oracle.rcs_radiation(m, cur[q], k, dirs, 6)
            assert so == 0
            assert np.max(np.abs(F[:, q, :] - Fo)) <= 1e-12 * np.max(np.abs(Fo))


def test_invalid_inputs(gpu_lib):
    with SynthMesh.plate(1.0, 1.0, 2, 2) as m:
        cur = np.ones(m.n_edges)
        assert gpu_rcs(gpu_lib, m, cur, 0.0, [[0, 0, 1]], 6)[0] == -1
        assert gpu_rcs(gpu_lib, m, cur, 1.0, [[0, 0, 1]], 7)[0] == -1
        assert gpu_rcs(gpu_lib, m, cur, 1.0, [[0, 0, np.nan]], 6)[0] == -1
        d = gpu_lib.peec_gb300_device_alloc(16 * m.n_edges)
        out = np.zeros(3, dtype=np.complex128)
        dirs = np.array([0.0, 0.0, 1.0])
        assert gpu_lib.peec_gb300_rcs_radiation_device(C.byref(m.mesh), C.byref(m.dual), d, 1, m.n_edges - 1,
                                                       1.0, dirs.ctypes.data_as(abi.c_double_p), 1, 6,
                                                       out.ctypes.data) == -1
        gpu_lib.peec_gb300_device_free(d)
