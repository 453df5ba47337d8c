"""GPU Lp / P assembly against the reference (golden fixtures made by the
reference itself) and the CPU oracle.  Tolerance: 1e-12 relative per entry
(the drop-in parity bar for Lp and P); exact zeros where the reference has
exact zeros (orthogonal edges)."""
import ctypes as C

import numpy as np
import pytest

from conftest import golden
from helpers import elem_rel_err, inductance, potential, quad_patch, rel_err
from peeeeeeeeeeeeeeeeeeec_gb300 import abi
from peeeeeeeeeeeeeeeeeeec_gb300.mesh import SynthMesh

pytestmark = pytest.mark.gpu
TOL = 1e-12


def test_quadrature_pairs_every_class(gpu_lib):
    q = golden("quadrature_cases")
    for k in range(len(q["K"])):
        a, b = quad_patch(q["a"][k]), quad_patch(q["b"][k])
        bb = a if q["same"][k] else b
        assert gpu_lib.quad_patch_classify_pair(C.byref(a), C.byref(bb), 0.5) == q["cls"][k]
        K = gpu_lib.quad_patch_kernel_1_over_r(C.byref(a), C.byref(bb), 4, 10, 12, 8, 0.5)
        assert abs(K - q["K"][k]) <= TOL * abs(q["K"][k]), (k, K, q["K"][k])


def test_pair_kernel_invalid_options_give_nan(gpu_lib):
    a = quad_patch([0, 0, 0, 1, 0, 0, 1, 1, 0, 0, 1, 0])
    assert np.isnan(gpu_lib.quad_patch_kernel_1_over_r(C.byref(a), C.byref(a), 7, 10, 12, 8, 0.5))
    assert np.isnan(gpu_lib.quad_patch_kernel_1_over_r(C.byref(a), C.byref(a), 4, 10, 12, 8, -1.0))
    assert np.isnan(gpu_lib.quad_patch_kernel_1_over_r(None, C.byref(a), 4, 10, 12, 8, 0.5))


@pytest.mark.parametrize("name", ["plate4", "plate8", "box421", "plate_msh"])
def test_matrices_match_reference(gpu_lib, name):
    g = golden(name)
    with SynthMesh.from_arrays(g["xyz"], g["quads"]) as m:
        s, L = inductance(gpu_lib, m)
        assert s == 0
        assert elem_rel_err(L, g["L"]) < TOL
        assert np.array_equal(L, L.T)
        s, P = potential(gpu_lib, m)
        assert s == 0
        assert elem_rel_err(P, g["P"]) < TOL
        assert np.array_equal(P, P.T)


@pytest.mark.parametrize("orders", [(4, 10, 12, 8), (2, 6, 6, 6), (6, 8, 16, 10), (3, 5, 4, 2)])
def test_other_orders_against_oracle(gpu_lib, oracle, orders):
    with SynthMesh.box(0.3, 0.2, 0.1, 3, 2, 1) as m:
        kw = dict(far_order=orders[0], near_order=orders[1], touching_order=orders[2], self_order=orders[3])
        s, L = inductance(gpu_lib, m, **kw)
        assert s == 0
        assert elem_rel_err(L, oracle.inductance(m, orders=orders)[1]) < TOL
        s, P = potential(gpu_lib, m, **kw)
        assert s == 0
        assert elem_rel_err(P, oracle.potential(m, orders=orders)[1]) < TOL


@pytest.mark.parametrize("near_factor", [0.0, 1.5])
def test_near_factor(gpu_lib, oracle, near_factor):
    with SynthMesh.plate(1.0, 0.5, 6, 3) as m:
        s, P = potential(gpu_lib, m, near_factor=near_factor)
        assert s == 0
        assert elem_rel_err(P, oracle.potential(m, near_factor=near_factor)[1]) < TOL


def test_config1_plate_16x16_against_oracle(gpu_lib, oracle):
    """The reference's CPU-runnable case: 1 m plate, 16 x 16 cells
    (Ne = 544, Nv = 289 in the reference's numbering)."""
    with SynthMesh.plate(1.0, 1.0, 16, 16) as m:
        assert (m.n_edges, m.n_nodes) == (544, 289)
        s, L = inductance(gpu_lib, m)
        assert s == 0 and elem_rel_err(L, oracle.inductance(m)[1]) < TOL
        s, P = potential(gpu_lib, m)
        assert s == 0 and elem_rel_err(P, oracle.potential(m)[1]) < TOL


def test_irregular_mesh_against_oracle(gpu_lib, oracle):
    """Seeded jittered plate with a bent row: skewed quads, mixed classes."""
    rng = np.random.default_rng(11)
    nx, ny = 7, 5
    xyz = np.array([(i / nx, j / ny, 0.0) for j in range(ny + 1) for i in range(nx + 1)])
    xyz[:, :2] += rng.uniform(-0.02, 0.02, (xyz.shape[0], 2))
    xyz[:, 2] = 0.1 * (xyz[:, 0] > 0.5) * (xyz[:, 0] - 0.5)
    quads = [(j * (nx + 1) + i, j * (nx + 1) + i + 1, (j + 1) * (nx + 1) + i + 1, (j + 1) * (nx + 1) + i)
             for j in range(ny) for i in range(nx)]
    with SynthMesh.from_arrays(xyz, np.array(quads)) as m:
        s, L = inductance(gpu_lib, m)
        assert s == 0
        Lo = oracle.inductance(m)[1]
        assert elem_rel_err(L, Lo) < TOL
        s, P = potential(gpu_lib, m)
        assert s == 0 and elem_rel_err(P, oracle.potential(m)[1]) < TOL


def test_single_entry_functions(gpu_lib, oracle):
    g = golden("box421")
    with SynthMesh.from_arrays(g["xyz"], g["quads"]) as m:
        lo = abi.InductanceOptions()
        gpu_lib.inductance_options_default(C.byref(lo), 1)
        po = abi.PotentialOptions()
        gpu_lib.potential_options_default(C.byref(po), 1)
        for a, b in [(0, 0), (3, 17), (17, 3), (5, 40), (55, 55)]:
            v = C.c_double(-1)
            assert gpu_lib.inductance_compute_pair(C.byref(m.mesh), C.byref(m.dual), a, b, C.byref(lo), C.byref(v)) == 0
            ref = g["L"][a, b]
            assert (v.value == 0.0) if ref == 0 else abs(v.value - ref) <= TOL * abs(ref)
        for i, j in [(0, 0), (2, 29), (29, 2), (10, 11)]:
            v = C.c_double(-1)
            assert gpu_lib.potential_compute_pair(C.byref(m.mesh), C.byref(m.dual), i, j, C.byref(po), C.byref(v)) == 0
            assert abs(v.value - g["P"][i, j]) <= TOL * abs(g["P"][i, j])
        v = C.c_double()
        assert gpu_lib.inductance_compute_pair(C.byref(m.mesh), C.byref(m.dual), 0, 56, C.byref(lo), C.byref(v)) == -1
        assert gpu_lib.potential_compute_pair(C.byref(m.mesh), C.byref(m.dual), 30, 0, C.byref(po), C.byref(v)) == -1


def test_errors_free_and_return_minus_one(gpu_lib):
    with SynthMesh.plate(1.0, 1.0, 3, 3) as m:
        s, L = inductance(gpu_lib, m, far_order=7)
        assert s == -1 and L is None
        s, P = potential(gpu_lib, m, near_factor=float("nan"))
        assert s == -1
        # a NaN coordinate makes every integral touching it non-finite
        m.mesh.xyz[0] = float("nan")
        lst = m.dual.node_patches[0]
        lst.patches[0].points[0] = float("nan")
        s, P = potential(gpu_lib, m)
        assert s == -1
        # an empty region makes its diagonal entry fail
    with SynthMesh.plate(1.0, 1.0, 3, 3) as m:
        m.dual.edge_patches[4].count = 0
        s, L = inductance(gpu_lib, m)
        assert s == -1


def test_device_assembly_matches_host_assembly(gpu_lib):
    with SynthMesh.plate(1.0, 1.0, 5, 4) as m:
        _, L = inductance(gpu_lib, m)
        n = m.n_edges
        d = gpu_lib.peec_gb300_device_alloc(n * n * 8)
        lo = abi.InductanceOptions()
        gpu_lib.inductance_options_default(C.byref(lo), 1)
        st = abi.PeecAssemblyStats()
        assert gpu_lib.peec_gb300_inductance_device(C.byref(m.mesh), C.byref(m.dual), C.byref(lo), d, C.byref(st)) == 0
        out = np.zeros((n, n))
        assert gpu_lib.peec_gb300_copy_to_host(out.ctypes.data, d, n * n * 8) == 0
        gpu_lib.peec_gb300_device_free(d)
        assert np.array_equal(out, L)
        assert st.near_pairs > 0 and st.potential_evaluations > 0


def test_repeatable_bitwise(gpu_lib):
    with SynthMesh.box(0.3, 0.2, 0.1, 3, 2, 1) as m:
        a = potential(gpu_lib, m)[1]
        b = potential(gpu_lib, m)[1]
        assert np.array_equal(a, b)


def test_potential_helpers(gpu_lib):
    g = golden("plate4")
    P = np.ascontiguousarray(g["P"])
    pm = abi.PotentialMatrix(P.shape[0], P.ctypes.data_as(abi.c_double_p))
    n = P.shape[0]
    F = np.zeros(n)
    assert gpu_lib.potential_build_self_capacitance(C.byref(pm), F.ctypes.data_as(abi.c_double_p)) == 0
    assert np.array_equal(F, 1.0 / np.diag(P))
    v = np.linspace(-1, 1, n)
    q = np.zeros(n)
    assert gpu_lib.potential_self_voltage_to_charge(C.byref(pm), v.ctypes.data_as(abi.c_double_p),
                                                    q.ctypes.data_as(abi.c_double_p)) == 0
    assert np.array_equal(q, v / np.diag(P))
    phi = np.zeros(n)
    assert gpu_lib.potential_self_voltage_to_full_potential(C.byref(pm), v.ctypes.data_as(abi.c_double_p),
                                                            phi.ctypes.data_as(abi.c_double_p)) == 0
    assert rel_err(phi, P @ (v / np.diag(P))) < 1e-14
    P2 = P.copy()
    P2[3, 3] = -1.0
    pm2 = abi.PotentialMatrix(n, P2.ctypes.data_as(abi.c_double_p))
    assert gpu_lib.potential_build_self_capacitance(C.byref(pm2), F.ctypes.data_as(abi.c_double_p)) == -1
    assert gpu_lib.potential_self_voltage_to_full_potential(C.byref(pm2), v.ctypes.data_as(abi.c_double_p),
                                                            phi.ctypes.data_as(abi.c_double_p)) == -1


def _assembly_stats(gpu_lib, m, which):
    n = m.n_edges if which == "L" else m.n_nodes
    d = gpu_lib.peec_gb300_device_alloc(n * n * 8)
    st = abi.PeecAssemblyStats()
    if which == "L":
        o = abi.InductanceOptions()
        gpu_lib.inductance_options_default(C.byref(o), 1)
        assert gpu_lib.peec_gb300_inductance_device(C.byref(m.mesh), C.byref(m.dual), C.byref(o), d, C.byref(st)) == 0
    else:
        o = abi.PotentialOptions()
        gpu_lib.potential_options_default(C.byref(o), 1)
        assert gpu_lib.peec_gb300_potential_device(C.byref(m.mesh), C.byref(m.dual), C.byref(o), d, C.byref(st)) == 0
    gpu_lib.peec_gb300_device_free(d)
    return st


def test_near_reuse_matches_individual_evaluation(gpu_lib):
    """Translated copies of a near pair share one evaluation unless one of its
    adaptive decisions is within 1e-6 of the threshold; the result agrees
    with evaluating every pair on its own."""
    with SynthMesh.box(0.4, 0.2, 0.1, 16, 8, 4) as m:
        prev = gpu_lib.peec_gb300_set_near_reuse(0)
        try:
            _, L0 = inductance(gpu_lib, m)
            _, P0 = potential(gpu_lib, m)
            st0 = _assembly_stats(gpu_lib, m, "P")
        finally:
            gpu_lib.peec_gb300_set_near_reuse(prev)
        gpu_lib.peec_gb300_set_near_reuse(1)
        _, L1 = inductance(gpu_lib, m)
        _, P1 = potential(gpu_lib, m)
        st1 = _assembly_stats(gpu_lib, m, "P")
        gpu_lib.peec_gb300_set_near_reuse(prev)
        assert elem_rel_err(L1, L0) < 1e-13
        assert elem_rel_err(P1, P0) < 1e-13
        assert st0.near_pairs_evaluated == st0.near_pairs
        assert st1.near_pairs == st0.near_pairs
        assert st1.near_pairs_evaluated * 10 < st1.near_pairs


def test_box_against_oracle_with_reuse(gpu_lib, oracle):
    """1.0 x 0.5 x 0.25 m PEC box at 5 cm (Ne = 1400, Nv = 702): every entry
    within 1e-12 of the oracle with near-pair reuse on (the default)."""
    with SynthMesh.box(1.0, 0.5, 0.25, 20, 10, 5) as m:
        s, L = inductance(gpu_lib, m)
        assert s == 0 and elem_rel_err(L, oracle.inductance(m)[1]) < TOL
        s, P = potential(gpu_lib, m)
        assert s == 0 and elem_rel_err(P, oracle.potential(m)[1]) < TOL


_NEAR_FORMS_PROBE = r"""
import sys
import numpy as np
sys.path.insert(0, {repo!r}); sys.path.insert(0, {tests!r})
from helpers import inductance, potential
from peeeeeeeeeeeeeeeeeeec_gb300 import abi
from peeeeeeeeeeeeeeeeeeec_gb300.mesh import SynthMesh
lib = abi.load_gpu_lib()
with SynthMesh.box(0.4, 0.2, 0.1, 8, 4, 2) as m:
    s1, L = inductance(lib, m)
    s2, P = potential(lib, m)
assert s1 == 0 and s2 == 0
np.savez(sys.argv[1], L=L, P=P)
"""


def test_level_and_depth_first_near_fields_agree(tmp_path):
    """The level-synchronous near field (default) and the depth-first warp
    form (PEEC_GB300_NEAR_LEVELS=0) walk the same refinement trees; they sum
    the accepted nodes in a different association (the reference's
    recursion vs a running sum), so entries agree to rounding."""
    import os
    import subprocess
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    code = _NEAR_FORMS_PROBE.format(repo=os.path.dirname(here), tests=here)
    res = {}
    for mode in ("1", "0"):
        env = dict(os.environ)
        env["PEEC_GB300_NEAR_LEVELS"] = mode
        path = str(tmp_path / ("near_%s.npz" % mode))
        r = subprocess.run([sys.executable, "-c", code, path], env=env, capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
        res[mode] = np.load(path)
    for key in ("L", "P"):
        a, b = res["1"][key], res["0"][key]
        assert np.array_equal(a == 0, b == 0)
        nz = b != 0
        assert np.max(np.abs(a[nz] - b[nz]) / np.abs(b[nz])) < 1e-13, key


def test_near_factor_zero_overlapping_plates(gpu_lib, oracle):
    """near_factor = 0 makes overlapping patches of two coincident-plane
    plates (shifted by a third of a cell, no shared vertex) FAR; the far
    rule must then keep the reference's R <= 0 skip (the FP64 form is used)
    and the entries match the oracle."""
    xyz, quads = [], []
    for dx in (0.0, 1.0 / 12.0):
        base = len(xyz)
        for j in range(5):
            for i in range(5):
                xyz.append((0.25 * i + dx, 0.25 * j, 0.0))
        for j in range(4):
            for i in range(4):
                v = base + j * 5 + i
                quads.append((v, v + 1, v + 6, v + 5))
    with SynthMesh.from_arrays(np.array(xyz), np.array(quads, dtype=np.int32)) as m:
        s, L = inductance(gpu_lib, m, near_factor=0.0)
        assert s == 0
        so, Lo = oracle.inductance(m, near_factor=0.0)
        assert so == 0
        assert elem_rel_err(L, Lo) < TOL
        s, P = potential(gpu_lib, m, near_factor=0.0)
        assert s == 0
        so, Po = oracle.potential(m, near_factor=0.0)
        assert so == 0
        assert elem_rel_err(P, Po) < TOL
