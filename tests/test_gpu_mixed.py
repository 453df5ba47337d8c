"""Mixed-precision complex solve (FP32 LU with a split-BF16x3 tcgen05 trailing
update, FP64 iterative refinement) against the FP64 path.

Gate: componentwise backward error <= 1e-10 (the harmonic driver's
acceptance test), and the refined solution agrees with the plain FP64 LU
solution to the accuracy that backward error allows."""
import ctypes as C

import numpy as np
import pytest

from helpers import ComplexLU, rel_err
from peeeeeeeeeeeeeeeeeeec_gb300 import abi
from peeeeeeeeeeeeeeeeeeec_gb300.mesh import SynthMesh

pytestmark = pytest.mark.gpu


def dev_put(lib, arr):
    p = lib.peec_gb300_device_alloc(arr.nbytes)
    assert lib.peec_gb300_copy_to_device(p, arr.ctypes.data, arr.nbytes) == 0
    return p


def mixed_solve(lib, Z, B, tol=1e-10, max_iter=30):
    Z = np.ascontiguousarray(Z, dtype=np.complex128)
    B = np.ascontiguousarray(B, dtype=np.complex128)
    n = Z.shape[0]
    nrhs = 1 if B.ndim == 1 else B.shape[0]
    dZ, dB = dev_put(lib, Z), dev_put(lib, B)
    dX = lib.peec_gb300_device_alloc(B.nbytes)
    be, it = C.c_double(), C.c_int()
    s = lib.peec_gb300_complex_solve_mixed_device(dZ, n, dB, dX, nrhs, tol, max_iter, C.byref(be), C.byref(it))
    X = np.zeros_like(B)
    lib.peec_gb300_copy_to_host(X.ctypes.data, dX, X.nbytes)
    Zback = np.zeros_like(Z)
    lib.peec_gb300_copy_to_host(Zback.ctypes.data, dZ, Z.nbytes)
    for p in (dZ, dB, dX):
        lib.peec_gb300_device_free(p)
    assert np.array_equal(Zback, Z)  # the input matrix is not modified
    return s, X, be.value, it.value


def backward_error(Z, x, b):
    r = Z @ x - b
    return np.max(np.abs(r) / (np.abs(Z) @ np.abs(x) + np.abs(b)))


@pytest.mark.parametrize("n", [64, 300, 513])
def test_random_systems(gpu_lib, n):
    rng = np.random.default_rng(n)
    Z = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)) + n ** 0.5 * np.eye(n)
    Z *= np.logspace(-4, 4, n)[:, None]  # badly scaled rows: equilibration matters
    b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    s, x, be, it = mixed_solve(gpu_lib, Z, b)
    assert s == 0, (be, it)
    assert be <= 1e-10 and backward_error(Z, x, b) <= 1e-10
    assert rel_err(x, np.linalg.solve(Z, b)) < 1e-8


def test_multiple_right_hand_sides(gpu_lib):
    rng = np.random.default_rng(7)
    n, k = 200, 4
    Z = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)) + 10 * np.eye(n)
    B = rng.standard_normal((k, n)) + 1j * rng.standard_normal((k, n))
    s, X, be, it = mixed_solve(gpu_lib, Z, B)
    assert s == 0
    for q in range(k):
        assert backward_error(Z, X[q], B[q]) <= 1e-10


@pytest.mark.parametrize("n,k", [(300, 40), (1000, 96)])
def test_many_right_hand_sides(gpu_lib, n, k):
    """32 or more right-hand sides take the blocked form (GEMM updates in the
    triangular solves, the FP64 residual as a GEMM): every right-hand side
    reaches the gate and agrees with LAPACK."""
    rng = np.random.default_rng(n + k)
    Z = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)) + n ** 0.5 * np.eye(n)
    Z *= np.logspace(-3, 3, n)[:, None]
    B = rng.standard_normal((k, n)) + 1j * rng.standard_normal((k, n))
    s, X, be, it = mixed_solve(gpu_lib, Z, B)
    assert s == 0, (be, it)
    assert be <= 1e-10
    Xr = np.linalg.solve(Z, B.T).T
    for q in range(k):
        assert backward_error(Z, X[q], B[q]) <= 1e-10
        assert rel_err(X[q], Xr[q]) < 1e-8


def test_peec_box_system_matches_plain_fp64(gpu_lib):
    """Harmonic MNA matrix of a small PEC box at 30 MHz (assembled on the
    GPU): the mixed solve reaches the 1e-10 gate and agrees with the plain
    FP64 complex LU."""
    with SynthMesh.box(0.4, 0.2, 0.1, 16, 8, 4) as m:
        ne, nv = m.n_edges, m.n_nodes
        n = ne + nv
        lo = abi.InductanceOptions()
        gpu_lib.inductance_options_default(C.byref(lo), 1)
        po = abi.PotentialOptions()
        gpu_lib.potential_options_default(C.byref(po), 1)
        dL = gpu_lib.peec_gb300_device_alloc(ne * ne * 8)
        dP = gpu_lib.peec_gb300_device_alloc(nv * nv * 8)
        dZ = gpu_lib.peec_gb300_device_alloc(n * n * 16)
        edges = np.ascontiguousarray(m.edges())
        dE = dev_put(gpu_lib, edges)
        assert gpu_lib.peec_gb300_inductance_device(C.byref(m.mesh), C.byref(m.dual), C.byref(lo), dL, None) == 0
        assert gpu_lib.peec_gb300_potential_device(C.byref(m.mesh), C.byref(m.dual), C.byref(po), dP, None) == 0
        assert gpu_lib.peec_gb300_harmonic_build_device(dL, dP, dE, None, ne, nv, 30e6, dZ) == 0
        Z = np.zeros((n, n), dtype=np.complex128)
        gpu_lib.peec_gb300_copy_to_host(Z.ctypes.data, dZ, Z.nbytes)
        for p in (dL, dP, dZ, dE):
            gpu_lib.peec_gb300_device_free(p)
    rng = np.random.default_rng(3)
    b = np.zeros(n, dtype=np.complex128)
    b[:ne] = rng.standard_normal(ne) + 1j * rng.standard_normal(ne)
    s, x, be, it = mixed_solve(gpu_lib, Z, b)
    assert s == 0, (be, it)
    assert backward_error(Z, x, b) <= 1e-10
    f = ComplexLU(gpu_lib, Z)
    assert f.status == 0
    _, xp = f.solve(b)
    f.free()
    assert rel_err(x, xp) < 1e-7


def mna_matrix(lib, m, freq):
    """The harmonic MNA matrix of mesh m at freq, assembled on the GPU."""
    ne, nv = m.n_edges, m.n_nodes
    n = ne + nv
    lo = abi.InductanceOptions()
    lib.inductance_options_default(C.byref(lo), 1)
    po = abi.PotentialOptions()
    lib.potential_options_default(C.byref(po), 1)
    dL = lib.peec_gb300_device_alloc(ne * ne * 8)
    dP = lib.peec_gb300_device_alloc(nv * nv * 8)
    dZ = lib.peec_gb300_device_alloc(n * n * 16)
    dE = dev_put(lib, np.ascontiguousarray(m.edges()))
    assert lib.peec_gb300_inductance_device(C.byref(m.mesh), C.byref(m.dual), C.byref(lo), dL, None) == 0
    assert lib.peec_gb300_potential_device(C.byref(m.mesh), C.byref(m.dual), C.byref(po), dP, None) == 0
    assert lib.peec_gb300_harmonic_build_device(dL, dP, dE, None, ne, nv, freq, dZ) == 0
    Z = np.zeros((n, n), dtype=np.complex128)
    lib.peec_gb300_copy_to_host(Z.ctypes.data, dZ, Z.nbytes)
    for p in (dL, dP, dZ, dE):
        lib.peec_gb300_device_free(p)
    return Z


def plate_system(lib, freq):
    """Plate 1.41 x 1.12 m, 18 x 15 cells (877 unknowns) at freq, excited by an
    x-polarised unit plane wave at normal incidence (U_e = E . l_e)."""
    with SynthMesh.plate(1.41, 1.12, 18, 15) as m:
        ne = m.n_edges
        Z = mna_matrix(lib, m, freq)
        vec = m.array("edge_vectors", (ne, 3))
    b = np.zeros(Z.shape[0], dtype=np.complex128)
    b[:ne] = -vec[:, 0]
    return Z, b


def test_bf16x3_factor_suffices_at_30mhz(gpu_lib):
    Z, b = plate_system(gpu_lib, 30e6)
    s, x, be, it = mixed_solve(gpu_lib, Z, b)
    assert s == 0, (be, it)
    assert backward_error(Z, x, b) <= 1e-10
    assert gpu_lib.peec_gb300_mixed_split_terms() == 3


def test_ladder_reaches_the_gate_at_1khz(gpu_lib):
    """At 1 kHz the equilibrated MNA matrix of the plate has a condition
    number near 2e8: refinement from the BF16x3 factor (about 16-bit trailing
    updates) stalls, the solve factors the FP32 matrix again with BF16x6
    products, and where refinement from that stalls too, GMRES-IR with the
    BF16x6 factor as preconditioner reaches the gate -- no FP64 LU."""
    Z, b = plate_system(gpu_lib, 1e3)
    s, x, be, it = mixed_solve(gpu_lib, Z, b)
    assert gpu_lib.peec_gb300_mixed_split_terms() == 6
    assert s == 0, (be, it, gpu_lib.peec_gb300_mixed_gmres_iterations())
    assert backward_error(Z, x, b) <= 1e-10


def test_fgmres_runs_right_hand_sides_in_lockstep(gpu_lib):
    """FGMRES-IR advances up to 8 right-hand sides in lockstep (one
    triangular solve, one pass over Z and one host round trip per step),
    each with its own Krylov basis and stopping: at 1 kHz every right-hand
    side of five reaches the gate, and each solution is bit-identical to the
    solve of that right-hand side alone (FGMRES starts from zero on the same
    BF16x6 factor)."""
    Z, b = plate_system(gpu_lib, 1e3)
    rng = np.random.default_rng(9)
    B = np.stack([b] + [b * (1.0 + 0.5 * rng.standard_normal(b.shape)) for _ in range(4)])
    s, X, be, it = mixed_solve(gpu_lib, Z, B)
    steps = gpu_lib.peec_gb300_mixed_gmres_iterations()
    assert s == 0, (be, it, steps)
    assert steps > 0
    for q in range(B.shape[0]):
        assert backward_error(Z, X[q], B[q]) <= 1e-10
    for q in (0, 3):
        s1, x1, be1, it1 = mixed_solve(gpu_lib, Z, B[q])
        assert s1 == 0
        if gpu_lib.peec_gb300_mixed_gmres_iterations() > 0 and gpu_lib.peec_gb300_mixed_split_terms() == 6:
            assert np.array_equal(x1, X[q])


BF16X6_SCRIPT = """
import ctypes as C, json, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
from peeeeeeeeeeeeeeeeeeec_gb300 import abi
lib = abi.load_gpu_lib()
rng = np.random.default_rng(1)
n = 700
Z = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)) + 3 * np.eye(n)
b = rng.standard_normal(n) + 0j
def put(a):
    p = lib.peec_gb300_device_alloc(a.nbytes)
    lib.peec_gb300_copy_to_device(p, a.ctypes.data, a.nbytes)
    return p
dZ, db, dx = put(Z), put(b), lib.peec_gb300_device_alloc(b.nbytes)
be, it = C.c_double(), C.c_int()
s = lib.peec_gb300_complex_solve_mixed_device(dZ, n, db, dx, 1, 1e-10, 30, C.byref(be), C.byref(it))
x = np.zeros_like(b)
lib.peec_gb300_copy_to_host(x.ctypes.data, dx, x.nbytes)
r = Z @ x - b
print(json.dumps({"status": s, "iterations": it.value, "terms": lib.peec_gb300_mixed_split_terms(),
                  "backward_error": float(np.max(np.abs(r) / (np.abs(Z) @ np.abs(x) + np.abs(b))))}))
"""


def test_bf16x6_from_the_start():
    """PEEC_GB300_MIXED_SPLIT=6 factors with BF16x6 products from the start
    (a fresh process: the switch is read once): the gate is reached, in no
    more sweeps than the BF16x3 factor needs."""
    import json
    import os
    import subprocess
    import sys
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = {}
    for terms in ("3", "6"):
        env = dict(os.environ, PEEC_GB300_MIXED_SPLIT=terms)
        r = subprocess.run([sys.executable, "-c", BF16X6_SCRIPT, repo], env=env, capture_output=True, text=True,
                           timeout=300)
        assert r.returncode == 0, r.stderr
        out[terms] = json.loads(r.stdout.strip().splitlines()[-1])
    for terms in ("3", "6"):
        assert out[terms]["status"] == 0 and out[terms]["backward_error"] <= 1e-10
        assert out[terms]["terms"] == int(terms)
    assert out["6"]["iterations"] <= out["3"]["iterations"]


def test_singular_and_bad_input(gpu_lib):
    Z = np.eye(40, dtype=np.complex128)
    Z[5, :] = 0
    s, _, _, _ = mixed_solve(gpu_lib, Z, np.ones(40, dtype=np.complex128))
    assert s == -2


def test_fp32_far_field_assembly_error(gpu_lib, oracle):
    """Mixed path assembly: FP32 far rule (near field still FP64).  The error
    against the FP64 oracle is stated: below 1e-6 relative per entry."""
    from helpers import inductance, potential
    with SynthMesh.box(0.3, 0.2, 0.1, 6, 4, 2) as m:
        prev = gpu_lib.peec_gb300_set_far_precision(2)
        try:
            s, L = inductance(gpu_lib, m)
            s2, P = potential(gpu_lib, m)
        finally:
            gpu_lib.peec_gb300_set_far_precision(prev)
        assert s == 0 and s2 == 0
        Lo, Po = oracle.inductance(m)[1], oracle.potential(m)[1]
        nz = Lo != 0
        assert np.array_equal(L != 0, nz)
        assert np.max(np.abs(L[nz] - Lo[nz]) / np.abs(Lo[nz])) < 1e-6
        assert np.max(np.abs(P - Po) / np.abs(Po)) < 1e-6
        # and the default mode is back to FP64-accurate
        s, L2 = inductance(gpu_lib, m)
        assert np.max(np.abs(L2[nz] - Lo[nz]) / np.abs(Lo[nz])) < 1e-12


def test_fp64_refinement_reaches_the_gate_at_low_frequency(gpu_lib):
    """At 1 kHz the MNA matrix of a small box is badly conditioned and the
    plain FP64 LU solution misses the 1e-10 backward-error gate on some right-
    hand sides; FP64 iterative refinement with the same factor reaches it."""
    with SynthMesh.box(0.4, 0.2, 0.1, 8, 4, 2) as m:
        ne, nv = m.n_edges, m.n_nodes
        n = ne + nv
        lo = abi.InductanceOptions()
        gpu_lib.inductance_options_default(C.byref(lo), 1)
        po = abi.PotentialOptions()
        gpu_lib.potential_options_default(C.byref(po), 1)
        dL = gpu_lib.peec_gb300_device_alloc(ne * ne * 8)
        dP = gpu_lib.peec_gb300_device_alloc(nv * nv * 8)
        dZ = gpu_lib.peec_gb300_device_alloc(n * n * 16)
        dE = dev_put(gpu_lib, np.ascontiguousarray(m.edges()))
        assert gpu_lib.peec_gb300_inductance_device(C.byref(m.mesh), C.byref(m.dual), C.byref(lo), dL, None) == 0
        assert gpu_lib.peec_gb300_potential_device(C.byref(m.mesh), C.byref(m.dual), C.byref(po), dP, None) == 0
        assert gpu_lib.peec_gb300_harmonic_build_device(dL, dP, dE, None, ne, nv, 1e3, dZ) == 0
    rng = np.random.default_rng(9)
    B = np.zeros((4, n), dtype=np.complex128)
    B[:, :ne] = rng.standard_normal((4, ne)) + 1j * rng.standard_normal((4, ne))
    dB, dX = dev_put(gpu_lib, B), gpu_lib.peec_gb300_device_alloc(B.nbytes)
    dLU = gpu_lib.peec_gb300_device_alloc(n * n * 16)
    assert gpu_lib.peec_gb300_copy_device(dLU, dZ, n * n * 16) == 0
    piv, perm = gpu_lib.peec_gb300_device_alloc(n * 8), gpu_lib.peec_gb300_device_alloc(n * 4)
    rs, cs = gpu_lib.peec_gb300_device_alloc(n * 8), gpu_lib.peec_gb300_device_alloc(n * 8)
    sc, col = C.c_double(), C.c_int()
    assert gpu_lib.peec_gb300_complex_lu_factor_device(dLU, n, 1e-14, piv, perm, rs, cs, C.byref(sc), C.byref(col)) == 0
    assert gpu_lib.peec_gb300_complex_lu_solve_device(dLU, perm, rs, cs, n, dB, dX, 4) == 0
    be, it = C.c_double(), C.c_int()
    s = gpu_lib.peec_gb300_complex_refine_device(dZ, dLU, perm, rs, cs, n, dB, dX, 4, 1e-10, 5, C.byref(be), C.byref(it))
    X = np.zeros_like(B)
    gpu_lib.peec_gb300_copy_to_host(X.ctypes.data, dX, X.nbytes)
    Z = np.zeros((n, n), dtype=np.complex128)
    gpu_lib.peec_gb300_copy_to_host(Z.ctypes.data, dZ, Z.nbytes)
    for p in (dL, dP, dZ, dE, dB, dX, dLU, piv, perm, rs, cs):
        gpu_lib.peec_gb300_device_free(p)
    assert s == 0, (be.value, it.value)
    for q in range(4):
        assert backward_error(Z, X[q], B[q]) <= 1e-10


def test_fp32_rounding_matches_ieee(gpu_lib):
    """The integer-arithmetic FP64 -> FP32 rounding of the equilibration
    against IEEE round-to-nearest-even (numpy), with ties, carries into the
    exponent, overflow, the subnormal flush, zeros, inf and NaN."""
    rng = np.random.default_rng(3)
    x = np.concatenate([
        rng.standard_normal(20000) * 10.0 ** rng.uniform(-30, 30, 20000),
        np.float64(np.float32(rng.standard_normal(2000))) * (1 + 2.0 ** -24),   # exact ties
        np.float64(np.float32(rng.standard_normal(2000))) * (1 - 2.0 ** -25),
        np.array([0.0, -0.0, 1.0, -1.0, 2.0 ** -126, 2.0 ** -127, 2.0 ** -149, 3.4028234663852886e38,
                  3.4028235677973366e38, 1e39, -1e39, np.inf, -np.inf, np.nan, 1.9999999999999998,
                  1.0 + 2.0 ** -24, 1.0 + 3 * 2.0 ** -24, 5e-324])])
    for shift in (0, 7, -5):
        n = x.size
        dx = gpu_lib.peec_gb300_device_alloc(x.nbytes)
        dy = gpu_lib.peec_gb300_device_alloc(n * 4)
        gpu_lib.peec_gb300_copy_to_device(dx, x.ctypes.data, x.nbytes)
        assert gpu_lib.peec_gb300_round_to_f32_device(dx, dy, n, shift) == 0
        y = np.zeros(n, dtype=np.float32)
        gpu_lib.peec_gb300_copy_to_host(y.ctypes.data, dy, y.nbytes)
        gpu_lib.peec_gb300_device_free(dx)
        gpu_lib.peec_gb300_device_free(dy)
        with np.errstate(over="ignore", under="ignore", invalid="ignore"):
            ref = (x * 2.0 ** -shift).astype(np.float32)
        tiny = np.abs(ref) < np.float32(2.0 ** -126)
        ref[tiny] = np.copysign(np.float32(0.0), ref[tiny])
        # a subnormal FP64 input (the last one) is flushed too
        ref[np.abs(x) < 2.0 ** -1022] = np.copysign(np.float32(0.0), x[np.abs(x) < 2.0 ** -1022])
        assert np.array_equal(y.view(np.uint32)[~np.isnan(ref)], ref.view(np.uint32)[~np.isnan(ref)]), shift
        assert np.all(np.isnan(y[np.isnan(ref)]))


_PANEL_FORMS_PROBE = r"""
import sys
import numpy as np
sys.path.insert(0, {repo!r}); sys.path.insert(0, {tests!r})
from peeeeeeeeeeeeeeeeeeec_gb300 import abi
from test_gpu_mixed import mixed_solve, backward_error
lib = abi.load_gpu_lib()
rng = np.random.default_rng(21)
out = []
for n in (700, 1900):
    Z = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)) + n ** 0.5 * np.eye(n)
    b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    s, x, be, it = mixed_solve(lib, Z, b)
    assert s == 0 and be <= 1e-10 and backward_error(Z, x, b) <= 1e-10, (n, s, be)
    out.append(x)
np.save(sys.argv[1], np.concatenate(out))
"""


@pytest.mark.parametrize("form", ["lean", "coop"])
def test_every_fp32_panel_form_reaches_the_gate(gpu_lib, form, tmp_path):
    """The mixed solve with each FP32 panel form (PEEC_GB300_MIXED_PANEL:
    cluster by default, lean grid, cooperative grid) reaches the 1e-10
    gate, and the solutions agree with the default form's."""
    import os
    import subprocess
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    code = _PANEL_FORMS_PROBE.format(repo=os.path.dirname(here), tests=here)
    sols = {}
    for f in ("default", form):
        env = dict(os.environ)
        env.pop("PEEC_GB300_MIXED_PANEL", None)
        if f != "default":
            env["PEEC_GB300_MIXED_PANEL"] = f
        path = str(tmp_path / (f + ".npy"))
        r = subprocess.run([sys.executable, "-c", code, path], env=env, capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
        sols[f] = np.load(path)
    assert rel_err(sols[form], sols["default"]) < 1e-8
