"""GPU real and complex LU against the reference's known answers
(reference tests/test_core.c:17-66, 328-337), its own factorisations
(golden fixtures) and the oracle.  Solutions: 1e-10 relative (the drop-in
bar for currents and potentials); pivots: identical where the reference's
choice is not a near tie."""
import numpy as np
import pytest

from conftest import golden
from helpers import ComplexLU, RealLU, rel_err

pytestmark = pytest.mark.gpu
ALGEBRA_TOL = 1e-11


def test_real_known_answer(gpu_lib):
    a = np.array([0, 2, 1, 1, -2, -3, 2, 3, 1], float).reshape(3, 3)
    exact = np.array([1, -2, 0.5])
    f = RealLU(gpu_lib, a)
    assert f.status == 0
    s, x = f.solve(a @ exact)
    assert s == 0 and np.max(np.abs(x - exact)) < ALGEBRA_TOL
    lu, piv = f.factors()
    assert piv.tolist() == [2, 2, 2] or piv[0] == 2   # |2| is the first maximum of column 0
    f.free()


def test_complex_known_answer(gpu_lib):
    a = np.array([[0, 2 + 1j], [1 - 1j, 3 + 0.5j]])
    exact = np.array([1 + 2j, -0.5 + 0.75j])
    f = ComplexLU(gpu_lib, a)
    assert f.status == 0
    s, x = f.solve(a @ exact)
    assert s == 0 and np.max(np.abs(x - exact)) < ALGEBRA_TOL
    f.free()


def test_complex_singular(gpu_lib):
    f = ComplexLU(gpu_lib, np.array([[1 + 1j, 2 + 2j], [2 + 2j, 4 + 4j]]))
    assert f.status == -2
    f.free()


def test_real_singular_and_zero(gpu_lib):
    f = RealLU(gpu_lib, np.array([[1.0, 2.0], [2.0, 4.0]]))
    assert f.status == -2 and f.f.factorized == 0
    f.free()
    f = RealLU(gpu_lib, np.zeros((3, 3)))
    assert f.status == -2
    f.free()
    a = np.eye(4)
    a[2, 2] = np.nan
    f = RealLU(gpu_lib, a)
    assert f.status == -2
    f.free()


def test_complex_zero_row_and_nonfinite(gpu_lib):
    a = np.eye(3, dtype=complex)
    a[1, :] = 0
    assert ComplexLU(gpu_lib, a).status == -2
    a = np.eye(3, dtype=complex)
    a[0, 2] = np.inf
    assert ComplexLU(gpu_lib, a).status == -2


def test_real_cases_match_reference(gpu_lib):
    g = golden("lu_cases")
    for n in (1, 7, 40, 97):
        f = RealLU(gpu_lib, g["real%d_a" % n])
        assert f.status == 0
        lu, piv = f.factors()
        assert np.array_equal(piv, g["real%d_piv" % n])
        assert rel_err(lu, g["real%d_lu" % n]) < 1e-12
        s, x = f.solve(g["real%d_b" % n])
        assert s == 0 and rel_err(x, g["real%d_x" % n]) < 1e-10
        det = gpu_lib.lu_determinant(f.f)
        assert abs(det - float(g["real%d_det" % n])) <= 1e-10 * abs(float(g["real%d_det" % n]))
        f.free()


def test_complex_cases_match_reference(gpu_lib):
    g = golden("lu_cases")
    for n in (1, 5, 33, 80):
        f = ComplexLU(gpu_lib, g["cplx%d_a" % n])
        assert f.status == 0
        lu, piv, rs, cs = f.factors()
        assert np.array_equal(piv, g["cplx%d_piv" % n])
        assert rel_err(rs, g["cplx%d_rs" % n]) < 1e-15 and rel_err(cs, g["cplx%d_cs" % n]) < 1e-15
        assert rel_err(lu, g["cplx%d_lu" % n]) < 1e-12
        s, x = f.solve(g["cplx%d_b" % n])
        assert s == 0 and rel_err(x, g["cplx%d_x" % n]) < 1e-10
        f.free()


@pytest.mark.parametrize("n", [31, 32, 33, 64, 65, 255, 700])
def test_real_sizes_against_oracle(gpu_lib, oracle, n):
    """Panel-width boundaries and ragged tiles."""
    rng = np.random.default_rng(n)
    a = rng.standard_normal((n, n))
    b = rng.standard_normal(n)
    f = RealLU(gpu_lib, a)
    assert f.status == 0
    s, lu_o, piv_o, swaps, scale = oracle.lu_factorize(a)
    lu, piv = f.factors()
    assert np.array_equal(piv, piv_o.astype(np.int64))
    assert f.f.swap_count == swaps and f.f.matrix_scale == scale
    assert rel_err(lu, lu_o) < 1e-10
    s, x = f.solve(b)
    _, xo = oracle.lu_solve(lu_o, piv_o, b)
    assert s == 0 and rel_err(x, xo) < 1e-10
    f.free()


@pytest.mark.parametrize("n", [1, 2, 33, 96, 321])
def test_complex_sizes_against_oracle(gpu_lib, oracle, n):
    rng = np.random.default_rng(100 + n)
    a = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    a *= np.logspace(-3, 3, n)[:, None]
    b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    f = ComplexLU(gpu_lib, a)
    assert f.status == 0
    s, lu_o, piv_o, swaps, scale, rs, cs = oracle.complex_lu_factorize(a)
    lu, piv, grs, gcs = f.factors()
    assert np.array_equal(piv, piv_o.astype(np.int64))
    assert rel_err(grs, rs) < 1e-15 and rel_err(gcs, cs) < 1e-15
    s, x = f.solve(b)
    _, xo = oracle.complex_lu_solve(lu_o, piv_o, rs, cs, b)
    assert s == 0 and rel_err(x, xo) < 1e-10
    f.free()


def test_solve_in_place_and_multiple(gpu_lib):
    rng = np.random.default_rng(5)
    n, k = 130, 7
    a = rng.standard_normal((n, n))
    B = rng.standard_normal((k, n))
    f = RealLU(gpu_lib, a)
    s, X = f.solve_multiple(B)
    assert s == 0
    assert rel_err(X, np.linalg.solve(a, B.T).T) < 1e-10
    # x == b is allowed
    import ctypes as C
    from helpers import dp
    b = B[0].copy()
    assert gpu_lib.lu_solve(C.byref(f.f), dp(b), dp(b)) == 0
    assert rel_err(b, X[0]) < 1e-14
    f.free()
    ac = a + 1j * rng.standard_normal((n, n))
    Bc = B + 1j * rng.standard_normal((k, n))
    fc = ComplexLU(gpu_lib, ac)
    s, Xc = fc.solve_multiple(Bc)
    assert s == 0 and rel_err(Xc, np.linalg.solve(ac, Bc.T).T) < 1e-10
    fc.free()


def test_solve_with_caller_built_factor(gpu_lib):
    """A factorisation struct filled by the caller (not by lu_factorize)
    is uploaded and used, and a changed factor is not served from the
    device cache."""
    import ctypes as C
    from helpers import dp
    from peeeeeeeeeeeeeeeeeeec_gb300 import abi
    rng = np.random.default_rng(9)
    n = 40
    a = rng.standard_normal((n, n))
    f = RealLU(gpu_lib, a)
    lu, piv = f.factors()
    lu2 = np.ascontiguousarray(lu)
    piv2 = np.ascontiguousarray(piv.astype(np.uintp))
    g = abi.LUFactorization(n, lu2.ctypes.data_as(abi.c_double_p), piv2.ctypes.data_as(abi.c_size_t_p),
                            0, 1.0, 1)
    b = rng.standard_normal(n)
    x = np.zeros(n)
    assert gpu_lib.lu_solve(C.byref(g), dp(b), dp(x)) == 0
    assert rel_err(x, np.linalg.solve(a, b)) < 1e-10
    lu2[:] = np.eye(n)
    piv2[:] = np.arange(n)
    assert gpu_lib.lu_solve(C.byref(g), dp(b), dp(x)) == 0
    assert np.array_equal(x, b)
    f.free()


def test_edited_factor_entry_is_seen_by_solve(gpu_lib, oracle):
    """A complex_lu_factorize result whose one off-diagonal entry (outside
    the cache's sampled fingerprint) is edited between two solves: the
    second solve uses the edited factor (it equals the oracle's solve with
    that factor), not a stale device copy."""
    import ctypes as C
    from helpers import cp
    rng = np.random.default_rng(21)
    n = 300
    a = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    f = ComplexLU(gpu_lib, a)
    assert f.status == 0
    s, x0 = f.solve(b)
    assert s == 0
    i, j = 5, 17                          # double index 2 (5 n + 17) is off the 4093-point sample grid
    step = (2 * n * n) // 4093 + 1
    assert (2 * (i * n + j)) % step and (2 * (i * n + j) + 1) % step
    raw = np.ctypeslib.as_array(C.cast(f.f.data, C.POINTER(C.c_double)), shape=(2 * n * n,))
    raw[2 * (i * n + j)] += 0.25
    lu, piv, rs, cs = f.factors()
    s, x1 = f.solve(b)
    assert s == 0
    _, xo = oracle.complex_lu_solve(np.ascontiguousarray(lu), piv.astype(np.uintp), rs, cs, b)
    assert rel_err(x1, xo) < 1e-12
    assert rel_err(x1, x0) > 1e-6
    f.free()


_PANEL_PROBE = r"""
import ctypes as C, hashlib, sys
import numpy as np
sys.path.insert(0, {repo!r}); sys.path.insert(0, {tests!r})
from helpers import ComplexLU, RealLU
from peeeeeeeeeeeeeeeeeeec_gb300 import abi
lib = abi.load_gpu_lib()
rng = np.random.default_rng(5)
h = hashlib.sha256()
for n in (700, 1500):
    a = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    f = ComplexLU(lib, a)
    lu, piv, rs, cs = f.factors()
    h.update(lu.tobytes()); h.update(piv.tobytes()); f.free()
    r = RealLU(lib, a.real)
    lu, piv = r.factors()
    h.update(lu.tobytes()); h.update(piv.tobytes()); r.free()
print(h.hexdigest())
"""


def test_lean_and_grid_panels_agree():
    """The lean FP64 panel (default: flag-published candidates, no grid
    barrier) and the cooperative grid panel (PEEC_GB300_PANEL=coop) make the
    same pivot choices and the same arithmetic: the factors agree bit for
    bit."""
    import os
    import subprocess
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    code = _PANEL_PROBE.format(repo=os.path.dirname(here), tests=here)
    out = {}
    for mode in ("coop", "lean"):
        env = dict(os.environ)
        if mode == "coop":
            env["PEEC_GB300_PANEL"] = "coop"
        else:
            env.pop("PEEC_GB300_PANEL", None)
        r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
        out[mode] = r.stdout.strip()
    assert out["coop"] == out["lean"]
