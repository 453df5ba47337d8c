"""The C-ABI library loads without a GPU and exports every function that
include/*.h declares; struct layouts match the reference's sizes."""
import ctypes as C
import os
import re
import subprocess

from peeeeeeeeeeeeeeeeeeec_gb300 import abi

INCLUDE = os.path.join(abi.REPO_DIR, "include")
DROP_IN = ["quadrature.h", "inductance.h", "potential.h", "lu.h", "complex_lu.h", "incidence.h", "matrix_export.h", "peec_gb300.h"]


def declared_functions(header):
    text = open(os.path.join(INCLUDE, header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"static inline[^{]*\{[^}]*\}", "", text)
    names = re.findall(r"\b([a-z_][a-z0-9_]*)\s*\([^;{]*\)\s*;", text)
    return [n for n in names if n not in ("if", "return", "sizeof")]


def exported(lib_path):
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], stdout=subprocess.PIPE, text=True).stdout
    return {line.split()[-1] for line in out.splitlines() if line.strip()}


def test_every_declared_symbol_is_exported():
    syms = exported(abi.GPU_LIB_PATH)
    missing = []
    for h in DROP_IN:
        for name in declared_functions(h):
            if name not in syms:
                missing.append((h, name))
    assert not missing, missing


def test_library_loads_and_binds_without_gpu():
    lib = abi.load_gpu_lib()
    for name, _, _ in abi.DROP_IN_SYMBOLS + abi.EXT_SYMBOLS:
        assert hasattr(lib, name)


def test_struct_layouts():
    assert C.sizeof(abi.QuadPatch) == 104
    assert C.sizeof(abi.Complex) == 16
    assert C.sizeof(abi.Mesh) == 3 * 8 + 12 * 8
    assert C.sizeof(abi.LUFactorization) == 48
    assert C.sizeof(abi.ComplexLUFactorization) == 64
    assert C.sizeof(abi.InductanceOptions) == 40
    assert C.sizeof(abi.PotentialOptions) == 32


def test_host_helpers_match_reference_formulas():
    """Defaults and pure-host helpers need no device."""
    lib = abi.load_gpu_lib()
    o = abi.InductanceOptions()
    lib.inductance_options_default(C.byref(o), 3)
    assert (o.far_order, o.near_order, o.touching_order, o.self_order) == (4, 10, 12, 8)
    assert o.near_factor == 0.5 and o.parallel_threads == 3 and o.direction_tolerance == 1e-10
    lo = abi.LUOptions()
    lib.lu_options_default(C.byref(lo), 2)
    assert lo.pivot_tolerance == 1e-14 and lo.parallel_threshold == 64
    x = (C.c_double * 16)()
    w = (C.c_double * 16)()
    assert lib.gauss_legendre_rule(7, x, w) == -1
    assert lib.gauss_legendre_rule(4, x, w) == 0
    p = abi.QuadPatch()
    for t, v in enumerate([0, 0, 0, 2, 0, 0, 2, 1, 0, 0, 1, 0]):
        p.points[t] = v
    assert lib.quad_patch_area(C.byref(p)) == 2.0
    assert lib.quad_patch_size(C.byref(p)) == 2.0
    assert lib.quad_patch_classify_pair(C.byref(p), C.byref(p), 0.5) == 0
    assert lib.quad_patch_area(None) == 0.0


def test_lu_argument_errors_without_gpu():
    lib = abi.load_gpu_lib()
    o = abi.LUOptions()
    lib.lu_options_default(C.byref(o), 0)   # parallel_threads < 1 is rejected
    f = abi.LUFactorization()
    a = (C.c_double * 4)(1, 0, 0, 1)
    assert lib.lu_factorize(a, 2, C.byref(o), C.byref(f)) == -1
    lib.lu_options_default(C.byref(o), 1)
    assert lib.lu_factorize(None, 2, C.byref(o), C.byref(f)) == -1
    assert lib.lu_factorize(a, 0, C.byref(o), C.byref(f)) == -1
    assert lib.lu_solve(C.byref(f), a, a) == -1           # not factorised
    assert lib.inductance_compute_matrix(None, None, None, None) == -1
