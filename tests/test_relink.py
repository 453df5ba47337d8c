"""The drop-in boundary checked against the reference's own sources (CPU).

1. Struct layouts: tests/abi_layout.c prints sizeof / offsetof of every
   struct the drop-in ABI shares with the reference; compiled against the
   reference's headers and against include/, the two outputs must be
   identical, and the ctypes declarations must agree with them.
2. Relinking: `make -C oracle relink` compiles the reference's unit tests
   (tests/test_core.c) and its CLI (src/main.c: the harmonic, transient and
   RCS drivers) from the reference's sources, unchanged, with the drop-in
   headers of include/ ahead of the reference's own, and links them against
   libpeec_gb300.so with the sources it replaces (quadrature.c,
   inductance.c, potential.c, lu.c, complex_lu.c, incidence.c,
   matrix_export.c) left out.  A missing or mistyped entry point fails the
   compile or the link.  Running them needs the GPU
   (tests/test_gpu_dropin.py).

The reference's sources come from the staged copy baseline/_ref/ (`make -C
oracle stage`); without it these tests are skipped.
"""
import ctypes as C
import os
import subprocess

import pytest

from peeeeeeeeeeeeeeeeeeec_gb300 import abi

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STAGE = os.path.join(REPO, "baseline", "_ref")
ORACLE_REF = os.path.join(REPO, "oracle", "_ref")
GPU_LIB = os.path.join(REPO, "peeeeeeeeeeeeeeeeeeec_gb300", "libpeec_gb300.so")

needs_reference = pytest.mark.skipif(not os.path.isdir(os.path.join(STAGE, "src")),
                                     reason="the reference's sources are not staged in baseline/_ref")


def layout(include_dir, tmp_path, tag):
    exe = str(tmp_path / ("layout_" + tag))
    subprocess.run(["gcc", "-std=c17", "-I" + include_dir, os.path.join(REPO, "tests", "abi_layout.c"), "-o", exe],
                   check=True)
    out = subprocess.run([exe], check=True, stdout=subprocess.PIPE, text=True).stdout
    return dict((k, int(v)) for k, v in (line.split() for line in out.splitlines()))


@needs_reference
def test_struct_layouts_match_reference_headers(tmp_path):
    ours = layout(os.path.join(REPO, "include"), tmp_path, "ours")
    ref = layout(os.path.join(STAGE, "include"), tmp_path, "ref")
    assert ours == ref
    for key, value in ref.items():
        name, _, field = key.partition(".")
        T = getattr(abi, name)
        if field:
            assert getattr(T, field).offset == value, key
        else:
            assert C.sizeof(T) == value, key


@needs_reference
def test_reference_drivers_link_against_library():
    assert os.path.exists(GPU_LIB), "build the library first (__graft_entry__.build())"
    r = subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "relink"], stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout[-4000:]
    hot = {"inductance_compute_matrix", "potential_compute_matrix", "complex_lu_factorize", "complex_lu_solve",
           "lu_factorize", "lu_solve", "incidence_build_PAT", "gauss_legendre_rule"}
    for exe in ("PeecSolver_gb300", "test_core_gb300"):
        path = os.path.join(ORACLE_REF, exe)
        undefined = set(subprocess.run(["nm", "-u", "--format=just-symbols", path], check=True,
                                       stdout=subprocess.PIPE, text=True).stdout.split())
        undefined = {s.split("@")[0] for s in undefined}
        # the hot path is not in the executable: it is bound to the library
        assert hot & undefined, exe
        exported = set(subprocess.run(["nm", "-D", "--defined-only", "--format=just-symbols", GPU_LIB], check=True,
                                      stdout=subprocess.PIPE, text=True).stdout.split())
        for s in hot & undefined:
            assert s in exported, s
        needed = subprocess.run(["readelf", "-d", path], check=True, stdout=subprocess.PIPE, text=True).stdout
        assert "libpeec_gb300.so" in needed
