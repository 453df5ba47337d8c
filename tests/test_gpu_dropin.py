"""The reference's own programs, unchanged, running on the GB300 library.

`make -C oracle relink` builds (on this host) the reference's unit tests
(tests/test_core.c) and its CLI PeecSolver (src/main.c with its harmonic,
transient and RCS drivers) twice from the reference's sources: *_gb300 with
the hot path (quadrature.c, inductance.c, potential.c, lu.c, complex_lu.c,
incidence.c, matrix_export.c) taken from libpeec_gb300.so, and *_ref on the
reference's own sources.  The tests run both and compare:

  test_core      every case the reference build passes also passes on the
                 GPU build (the reference's own tolerances: known-answer
                 LUs, quadrature identities, the analytic harmonic loop, the
                 singular matrix, the transient orders)
  scattering     the reference's CLI gate on meshes/plate.msh at 1 Hz,
                 1 kHz, 1 MHz (backward error <= 1e-9, reference
                 tests/run_tests.py:95-106); the exported L and P within
                 1e-12 of the reference build's (per entry, relative to the
                 largest entry), A identical, P A^T within 1e-12; the
                 printed max |I_e| and |V_j| equal to the printed digits
  rcs            sigma within 1e-9 relative, 3 directions
  lightning      node potentials and edge currents of every VTK snapshot
                 within 1e-9 of the largest value of the snapshot

The reference's sources come from the staged copy baseline/_ref/; without
it the tests are skipped.
"""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STAGE = os.path.join(REPO, "baseline", "_ref")
BIN = os.path.join(REPO, "oracle", "_ref")

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not os.path.isdir(os.path.join(STAGE, "src")),
                                 reason="the reference's sources are not staged in baseline/_ref")]


@pytest.fixture(scope="module")
def programs(gpu_lib):
    r = subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "relink"], stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout[-4000:]
    return {k: os.path.join(BIN, k) for k in ("test_core_gb300", "test_core_ref", "PeecSolver_gb300",
                                              "PeecSolver_ref")}


@pytest.fixture(scope="module")
def workdir(tmp_path_factory):
    d = tmp_path_factory.mktemp("cli")
    shutil.copytree(os.path.join(STAGE, "meshes"), str(d / "meshes"))
    return d


def run(cmd, cwd):
    return subprocess.run(cmd, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=300)


def test_reference_unit_tests(programs, workdir):
    cases = run([programs["test_core_ref"], "--list"], workdir).stdout.split()
    assert len(cases) >= 15
    failed = []
    for case in cases:
        ref = run([programs["test_core_ref"], case], workdir)
        gpu = run([programs["test_core_gb300"], case], workdir)
        if ref.returncode == 0 and ("PASS " + case) in ref.stdout:
            if not (gpu.returncode == 0 and ("PASS " + case) in gpu.stdout):
                failed.append((case, gpu.stdout[-500:], gpu.stderr[-500:]))
    assert not failed, failed


def read_mtx(path):
    """Dense array (column-major) or coordinate (1-based) Matrix Market."""
    with open(path) as f:
        head = f.readline()
        lines = [ln for ln in f if not ln.startswith("%")]
    dims = [int(v) for v in lines[0].split()]
    rows, cols = dims[0], dims[1]
    if "coordinate" in head:
        out = np.zeros((rows, cols))
        for ln in lines[1:1 + dims[2]]:
            i, j, v = ln.split()
            out[int(i) - 1, int(j) - 1] = float(v)
        return out
    vals = np.array([float(v) for v in lines[1:1 + rows * cols]])
    return vals.reshape(cols, rows).T


def solver_output(text):
    out = {}
    for key, pat in (("be", r"Backward error\s*:\s*(\S+)"), ("imax", r"Maximum \|I_e\|\s*:\s*(\S+)"),
                     ("vmax", r"Maximum \|V_j\|\s*:\s*(\S+)")):
        m = re.search(pat, text)
        out[key] = float(m.group(1)) if m else None
    return out


@pytest.mark.parametrize("frequency", ["1", "1000", "1e6"])
def test_reference_cli_scattering(programs, workdir, frequency):
    res = {}
    for tag in ("ref", "gb300"):
        mdir = str(workdir / ("mats_%s_%s" % (tag, frequency)))
        p = run([programs["PeecSolver_" + tag], "--task", "scattering", "--mesh", "meshes/plate.msh", "--frequency",
                 frequency, "--parallel", "1", "--save-matrices", "--matrix-dir", mdir], workdir)
        assert p.returncode == 0 and "ERROR:" not in p.stderr, (tag, p.stderr[-2000:])
        res[tag] = (solver_output(p.stdout), mdir)
    (o_ref, d_ref), (o_gpu, d_gpu) = res["ref"], res["gb300"]
    assert o_gpu["be"] is not None and o_gpu["be"] <= 1e-9
    for key in ("imax", "vmax"):  # printed with 10 significant digits
        assert abs(o_gpu[key] - o_ref[key]) <= 5e-10 * abs(o_ref[key]), (key, o_gpu[key], o_ref[key])
    for name, tol in (("L", 1e-12), ("P", 1e-12), ("PAT", 1e-12), ("A", 0.0)):
        a, b = read_mtx(os.path.join(d_gpu, name + ".mtx")), read_mtx(os.path.join(d_ref, name + ".mtx"))
        assert a.shape == b.shape
        assert np.max(np.abs(a - b)) <= tol * np.max(np.abs(b)), name


def test_reference_cli_rcs(programs, workdir):
    sig = {}
    for tag in ("ref", "gb300"):
        out = str(workdir / ("rcs_%s.csv" % tag))
        p = run([programs["PeecSolver_" + tag], "--task", "rcs", "--mesh", "meshes/plate.msh", "--ka", "0.02", "--a",
                 "1", "--parallel", "1", "--rcs-dual", "--phi-start", "0", "--phi-end", "90", "--phi-step", "45",
                 "--rcs-order", "4", "--output", out], workdir)
        assert p.returncode == 0 and "ERROR:" not in p.stderr, (tag, p.stderr[-2000:])
        rows = [ln.split(",") for ln in open(out).read().strip().splitlines()[1:]]
        sig[tag] = np.array([float(r[2]) for r in rows])
    assert sig["gb300"].shape == (3,)
    assert np.max(np.abs(sig["gb300"] - sig["ref"]) / sig["ref"]) <= 1e-9


def vtk_arrays(path):
    """Every numeric block of a legacy ASCII VTK file, keyed by the section
    header it follows (POINTS, POLYGONS / LINES, SCALARS name, VECTORS
    name)."""
    blocks, key, vals = {}, None, []
    for line in open(path):
        parts = line.split()
        if not parts:
            continue
        try:
            vals.extend(float(v) for v in parts)
        except ValueError:
            if parts[0] == "LOOKUP_TABLE":
                continue
            if key is not None and vals:
                blocks[key] = np.array(vals)
            key, vals = line.strip(), []
    if key is not None and vals:
        blocks[key] = np.array(vals)
    return blocks


def test_reference_cli_lightning(programs, workdir):
    dirs = {}
    for tag in ("ref", "gb300"):
        vdir = str(workdir / ("vtk_" + tag))
        p = run([programs["PeecSolver_" + tag], "--task", "lightning", "--mesh", "meshes/plate.msh", "--dt", "1e-7",
                 "--t-end", "2e-6", "--time-order", "2", "--strike-node", "0", "--return-node", "99", "--parallel",
                 "1", "--vtk", "--vtk-dir", vdir, "--vtk-every", "5"], workdir)
        assert p.returncode == 0 and "ERROR:" not in p.stderr, (tag, p.stderr[-2000:])
        dirs[tag] = vdir
    files = sorted(os.listdir(dirs["ref"]))
    assert files and files == sorted(os.listdir(dirs["gb300"]))
    for f in files:
        a, b = vtk_arrays(os.path.join(dirs["gb300"], f)), vtk_arrays(os.path.join(dirs["ref"], f))
        assert a.keys() == b.keys(), f
        for k in b:
            scale = max(np.max(np.abs(b[k])), 1e-300)
            assert np.max(np.abs(a[k] - b[k])) <= 1e-9 * scale, (f, k)
