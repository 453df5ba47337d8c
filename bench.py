"""Benchmark: plain-FP64 harmonic PEEC solves on one GB300.

Workload (one step = one solve): closed PEC box 2.0 x 1.0 x 0.5 m meshed at
5 cm (2800 cells, Ne = 5600 edges, Nv = 2802 nodes, N = 8402 complex
unknowns), 30 MHz, one x-polarised unit plane wave incident from +z:
  assemble Lp (Ne^2) and P (Nv^2) from the 1/R panel integrals,
  fill the MNA matrix Z = [R + jwL, A; -P A^T, jw I] (PEC: R = 0),
  complex LU factorisation (equilibrated, partial pivoting),
  solve, and gate on the componentwise backward error <= 1e-10.
Lp and P are quasi-static (the reference has no retardation).

  value   solves/s with the geometry resident and every matrix built,
          factored and checked in HBM (extension API, CUDA-event timed on
          the library stream)
  e2e     the same solve through the drop-in C ABI with host buffers:
          inductance_compute_matrix, potential_compute_matrix, host MNA
          fill (what the reference's harmonic driver does), complex_lu_
          factorize, complex_lu_solve, and the backward error of the
          solution (Z, x and b uploaded, the library's device kernel)
  --impl reference   the reference's own CPU code on the host cores (its
          sources built here with its release flags; the bit-exact oracle
          port where they are absent), on a bounded sample extrapolated to
          one solve (oracle/cpu_baseline.py)
Legs beside the headline: the mixed-precision solve, serving (config 5:
Poisson harmonic and lightning requests), the config-4 sweep on 12 of its
48 meshes (--batch), transient, retarded, RCS, incidence and far-rule
precision;
--config3 and --config4 run those configurations alone.
Multi-GPU: the path does not shard; --gpus N runs N independent replicas
(one process per GPU) and reports the aggregate.
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

FREQ = 30e6
C0 = 299792458.0
BOX = (2.0, 1.0, 0.5, 40, 20, 10)
WORKLOAD = "pec_box_2x1x0.5m_5cm_30MHz_planewave"
METRIC = "PEEC solves/s at <=1e-10 backward error (plain FP64 GPU path)"


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), \
        int(os.environ.get("LOCAL_RANK", "0"))


# ---------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.QUERY, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            for k, name in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


# ---------------------------------------------------------------------
# workload pieces
# ---------------------------------------------------------------------
def make_mesh():
    from peeeeeeeeeeeeeeeeeeec_gb300.mesh import SynthMesh
    return SynthMesh.box(*BOX)


def set_box(spec):
    """--box lx,ly,lz,nx,ny,nz (a smaller case for profiling runs)."""
    global BOX, WORKLOAD
    v = spec.split(",")
    BOX = (float(v[0]), float(v[1]), float(v[2]), int(v[3]), int(v[4]), int(v[5]))
    WORKLOAD = "pec_box_%gx%gx%gm_%dx%dx%d_cells_30MHz_planewave" % BOX


def plane_wave(m):
    """Host copy of the right-hand side [-U_e ; 0] (same formula as the
    device kernel): x-polarised, incident from +z."""
    k0 = 2 * np.pi * FREQ / C0
    kh, eh = np.array([0.0, 0.0, -1.0]), np.array([1.0, 0.0, 0.0])
    ctr = m.array("edge_centers", (m.n_edges, 3))
    vec = m.array("edge_vectors", (m.n_edges, 3))
    phase = -k0 * (ctr @ kh)
    proj = vec @ eh
    h = 0.5 * k0 * (vec @ kh)
    sinc = np.where(np.abs(h) < 1e-8, 1 - h * h / 6, np.sin(h) / np.where(h == 0, 1, h))
    b = np.zeros(m.n_edges + m.n_nodes, dtype=np.complex128)
    b[:m.n_edges] = -proj * np.exp(1j * phase) * sinc
    return b


def _row_blocks(n, fn, threads=None):
    """fn(r0, r1) over row blocks on the host's cores (numpy releases the
    GIL inside its array operations)."""
    import concurrent.futures as cf
    threads = threads or os.cpu_count() or 1
    step = max(64, (n + 4 * threads - 1) // (4 * threads))
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(lambda r0: fn(r0, min(n, r0 + step)), range(0, n, step)))


def host_mna(L, P, edges, freq):
    """Z = [jwL, A; -P A^T, jw I] on the host, as the reference's
    harmonic_build_system does (PEC: R = 0), row blocks on all host cores."""
    ne, nv = L.shape[0], P.shape[0]
    n = ne + nv
    w = 2 * np.pi * freq
    Z = np.empty((n, n), dtype=np.complex128)
    ea, eb = edges[:, 0], edges[:, 1]

    def fill(r0, r1):
        blk = Z[r0:r1]
        blk[:] = 0.0
        e0, e1 = min(r0, ne), min(r1, ne)
        if e1 > e0:
            blk[:e1 - e0, :ne].imag = w * L[e0:e1]
            idx = np.arange(e0, e1)
            blk[idx - r0, ne + ea[e0:e1]] = -1.0
            blk[idx - r0, ne + eb[e0:e1]] = 1.0
        v0, v1 = max(r0, ne) - ne, max(r1, ne) - ne
        if v1 > v0:
            sub = blk[max(r0, ne) - r0:]
            sub[:, :ne].real = -(P[v0:v1, eb] - P[v0:v1, ea])
            sub[np.arange(v1 - v0), ne + np.arange(v0, v1)] = 1j * w

    _row_blocks(n, fill)
    return Z


class DeviceSolve:
    """One solve with every matrix in HBM (extension API)."""

    def __init__(self, lib, m):
        from peeeeeeeeeeeeeeeeeeec_gb300 import abi
        self.lib, self.m, self.abi = lib, m, abi
        ne, nv = m.n_edges, m.n_nodes
        self.ne, self.nv, self.n = ne, nv, ne + nv
        n = self.n
        al = lib.peec_gb300_device_alloc
        self.dL, self.dP = al(ne * ne * 8), al(nv * nv * 8)
        self.dZ, self.dLU = al(n * n * 16), al(n * n * 16)
        self.db, self.dx = al(n * 16), al(n * 16)
        self.dpiv, self.dperm = al(n * 8), al(n * 4)
        self.drow, self.dcol = al(n * 8), al(n * 8)
        self.dedges = al(ne * 2 * 4)
        self.dctr, self.dvec = al(ne * 24), al(ne * 24)
        for p in (self.dL, self.dP, self.dZ, self.dLU, self.db, self.dx):
            if not p:
                raise RuntimeError("device allocation failed")
        e = np.ascontiguousarray(m.edges())
        lib.peec_gb300_copy_to_device(self.dedges, e.ctypes.data, e.nbytes)
        ctr = np.ascontiguousarray(m.array("edge_centers", (ne, 3)))
        vec = np.ascontiguousarray(m.array("edge_vectors", (ne, 3)))
        lib.peec_gb300_copy_to_device(self.dctr, ctr.ctypes.data, ctr.nbytes)
        lib.peec_gb300_copy_to_device(self.dvec, vec.ctypes.data, vec.nbytes)
        self.lo = abi.InductanceOptions()
        lib.inductance_options_default(C.byref(self.lo), 1)
        self.po = abi.PotentialOptions()
        lib.potential_options_default(C.byref(self.po), 1)
        self.stL, self.stP = abi.PeecAssemblyStats(), abi.PeecAssemblyStats()
        self.kh = (C.c_double * 3)(0.0, 0.0, -1.0)
        self.eh = (C.c_double * 3)(1.0, 0.0, 0.0)
        self.k0 = 2 * np.pi * FREQ / C0
        self.phase_ms = {}
        self.phase_ms_mixed = {}
        self.mixed_iters = 0

    def step(self, timed_phases=False):
        lib, m, n = self.lib, self.m, self.n
        ev = [lib.peec_gb300_event_record()]
        assert lib.peec_gb300_inductance_device(C.byref(m.mesh), C.byref(m.dual), C.byref(self.lo), self.dL,
                                                C.byref(self.stL)) == 0
        ev.append(lib.peec_gb300_event_record())
        assert lib.peec_gb300_potential_device(C.byref(m.mesh), C.byref(m.dual), C.byref(self.po), self.dP,
                                               C.byref(self.stP)) == 0
        ev.append(lib.peec_gb300_event_record())
        assert lib.peec_gb300_harmonic_build_device(self.dL, self.dP, self.dedges, None, self.ne, self.nv, FREQ,
                                                    self.dZ) == 0
        ev.append(lib.peec_gb300_event_record())
        assert lib.peec_gb300_copy_device(self.dLU, self.dZ, n * n * 16) == 0  # Z stays for the residual
        ev.append(lib.peec_gb300_event_record())
        scale, col = C.c_double(), C.c_int()
        s = lib.peec_gb300_complex_lu_factor_device(self.dLU, n, 1e-14, self.dpiv, self.dperm, self.drow, self.dcol,
                                                    C.byref(scale), C.byref(col))
        assert s == 0, "factorisation failed"
        ev.append(lib.peec_gb300_event_record())
        assert lib.peec_gb300_plane_wave_rhs_device(self.dctr, self.dvec, self.ne, self.nv, self.kh, self.eh,
                                                    self.k0, self.db) == 0
        assert lib.peec_gb300_complex_lu_solve_device(self.dLU, self.dperm, self.drow, self.dcol, n, self.db,
                                                      self.dx, 1) == 0
        ev.append(lib.peec_gb300_event_record())
        out = (C.c_double * 3)()
        assert lib.peec_gb300_backward_error_device(self.dZ, n, self.dx, self.db, 1, out) == 0
        ev.append(lib.peec_gb300_event_record())
        names = ["assemble_Lp", "assemble_P", "mna_fill", "copy_Z_for_factor", "complex_lu", "rhs_solve",
                 "backward_error"]
        for k, name in enumerate(names):
            self.phase_ms.setdefault(name, []).append(lib.peec_gb300_event_elapsed_ms(ev[k], ev[k + 1]))
        for tag, st in (("Lp", self.stL), ("P", self.stP)):
            for f in ("ms_prepare", "ms_near", "ms_far"):
                self.phase_ms.setdefault(tag + "_" + f[3:], []).append(getattr(st, f))
        self.work = {"Lp_near_pairs": self.stL.near_pairs, "Lp_near_pairs_evaluated": self.stL.near_pairs_evaluated,
                     "Lp_near_pairs_reevaluated": self.stL.near_pairs_reevaluated,
                     "P_near_pairs_evaluated": self.stP.near_pairs_evaluated,
                     "Lp_potential_evals": self.stL.potential_evaluations,
                     "Lp_far_point_pairs": self.stL.far_point_pairs,
                     "P_near_pairs": self.stP.near_pairs, "P_potential_evals": self.stP.potential_evaluations,
                     "P_far_point_pairs": self.stP.far_point_pairs}
        for e in ev:
            lib.peec_gb300_event_destroy(e)
        return out[0]

    def step_mixed(self):
        """The mixed-precision solve of the same system: FP32 far field (the
        near field stays FP64), FP32 LU with split-BF16x3 tcgen05 trailing
        updates, FP64 iterative refinement to the same 1e-10 gate."""
        lib, m, n = self.lib, self.m, self.n
        prev = lib.peec_gb300_set_far_precision(2)
        ev = [lib.peec_gb300_event_record()]
        assert lib.peec_gb300_inductance_device(C.byref(m.mesh), C.byref(m.dual), C.byref(self.lo), self.dL,
                                                C.byref(self.stL)) == 0
        ev.append(lib.peec_gb300_event_record())
        assert lib.peec_gb300_potential_device(C.byref(m.mesh), C.byref(m.dual), C.byref(self.po), self.dP,
                                               C.byref(self.stP)) == 0
        ev.append(lib.peec_gb300_event_record())
        lib.peec_gb300_set_far_precision(prev)
        assert lib.peec_gb300_harmonic_build_device(self.dL, self.dP, self.dedges, None, self.ne, self.nv, FREQ,
                                                    self.dZ) == 0
        assert lib.peec_gb300_plane_wave_rhs_device(self.dctr, self.dvec, self.ne, self.nv, self.kh, self.eh,
                                                    self.k0, self.db) == 0
        ev.append(lib.peec_gb300_event_record())
        be, it = C.c_double(), C.c_int()
        s = lib.peec_gb300_complex_solve_mixed_device(self.dZ, n, self.db, self.dx, 1, 1e-10, 30, C.byref(be),
                                                      C.byref(it))
        assert s == 0, "mixed solve did not converge: status %d, backward error %g" % (s, be.value)
        ev.append(lib.peec_gb300_event_record())
        names = ["assemble_Lp", "assemble_P", "mna_fill_rhs", "mixed_solve"]
        for k, name in enumerate(names):
            self.phase_ms_mixed.setdefault(name, []).append(lib.peec_gb300_event_elapsed_ms(ev[k], ev[k + 1]))
        for tag, st in (("Lp", self.stL), ("P", self.stP)):
            for f in ("ms_near", "ms_far"):
                self.phase_ms_mixed.setdefault(tag + "_" + f[3:], []).append(getattr(st, f))
        mp, mf, mr = C.c_double(), C.c_double(), C.c_double()
        self.mixed_iters = lib.peec_gb300_mixed_timing(C.byref(mp), C.byref(mf), C.byref(mr))
        for name, v in (("solve_prepare", mp), ("solve_factor", mf), ("solve_refine", mr)):
            self.phase_ms_mixed.setdefault(name, []).append(v.value)
        for e in ev:
            lib.peec_gb300_event_destroy(e)
        return be.value

    def free(self):
        for p in (self.dL, self.dP, self.dZ, self.dLU, self.db, self.dx, self.dpiv, self.dperm, self.drow, self.dcol,
                  self.dedges, self.dctr, self.dvec):
            self.lib.peec_gb300_device_free(p)


def transient_leg(lib, ds, n_steps):
    """Lightning transient on the same box (PEC, trapezoidal, dt 0.1 us): the
    10/350 us 100 kA first stroke injected at a seeded top-face node and
    returned at node 0, every step's right-hand side and solve on the device
    with the factorised system resident.  CUDA-event timed."""
    from peeeeeeeeeeeeeeeeeeec_gb300.workloads import LIGHTNING_10_350 as W
    m = ds.m
    xyz = m.array("xyz", (m.n_nodes, 3))
    top = np.flatnonzero(xyz[:, 2] >= xyz[:, 2].max() - 1e-12)
    strike = int(np.random.default_rng(3).choice(top))
    h = C.c_void_p()
    e0 = lib.peec_gb300_event_record()
    s = lib.peec_gb300_transient_create(ds.dL, ds.dP, ds.dedges, None, ds.ne, ds.nv, 2, 1e-7, C.byref(h))
    e1 = lib.peec_gb300_event_record()
    lib.peec_gb300_synchronize()
    assert s == 0, "transient system failed"
    create_ms = lib.peec_gb300_event_elapsed_ms(e0, e1)
    al = lib.peec_gb300_device_alloc
    dI, dV = al(ds.ne * 8), al(ds.nv * 8)
    probes = np.array([strike, 0], dtype=np.int32)
    dpn, dpr = al(8), al(n_steps * 2 * 8)
    lib.peec_gb300_copy_to_device(dpn, probes.ctypes.data, probes.nbytes)
    out = {}
    for rep in range(2):  # the first run warms the pools
        z = np.zeros(max(ds.ne, ds.nv))
        lib.peec_gb300_copy_to_device(dI, z.ctypes.data, ds.ne * 8)
        lib.peec_gb300_copy_to_device(dV, z.ctypes.data, ds.nv * 8)
        steps = n_steps if rep else 16
        l0 = lib.peec_gb300_launch_count()
        e0 = lib.peec_gb300_event_record()
        s = lib.peec_gb300_transient_lightning(h, W["K"], W["alpha"], W["beta"], W["delay"], strike, 0, 0, steps,
                                               dI, dV, dpn, 2, None, 0, dpr)
        e1 = lib.peec_gb300_event_record()
        lib.peec_gb300_synchronize()
        assert s == 0, "transient run failed"
        ms = lib.peec_gb300_event_elapsed_ms(e0, e1)
        out = {"value": steps / (ms / 1e3), "unit": "steps/s", "ms_per_step": ms / steps, "steps": steps,
               "system_create_ms": create_ms, "gpu_launches": int(lib.peec_gb300_launch_count() - l0),
               "scheme": "trapezoidal", "dt_s": 1e-7, "strike_node": strike, "return_node": 0,
               "source": "10/350 us, 100 kA: K %.6g A, alpha %.6g 1/s, beta %.6g 1/s" % (W["K"], W["alpha"],
                                                                                     W["beta"])}
    V = np.zeros((n_steps, 2))
    lib.peec_gb300_copy_to_host(V.ctypes.data, dpr, V.nbytes)
    out["peak_strike_node_self_voltage_V"] = float(np.max(np.abs(V[:, 0])))
    lib.peec_gb300_transient_destroy(h)
    for p in (dI, dV, dpn, dpr):
        lib.peec_gb300_device_free(p)
    return out


def rcs_leg(lib, ds, x_mixed):
    """RCS of the solved box (rcs.c:701-1140, dual-patch quadrature, order 6):
    the monostatic direction (+z, the incident wave travels along -z) and a
    360-direction bistatic sweep in the xy plane, for the plain FP64 and the
    mixed solution at once (two solutions, one call); the mixed path's RCS
    error against the FP64 LU solution is stated."""
    n, ne = ds.n, ds.ne
    lib.peec_gb300_copy_device(x_mixed + n * 16, ds.dx, n * 16)  # [mixed, plain]
    ph = np.radians(np.arange(360.0))
    dirs = np.concatenate([[[0.0, 0.0, 1.0]], np.stack([np.cos(ph), np.sin(ph), np.zeros_like(ph)], 1)])
    dirs = np.ascontiguousarray(dirs)
    out = np.zeros((dirs.shape[0], 2, 3), dtype=np.complex128)
    k = ds.k0
    args = (C.byref(ds.m.mesh), C.byref(ds.m.dual), x_mixed, 2, n, k, dirs.ctypes.data_as(ds.abi.c_double_p),
            dirs.shape[0], 6, out.ctypes.data)
    assert lib.peec_gb300_rcs_radiation_device(*args) == 0  # warm
    ts = []
    for _ in range(3):
        t = time.perf_counter()
        assert lib.peec_gb300_rcs_radiation_device(*args) == 0
        ts.append(time.perf_counter() - t)
    xs = np.zeros(2 * n, dtype=np.complex128)
    lib.peec_gb300_copy_to_host(xs.ctypes.data, x_mixed, xs.nbytes)
    Im, Ip = xs[:ne], xs[n:n + ne]
    cur_err = float(np.max(np.abs(Im - Ip)) / np.max(np.abs(Ip)))
    eta0 = np.sqrt(4e-7 * np.pi / 8.8541878128e-12)
    T = dirs[:, None, :] * np.sum(dirs[:, None, :] * out, axis=2)[:, :, None] - out
    sigma = k * k * eta0 * eta0 * np.sum(np.abs(T) ** 2, axis=2) / (4 * np.pi)  # E0 = 1 V/m
    sm, sp = sigma[:, 0], sigma[:, 1]
    return {"value": 1.0 / statistics.median(ts), "unit": "RCS sweeps/s",
            "ms_per_sweep": 1e3 * statistics.median(ts), "directions": int(dirs.shape[0]), "solutions": 2,
            "edges": ne, "surface_order": 6,
            "monostatic_sigma_dbsm": {"plain_fp64": float(10 * np.log10(sp[0])), "mixed": float(10 * np.log10(sm[0]))},
            "mixed_vs_fp64_max_rel_sigma_err": float(np.max(np.abs(sm - sp) / np.abs(sp))),
            "mixed_vs_fp64_rel_radiation_err": float(np.max(np.abs(out[:, 0] - out[:, 1])) / np.max(np.abs(out[:, 1]))),
            "edge_current_rel_err": cur_err}


def incidence_leg(lib, ds, reps=5):
    """The incidence products (incidence.h) on the resident P and edge list:
    P A^T (Nv x Ne), A P A^T (Ne x Ne), A S (Ne x Nv).  Gathers from P, so
    HBM-bound: algorithmic bytes = the output written + P read once.  Each
    call is timed with events around the device-resident API (its final
    synchronisation included), best of `reps`."""
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            hbm = json.load(f).get("hbm_gbs", 6800.0)
    except (OSError, ValueError):
        hbm = 6800.0
    ne, nv = ds.ne, ds.nv
    out = lib.peec_gb300_device_alloc(max(ne * ne, ne * nv) * 8)
    bad = C.c_longlong()
    calls = {"P_AT": (lambda: lib.peec_gb300_pat_device(ds.dP, ds.dedges, nv, ne, out, C.byref(bad)), nv * ne),
             "A_P_AT": (lambda: lib.peec_gb300_apat_device(ds.dP, ds.dedges, nv, ne, out), ne * ne),
             "A_S": (lambda: lib.peec_gb300_as_device(ds.dP, ds.dedges, nv, ne, out), ne * nv)}
    res = {}
    for name, (call, count) in calls.items():
        best = float("inf")
        for _ in range(reps):
            e0 = lib.peec_gb300_event_record()
            assert call() == 0, name
            e1 = lib.peec_gb300_event_record()
            best = min(best, lib.peec_gb300_event_elapsed_ms(e0, e1))
            lib.peec_gb300_event_destroy(e0)
            lib.peec_gb300_event_destroy(e1)
        nbytes = 8.0 * (count + nv * nv)
        res[name] = {"ms": best, "output_entries": count, "algorithmic_bytes": nbytes,
                     "GB_s": nbytes / best / 1e6, "frac_of_hbm": nbytes / best / 1e6 / hbm}
    lib.peec_gb300_device_free(out)
    res["note"] = "time of the device-resident call including its final synchronisation; peak = measured HBM copy"
    return res


def retarded_leg(lib, ds):
    """The same box and frequency with the retarded kernel exp(-jkR)/R on Lp
    and P (complex assembly, complex MNA fill, mixed solve to the 1e-10
    gate).  CUDA-event timed, one pass after a warm one."""
    m, n = ds.m, ds.n
    k = 2 * np.pi * FREQ / C0
    al = lib.peec_gb300_device_alloc
    dLc, dPc = al(ds.ne * ds.ne * 16), al(ds.nv * ds.nv * 16)
    out = {}
    prev = lib.peec_gb300_set_far_precision(2)  # the mixed path's FP32 far rule
    for rep in range(2):
        ev = [lib.peec_gb300_event_record()]
        assert lib.peec_gb300_inductance_retarded_device(C.byref(m.mesh), C.byref(m.dual), C.byref(ds.lo), k, dLc,
                                                         None) == 0
        ev.append(lib.peec_gb300_event_record())
        assert lib.peec_gb300_potential_retarded_device(C.byref(m.mesh), C.byref(m.dual), C.byref(ds.po), k, dPc,
                                                        None) == 0
        ev.append(lib.peec_gb300_event_record())
        assert lib.peec_gb300_harmonic_build_retarded_device(dLc, dPc, ds.dedges, None, ds.ne, ds.nv, FREQ,
                                                             ds.dZ) == 0
        assert lib.peec_gb300_plane_wave_rhs_device(ds.dctr, ds.dvec, ds.ne, ds.nv, ds.kh, ds.eh, ds.k0,
                                                    ds.db) == 0
        ev.append(lib.peec_gb300_event_record())
        be, it = C.c_double(), C.c_int()
        s = lib.peec_gb300_complex_solve_mixed_device(ds.dZ, n, ds.db, ds.dx, 1, 1e-10, 30, C.byref(be), C.byref(it))
        ev.append(lib.peec_gb300_event_record())
        lib.peec_gb300_synchronize()
        assert s == 0, "retarded mixed solve: status %d" % s
        ms = [lib.peec_gb300_event_elapsed_ms(ev[i], ev[i + 1]) for i in range(4)]
        out = {"value": 1000.0 / sum(ms), "unit": "solves/s", "ms_per_step": sum(ms),
               "phase_ms": {"assemble_Lp_retarded": ms[0], "assemble_P_retarded": ms[1], "mna_fill_rhs": ms[2],
                            "mixed_solve": ms[3]},
               "backward_error": be.value, "refinement_iterations": it.value, "wave_number_per_m": k,
               "kernel": "exp(-jkR)/R: static integral (FP64 near field, FP32 far rule) + "
                         "(exp(-jkR)-1)/R by the far product rule on the FP32 pipes"}
        for e in ev:
            lib.peec_gb300_event_destroy(e)
    lib.peec_gb300_set_far_precision(prev)
    for p in (dLc, dPc):
        lib.peec_gb300_device_free(p)
    return out


def far_precision_leg(lib, ds):
    """Lp + P assembly of the same box with each far-rule arithmetic: native
    FP64 (the reference's), double-float on the FP32 pipes (the plain path's
    default) and FP32 (the mixed path's), CUDA-event timed after a warm
    pass; entry errors against the native FP64 matrices."""
    m = ds.m
    out, ref = {}, None
    prev = lib.peec_gb300_set_far_precision(0)
    for mode, name in ((0, "fp64_native"), (1, "double_float"), (2, "fp32")):
        lib.peec_gb300_set_far_precision(mode)
        for rep in range(2):
            e0 = lib.peec_gb300_event_record()
            assert lib.peec_gb300_inductance_device(C.byref(m.mesh), C.byref(m.dual), C.byref(ds.lo), ds.dL,
                                                    C.byref(ds.stL)) == 0
            e1 = lib.peec_gb300_event_record()
            assert lib.peec_gb300_potential_device(C.byref(m.mesh), C.byref(m.dual), C.byref(ds.po), ds.dP,
                                                   C.byref(ds.stP)) == 0
            e2 = lib.peec_gb300_event_record()
            lib.peec_gb300_synchronize()
            ms = (lib.peec_gb300_event_elapsed_ms(e0, e1), lib.peec_gb300_event_elapsed_ms(e1, e2))
            for e in (e0, e1, e2):
                lib.peec_gb300_event_destroy(e)
        L = np.zeros((ds.ne, ds.ne))
        P = np.zeros((ds.nv, ds.nv))
        lib.peec_gb300_copy_to_host(L.ctypes.data, ds.dL, L.nbytes)
        lib.peec_gb300_copy_to_host(P.ctypes.data, ds.dP, P.nbytes)
        out[name] = {"Lp_ms": ms[0], "P_ms": ms[1], "Lp_far_ms": ds.stL.ms_far, "P_far_ms": ds.stP.ms_far}
        if ref is None:
            ref = (L, P)
        else:
            for tag, a, b in (("Lp", L, ref[0]), ("P", P, ref[1])):
                nz = b != 0
                out[name][tag + "_max_rel_err_vs_fp64"] = float(np.max(np.abs(a[nz] - b[nz]) / np.abs(b[nz])))
    lib.peec_gb300_set_far_precision(prev)
    out["note"] = ("the plain path (value) uses double_float: FP32-pipe arithmetic carrying ~48 bits, within 1e-12 "
                   "of the reference; fp64_native is the same rule on the FP64 pipe")
    return out


def retarded_plain_leg(lib, ds):
    """One plain FP64 solve of the retarded system (complex Lp / P with
    exp(-jkR)/R: static part double-float far rule + FP64 near field,
    retardation correction on the FP32 pipes; complex FP64 LU), after the
    mixed retarded leg has warmed the kernels.  CUDA-event timed."""
    m, n = ds.m, ds.n
    k = 2 * np.pi * FREQ / C0
    al = lib.peec_gb300_device_alloc
    dLc, dPc = al(ds.ne * ds.ne * 16), al(ds.nv * ds.nv * 16)
    ev = [lib.peec_gb300_event_record()]
    assert lib.peec_gb300_inductance_retarded_device(C.byref(m.mesh), C.byref(m.dual), C.byref(ds.lo), k, dLc,
                                                     None) == 0
    assert lib.peec_gb300_potential_retarded_device(C.byref(m.mesh), C.byref(m.dual), C.byref(ds.po), k, dPc,
                                                    None) == 0
    ev.append(lib.peec_gb300_event_record())
    assert lib.peec_gb300_harmonic_build_retarded_device(dLc, dPc, ds.dedges, None, ds.ne, ds.nv, FREQ, ds.dZ) == 0
    assert lib.peec_gb300_copy_device(ds.dLU, ds.dZ, n * n * 16) == 0
    assert lib.peec_gb300_plane_wave_rhs_device(ds.dctr, ds.dvec, ds.ne, ds.nv, ds.kh, ds.eh, ds.k0, ds.db) == 0
    ev.append(lib.peec_gb300_event_record())
    scale, col = C.c_double(), C.c_int()
    assert lib.peec_gb300_complex_lu_factor_device(ds.dLU, n, 1e-14, ds.dpiv, ds.dperm, ds.drow, ds.dcol,
                                                   C.byref(scale), C.byref(col)) == 0
    assert lib.peec_gb300_complex_lu_solve_device(ds.dLU, ds.dperm, ds.drow, ds.dcol, n, ds.db, ds.dx, 1) == 0
    ev.append(lib.peec_gb300_event_record())
    out3 = (C.c_double * 3)()
    assert lib.peec_gb300_backward_error_device(ds.dZ, n, ds.dx, ds.db, 1, out3) == 0
    ms = [lib.peec_gb300_event_elapsed_ms(ev[i], ev[i + 1]) for i in range(3)]
    for e in ev:
        lib.peec_gb300_event_destroy(e)
    for p in (dLc, dPc):
        lib.peec_gb300_device_free(p)
    return {"value": 1000.0 / sum(ms), "unit": "solves/s", "ms_per_step": sum(ms),
            "phase_ms": {"assemble_Lp_P_retarded": ms[0], "fill_copy_rhs": ms[1], "complex_lu_solve": ms[2]},
            "backward_error": out3[0], "precision": "plain: FP64 LU; static far rule double-float, near field FP64, "
                                                    "retardation correction FP32 pipes"}


def config3(lib, nrhs=720, box=(2.0, 1.0, 0.5, 80, 40, 20)):
    """Config 3: the 2.5 cm box (80 x 40 x 20 cells: Ne 22400, Nv 11202,
    N 33602) at 100 MHz with retarded Lp / P (FP32 far rule, FP64 near
    field) and nrhs plane waves: theta = 90 deg, phi at 1-degree steps,
    theta and phi polarisations (720 = 360 x 2; incident_field.c:110-230
    basis).  The mixed solve of all right-hand sides at once (FP32 LU,
    split-BF16x3 tensor-core updates, blocked many-right-hand-side FP32
    substitution, FP64 refinement with a GEMM-form residual, to the 1e-10
    gate), then the plain FP64 LU of the same Z and its solve of every
    right-hand side as the reference for the current and RCS errors.  One
    JSON line; not part of the default run."""
    from peeeeeeeeeeeeeeeeeeec_gb300.mesh import SynthMesh
    m = SynthMesh.box(*box)
    ds = DeviceSolve(lib, m)
    n, ne, nv = ds.n, ds.ne, ds.nv
    f = 100e6
    k = 2 * np.pi * f / C0
    al = lib.peec_gb300_device_alloc
    dLc, dPc = al(ne * ne * 16), al(nv * nv * 16)
    dB, dX, dXr = al(nrhs * n * 16), al(nrhs * n * 16), al(nrhs * n * 16)
    assert dLc and dPc and dB and dX and dXr
    prev = lib.peec_gb300_set_far_precision(2)
    ev = [lib.peec_gb300_event_record()]
    st = ds.abi.PeecAssemblyStats(), ds.abi.PeecAssemblyStats()
    assert lib.peec_gb300_inductance_retarded_device(C.byref(m.mesh), C.byref(m.dual), C.byref(ds.lo), k, dLc,
                                                     C.byref(st[0])) == 0
    ev.append(lib.peec_gb300_event_record())
    assert lib.peec_gb300_potential_retarded_device(C.byref(m.mesh), C.byref(m.dual), C.byref(ds.po), k, dPc,
                                                    C.byref(st[1])) == 0
    ev.append(lib.peec_gb300_event_record())
    assert lib.peec_gb300_harmonic_build_retarded_device(dLc, dPc, ds.dedges, None, ne, nv, f, ds.dZ) == 0
    phis = np.radians(np.arange(nrhs // 2, dtype=np.float64))
    waves = []
    for ph in phis:  # theta = 90 deg: k_hat = -(cos phi, sin phi, 0)
        kh = (-np.cos(ph), -np.sin(ph), -0.0)
        waves.append((kh, (0.0, 0.0, -1.0)))               # e_theta
        waves.append((kh, (-np.sin(ph), np.cos(ph), 0.0)))  # e_phi
    for q, (kh, eh) in enumerate(waves[:nrhs]):
        assert lib.peec_gb300_plane_wave_rhs_device(ds.dctr, ds.dvec, ne, nv, (C.c_double * 3)(*kh),
                                                    (C.c_double * 3)(*eh), k, dB + q * n * 16) == 0
    ev.append(lib.peec_gb300_event_record())
    lib.peec_gb300_set_far_precision(prev)
    lib.peec_gb300_synchronize()
    asm = [lib.peec_gb300_event_elapsed_ms(ev[i], ev[i + 1]) for i in range(3)]
    for p in (dLc, dPc):
        lib.peec_gb300_device_free(p)
    be, it = C.c_double(), C.c_int()
    lib.peec_gb300_lu_timing_enable(1)
    e0 = lib.peec_gb300_event_record()
    s = lib.peec_gb300_complex_solve_mixed_device(ds.dZ, n, dB, dX, nrhs, 1e-10, 30, C.byref(be), C.byref(it))
    e1 = lib.peec_gb300_event_record()
    lib.peec_gb300_synchronize()
    assert s == 0, "mixed solve failed: %d (backward error %g)" % (s, be.value)
    mixed_ms = lib.peec_gb300_event_elapsed_ms(e0, e1)
    mt = [C.c_double() for _ in range(4)]
    lib.peec_gb300_lu_timing(*[C.byref(x) for x in mt])
    tt = [C.c_double() for _ in range(2)]
    lib.peec_gb300_lu_timing_trailing(*[C.byref(x) for x in tt])
    lib.peec_gb300_lu_timing_enable(0)
    mp, mf, mr = C.c_double(), C.c_double(), C.c_double()
    lib.peec_gb300_mixed_timing(C.byref(mp), C.byref(mf), C.byref(mr))
    # FP64 reference: the plain LU of the same Z, every right-hand side
    assert lib.peec_gb300_copy_device(ds.dLU, ds.dZ, n * n * 16) == 0
    t0 = time.perf_counter()
    scale, col = C.c_double(), C.c_int()
    assert lib.peec_gb300_complex_lu_factor_device(ds.dLU, n, 1e-14, ds.dpiv, ds.dperm, ds.drow, ds.dcol,
                                                   C.byref(scale), C.byref(col)) == 0
    lib.peec_gb300_synchronize()
    t_fp64_factor = time.perf_counter() - t0
    assert lib.peec_gb300_complex_lu_solve_device(ds.dLU, ds.dperm, ds.drow, ds.dcol, n, dB, dXr, nrhs) == 0
    lib.peec_gb300_synchronize()
    t_fp64 = time.perf_counter() - t0
    out3 = (C.c_double * 3)()
    assert lib.peec_gb300_backward_error_device(ds.dZ, n, dXr, dB, nrhs, out3) == 0
    X = np.zeros((nrhs, n), dtype=np.complex128)
    Xr = np.zeros((nrhs, n), dtype=np.complex128)
    lib.peec_gb300_copy_to_host(X.ctypes.data, dX, X.nbytes)
    lib.peec_gb300_copy_to_host(Xr.ctypes.data, dXr, Xr.nbytes)
    cur = np.max(np.abs(X[:, :ne] - Xr[:, :ne]), axis=1) / np.max(np.abs(Xr[:, :ne]), axis=1)
    pot = np.max(np.abs(X[:, ne:] - Xr[:, ne:]), axis=1) / np.max(np.abs(Xr[:, ne:]), axis=1)
    # RCS of the first two right-hand sides (theta and phi polarisation at
    # phi = 0) in 361 directions, mixed against FP64
    x_pair = al(4 * n * 16)
    lib.peec_gb300_copy_device(x_pair, dX, n * 16)
    lib.peec_gb300_copy_device(ds.dx, dXr, n * 16)
    ds.k0 = k
    rcs = rcs_leg(lib, ds, x_pair)
    lib.peec_gb300_device_free(x_pair)
    for p in (dB, dX, dXr):
        lib.peec_gb300_device_free(p)
    bf16 = 1933.8
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as fh:
            bf16 = json.load(fh).get("bf16_tflops", bf16)
    except Exception:
        pass
    tflops = tt[1].value / (tt[0].value * 1e-3) / 1e12 if tt[0].value > 0 else None
    line = {"metric": "config 3 (box %gx%gx%g m, %dx%dx%d cells, 100 MHz, retarded Lp / P, %d plane waves): "
                      "mixed solve" % (box + (nrhs,)),
            "value": nrhs * 1000.0 / mixed_ms, "unit": "right-hand sides solved to the gate per second",
            "n_unknowns": n, "Ne": ne, "Nv": nv, "nrhs": nrhs,
            "assembly_ms": {"Lp_retarded": asm[0], "P_retarded": asm[1], "mna_fill_rhs": asm[2]},
            "mixed_solve_ms": mixed_ms, "mixed_phase_ms": {"prepare": mp.value, "factor": mf.value,
                                                           "refine": mr.value},
            "backward_error": be.value, "refinement_iterations": it.value,
            "lu_phases": {"panel_ms": mt[0].value, "swap_trsm_split_ms": mt[1].value, "tc_update_ms": mt[2].value,
                          "trailing_gemm_ms": tt[0].value, "trailing_gemm_issued_bf16_flops": tt[1].value},
            "trailing_gemm_roofline": {"bound": "tensor", "achieved": tflops, "peak": bf16, "unit": "TFLOP/s",
                                       "frac": tflops / bf16 if tflops else None,
                                       "peak_source": "measured (MEASURED_PEAKS.json, cuBLAS BF16 burst)"},
            "fp64_lu_reference_s": {"factor": t_fp64_factor, "factor_and_solve_all_rhs": t_fp64},
            "fp64_backward_error": out3[0],
            "mixed_vs_fp64_time": t_fp64 / (mixed_ms * 1e-3),
            "errors_vs_fp64_lu": {"edge_current_rel_max_over_rhs": float(cur.max()),
                                  "edge_current_rel_median": float(np.median(cur)),
                                  "node_potential_rel_max_over_rhs": float(pot.max()),
                                  "radiation_vector_rel": rcs["mixed_vs_fp64_rel_radiation_err"],
                                  "sigma_rel_max_over_361_directions": rcs["mixed_vs_fp64_max_rel_sigma_err"]},
            "near_pairs": {"Lp": st[0].near_pairs, "P": st[1].near_pairs},
            "data": "synthetic (seeded box mesh, unit plane waves)", "dtype": "mixed (see metric)"}
    print(json.dumps(line), flush=True)
    ds.free()
    m.close()



def config4(lib, n_meshes=48, n_freqs=64, nrhs=4, workers=4, plain_stride=1):
    """Config 4: n_meshes seeded boxes / plates (sides U(0.2, 2.0) m, cell size
    chosen for N = Ne + Nv ~ U(300, 4000)), each at n_freqs log-spaced
    frequencies from 1 kHz to 100 MHz with nrhs plane waves.  Both arms run
    the meshes largest first on `workers` host threads (one CUDA stream each)
    and time the whole arm on the wall clock: Lp / P assembly included.
      mixed  a sweep plan per mesh (peec_gb300_sweep_*): the autotuner at
             six probe frequencies across the band picks the frequency
             below which the robust graph (BF16x6) runs and the tile width
             of the wide tensor-core updates; the mixed solve recorded into
             CUDA graphs (refinement sweeps past the gate are no-ops) is
             replayed for every frequency;
             systems the fast graph leaves above the gate are replayed
             with the robust graph, then solved again by the precision
             ladder, then the FP64 LU with FP64 refinement
      plain  per system: MNA fill, FP64 complex LU, solve, FP64 iterative
             refinement with that factor to the same gate (every
             plain_stride-th frequency; throughput over the systems run)
    Throughput = systems whose componentwise backward error <= 1e-10 / wall
    time."""
    import concurrent.futures as cf
    from peeeeeeeeeeeeeeeeeeec_gb300 import workloads as W
    pool = W.serving_meshes(seed=11, count=n_meshes, lo=300, hi=4000)
    order = sorted(range(len(pool)), key=lambda i: -(pool[i][0].n_edges + pool[i][0].n_nodes))
    freqs = np.logspace(3.0, 8.0, n_freqs)
    waves = [W.plane_waves(np.random.default_rng(100 + i), nrhs) for i in range(len(pool))]
    lo, po = ds_opts(lib)

    def assemble(m):
        ne, nv = m.n_edges, m.n_nodes
        al = lib.peec_gb300_device_alloc
        d = {"L": al(ne * ne * 8), "P": al(nv * nv * 8), "e": al(ne * 8), "c": al(ne * 24), "v": al(ne * 24)}
        assert lib.peec_gb300_inductance_device(C.byref(m.mesh), C.byref(m.dual), C.byref(lo), d["L"], None) == 0
        assert lib.peec_gb300_potential_device(C.byref(m.mesh), C.byref(m.dual), C.byref(po), d["P"], None) == 0
        for key, arr in (("e", np.ascontiguousarray(m.edges(), dtype=np.int32)),
                         ("c", m.array("edge_centers", (ne, 3))), ("v", m.array("edge_vectors", (ne, 3)))):
            assert lib.peec_gb300_copy_to_device(d[key], np.ascontiguousarray(arr).ctypes.data, arr.nbytes) == 0
        return d

    def free(d):
        for p in d.values():
            lib.peec_gb300_device_free(p)

    def mixed_mesh(i):
        m = pool[i][0]
        ne, nv = m.n_edges, m.n_nodes
        n = ne + nv
        d = assemble(m)
        kh, eh = (np.ascontiguousarray(a) for a in waves[i])
        plan = lib.peec_gb300_sweep_create(d["L"], d["P"], d["e"], None, d["c"], d["v"], ne, nv, nrhs,
                                           kh.ctypes.data_as(ds_abi().c_double_p),
                                           eh.ctypes.data_as(ds_abi().c_double_p), None)
        assert plan, "sweep plan"
        t = ds_abi().PeecSweepTuning()
        ms = C.c_double()
        probes = np.ascontiguousarray(freqs[np.linspace(0, len(freqs) - 1, 6).round().astype(int)])
        assert lib.peec_gb300_sweep_tune(plan, probes.ctypes.data_as(ds_abi().c_double_p), len(probes), C.byref(t),
                                         C.byref(ms)) == 0
        fsplit, rob = C.c_double(), ds_abi().PeecSweepTuning()
        lib.peec_gb300_sweep_split(plan, C.byref(fsplit), C.byref(rob))
        dX = lib.peec_gb300_device_alloc(len(freqs) * nrhs * n * 16)
        be = np.zeros(len(freqs))
        fb = np.zeros(len(freqs), dtype=np.int32)
        f = np.ascontiguousarray(freqs)
        s = lib.peec_gb300_sweep_run(plan, f.ctypes.data_as(ds_abi().c_double_p), len(freqs), 1e-10, dX,
                                     be.ctypes.data_as(ds_abi().c_double_p), fb.ctypes.data_as(ds_abi().c_int_p))
        assert s >= 0, "sweep run failed"
        lib.peec_gb300_sweep_destroy(plan)
        lib.peec_gb300_device_free(dX)
        free(d)
        return {"n": n, "be": be, "fb": fb, "tuning": (t.split_terms, t.sweeps, t.tile_bn), "graph_ms": ms.value,
                "split_hz": fsplit.value, "robust": (rob.split_terms, rob.sweeps)}

    def plain_mesh(i):
        m = pool[i][0]
        ne, nv = m.n_edges, m.n_nodes
        n = ne + nv
        d = assemble(m)
        al = lib.peec_gb300_device_alloc
        dZ, dLU, dB, dX = al(n * n * 16), al(n * n * 16), al(nrhs * n * 16), al(nrhs * n * 16)
        dpiv, dperm, drs, dcs = al(n * 8), al(n * 4), al(n * 8), al(n * 8)
        kh, eh = waves[i]
        bes = []
        for fr in freqs[::plain_stride]:
            assert lib.peec_gb300_harmonic_build_device(d["L"], d["P"], d["e"], None, ne, nv, fr, dZ) == 0
            assert lib.peec_gb300_copy_device(dLU, dZ, n * n * 16) == 0
            scale, col = C.c_double(), C.c_int()
            s = lib.peec_gb300_complex_lu_factor_device(dLU, n, 1e-14, dpiv, dperm, drs, dcs, C.byref(scale),
                                                        C.byref(col))
            if s != 0:
                bes.append(np.inf)
                continue
            for q in range(nrhs):
                kq, eq = (C.c_double * 3)(*kh[q]), (C.c_double * 3)(*eh[q])
                assert lib.peec_gb300_plane_wave_rhs_device(d["c"], d["v"], ne, nv, kq, eq, 2 * np.pi * fr / C0,
                                                            dB + q * n * 16) == 0
            assert lib.peec_gb300_complex_lu_solve_device(dLU, dperm, drs, dcs, n, dB, dX, nrhs) == 0
            be, it = C.c_double(), C.c_int()
            r = lib.peec_gb300_complex_refine_device(dZ, dLU, dperm, drs, dcs, n, dB, dX, nrhs, 1e-10, 10,
                                                     C.byref(be), C.byref(it))
            bes.append(be.value if r >= 0 else np.inf)
        for p in (dZ, dLU, dB, dX, dpiv, dperm, drs, dcs):
            lib.peec_gb300_device_free(p)
        free(d)
        return {"n": n, "be": np.array(bes)}

    out = {"systems": "%d meshes x %d frequencies (1 kHz - 100 MHz, log) x %d plane waves = %d"
                      % (len(pool), len(freqs), nrhs, len(pool) * len(freqs)),
           "unknowns": sorted(m.n_edges + m.n_nodes for m, _ in pool), "workers": workers}
    for arm, fn in (("mixed", mixed_mesh), ("plain", plain_mesh)):
        lib.peec_gb300_synchronize()
        t0 = time.perf_counter()
        with cf.ThreadPoolExecutor(max_workers=workers) as ex:
            res = list(ex.map(fn, order))
        span = time.perf_counter() - t0
        be = np.concatenate([r["be"] for r in res])
        ok = int(np.sum(be <= 1e-10))
        out[arm] = {"value": ok / span, "unit": "systems/s", "systems": int(be.size), "at_gate": ok,
                    "wall_s": span, "max_backward_error": float(np.max(be))}
        if arm == "mixed":
            fb = np.concatenate([r["fb"] for r in res])
            out[arm]["graph_replays_at_gate"] = int(np.sum(fb == 0))
            out[arm]["robust_graph_after_fast"] = int(np.sum(fb == 3))
            out[arm]["fallback_mixed_ladder"] = int(np.sum(fb == 1))
            out[arm]["fallback_fp64"] = int(np.sum(fb == 2))
            out[arm]["tuning"] = {str(r["n"]): {"split_terms": r["tuning"][0], "sweeps": r["tuning"][1],
                                                "tile_bn": r["tuning"][2], "graph_ms_per_system": r["graph_ms"],
                                                "robust_below_hz": r["split_hz"],
                                                "robust_terms_sweeps": list(r["robust"])}
                                  for r in res}
        else:
            out[arm]["frequency_stride"] = plain_stride
    out["mixed_vs_plain"] = out["mixed"]["value"] / out["plain"]["value"]
    for m, _ in pool:
        m.close()
    return out


def ds_abi():
    from peeeeeeeeeeeeeeeeeeec_gb300 import abi
    return abi


def ds_opts(lib):
    abi = ds_abi()
    lo, po = abi.InductanceOptions(), abi.PotentialOptions()
    lib.inductance_options_default(C.byref(lo), 1)
    lib.potential_options_default(C.byref(po), 1)
    return lo, po


def serving_leg(lib, window_s, workers, lightning_steps=4096):
    """Poisson arrivals at 200 requests/s over window_s, two request types:
    70% harmonic requests (seeded boxes / plates of 500-12000 unknowns,
    1-100 MHz, 1-64 plane waves) and 30% lightning runs on the 5 cm box
    (10/350 us 100 kA stroke at a seeded top-face node, returned at node 0,
    lightning_steps trapezoidal steps of 0.1 us on the device-resident
    factor).  Replayed once with the mixed-precision harmonic solve and once
    with the plain FP64 LU through one server (150 GB budget) whose Lp / P
    and transient caches were warmed first.  Latency = completion -
    submission on the server clock, per request type."""
    from peeeeeeeeeeeeeeeeeeec_gb300 import workloads as W
    from peeeeeeeeeeeeeeeeeeec_gb300.mesh import SynthMesh
    from peeeeeeeeeeeeeeeeeeec_gb300.server import Server
    pool = W.serving_meshes(seed=5, count=6)
    box = SynthMesh.box(*BOX)
    box_key = 1000
    xyz = box.array("xyz", (box.n_nodes, 3))
    top = np.flatnonzero(xyz[:, 2] >= xyz[:, 2].max() - 1e-12)
    reqs = W.serving_mix(seed=7, n_meshes=len(pool), rate_hz=200.0, window_s=window_s, top_nodes=top)
    LW = W.LIGHTNING_10_350
    n_l = sum(1 for r in reqs if r[0] == "lightning")
    out = {"arrivals": "Poisson 200/s over %.2f s: %d requests (%d harmonic, %d lightning)"
                       % (window_s, len(reqs), len(reqs) - n_l, n_l),
           "meshes": ["%s, N=%d" % (d, m.n_edges + m.n_nodes) for m, d in pool],
           "lightning": "box %gx%gx%g m (N=%d), %d steps, dt 0.1 us, trapezoidal, 10/350 us 100 kA"
                        % (BOX[0], BOX[1], BOX[2], box.n_edges + box.n_nodes, lightning_steps),
           "workers": workers, "hbm_budget_gb": 150}

    def lightning(srv, strike, steps):
        return srv.submit_transient(box, box_key, steps, (LW["K"], LW["alpha"], LW["beta"], LW["delay"], strike, 0),
                                    scheme=2, dt=1e-7, probe_nodes=[strike])

    with Server(150 << 30, workers) as srv:
        warm = [srv.submit(m, i, 30e6, [[0.0, 0.0, -1.0]], [[1.0, 0.0, 0.0]], mixed=True)
                for i, (m, _) in enumerate(pool)]
        warm.append(lightning(srv, int(top[0]), 8))
        for t in warm:
            srv.wait(t)
        for mode in ("mixed", "plain"):
            t0 = time.perf_counter()
            tickets = []
            for r in reqs:
                d = t0 + r[1] - time.perf_counter()
                if d > 0:
                    time.sleep(d)
                if r[0] == "lightning":
                    tickets.append(("lightning", lightning(srv, r[2], lightning_steps)))
                else:
                    _, _, mi, f, k, e = r
                    tickets.append(("harmonic", srv.submit(pool[mi][0], mi, f, k, e, mixed=(mode == "mixed"))))
            res = [(kind, srv.wait(t)[1]) for kind, t in tickets]
            # per request: type, unknowns, right-hand sides (harmonic), frequency
            # MHz (harmonic), queue wait and service time (s), refinement
            # iterations or steps, fallback rung
            detail = []
            for (kind, r), q in zip(res, reqs):
                if kind == "harmonic":
                    m_ = pool[q[2]][0]
                    detail.append(["h", m_.n_edges + m_.n_nodes, len(q[4]), round(q[3] / 1e6, 2),
                                   round(r["t_start"] - r["t_submit"], 3), round(r["t_end"] - r["t_start"], 3),
                                   r.get("iterations"), r.get("fallback", 0)])
                else:
                    detail.append(["l", box.n_edges + box.n_nodes, 1, None, round(r["t_start"] - r["t_submit"], 3),
                                   round(r["t_end"] - r["t_start"], 3), r.get("iterations"), 0])
            span = max(r["t_end"] for _, r in res) - min(r["t_submit"] for _, r in res)
            ok_h = sum(1 for k, r in res if k == "harmonic" and r["status"] == 0 and r["backward_error"] <= 1e-10)
            ok_l = sum(1 for k, r in res if k == "lightning" and r["status"] == 0)
            per = {}
            for kind in ("harmonic", "lightning"):
                lat = np.array([r["t_end"] - r["t_submit"] for k, r in res if k == kind])
                if lat.size:
                    per[kind] = {"requests": int(lat.size), "p50_latency_s": float(np.percentile(lat, 50)),
                                 "p99_latency_s": float(np.percentile(lat, 99))}
            lat_all = np.array([r["t_end"] - r["t_submit"] for _, r in res])
            hb = [r["backward_error"] for k, r in res if k == "harmonic"]
            out[mode] = {"value": ok_h / span, "unit": "harmonic solves/s", "completed_at_gate": ok_h,
                         "lightning_runs_completed": ok_l, "lightning_runs_per_s": ok_l / span,
                         "requests_per_s": (ok_h + ok_l) / span, "requests": len(res),
                         "p50_latency_s": float(np.percentile(lat_all, 50)),
                         "p99_latency_s": float(np.percentile(lat_all, 99)), "per_type": per, "makespan_s": span,
                         "fallbacks_to_fp64": sum(r.get("fallback", 0) for k, r in res if k == "harmonic"),
                         "max_backward_error": max(hb) if hb else None,
                         "per_request": {"fields": ["type", "unknowns", "rhs", "MHz", "wait_s", "service_s",
                                                    "iterations", "fallback"], "rows": detail}}
    out["mixed_vs_plain"] = out["mixed"]["value"] / out["plain"]["value"]
    for m, _ in pool:
        m.close()
    box.close()
    return out


def drop_in_solve(lib, m, b_host, edges):
    from peeeeeeeeeeeeeeeeeeec_gb300 import abi
    lo = abi.InductanceOptions()
    lib.inductance_options_default(C.byref(lo), 1)
    L = abi.InductanceMatrix()
    assert lib.inductance_compute_matrix(C.byref(m.mesh), C.byref(m.dual), C.byref(lo), C.byref(L)) == 0
    Lh = np.ctypeslib.as_array(L.data, shape=(L.n, L.n))
    po = abi.PotentialOptions()
    lib.potential_options_default(C.byref(po), 1)
    P = abi.PotentialMatrix()
    assert lib.potential_compute_matrix(C.byref(m.mesh), C.byref(m.dual), C.byref(po), C.byref(P)) == 0
    Ph = np.ctypeslib.as_array(P.data, shape=(P.n, P.n))
    Z = host_mna(Lh, Ph, edges, FREQ)
    lib.inductance_free(C.byref(L))
    lib.potential_free(C.byref(P))
    n = Z.shape[0]
    o = abi.ComplexLUOptions()
    lib.complex_lu_options_default(C.byref(o), 1)
    f = abi.ComplexLUFactorization()
    cp = lambda v: C.cast(v.ctypes.data, C.POINTER(abi.Complex))  # noqa: E731
    assert lib.complex_lu_factorize(cp(Z), n, C.byref(o), C.byref(f)) == 0
    x = np.zeros(n, dtype=np.complex128)
    assert lib.complex_lu_solve(C.byref(f), cp(b_host), cp(x)) == 0
    lib.complex_lu_free(C.byref(f))
    # the gate: Z, x and b uploaded, the library's backward error on the
    # device (numpy on the host took 0.28 s of the 2.1 s here)
    dev = [lib.peec_gb300_device_alloc(a.nbytes) for a in (Z, x, b_host)]
    for p, a in zip(dev, (Z, x, b_host)):
        assert lib.peec_gb300_copy_to_device(p, a.ctypes.data, a.nbytes) == 0
    out = (C.c_double * 3)()
    assert lib.peec_gb300_backward_error_device(dev[0], n, dev[1], dev[2], 1, out) == 0
    for p in dev:
        lib.peec_gb300_device_free(p)
    be = out[0]
    h2d = 2 * Z.nbytes + 2 * b_host.nbytes + x.nbytes + geometry_bytes(m) * 2
    d2h = (Lh.size + Ph.size) * 8 + Z.nbytes + n * 8 + x.nbytes
    return be, h2d, d2h


def geometry_bytes(m):
    """Patch corners + per-region data uploaded by one assembly call."""
    np_e = sum(m.dual.edge_patches[r].count for r in range(m.n_edges))
    np_v = sum(m.dual.node_patches[r].count for r in range(m.n_nodes))
    return (np_e + np_v) * (96 + 8) // 2 + (m.n_edges + m.n_nodes) * 40 // 2


# ---------------------------------------------------------------------
# CPU: the reference's own code (or the oracle port) on a bounded sample
# ---------------------------------------------------------------------
def cpu_reference(prefer="reference"):
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    from cpu_baseline import CpuReference
    return CpuReference(prefer)


def run_reference(args, rank, world):
    """The reference's CPU path on this host's cores (rank 0 only): each step
    is one bounded sample of the 5 cm box solve (oracle/cpu_baseline.py),
    extrapolated to one full solve; value = 1 / median extrapolated seconds.
    ms_per_step is the measured wall time of one sample.  After the timed
    steps, one smaller sample on one thread."""
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    from cpu_baseline import run_steps
    impl = cpu_reference()
    threads = os.cpu_count()
    t0 = time.perf_counter()
    impl.mesh(BOX)
    impl.solve_chain(FREQ, threads)  # set-up: the 2102-unknown system's Lp / P
    setup_s = time.perf_counter() - t0
    sec, parts, measured, desc = run_steps(impl, BOX, FREQ, threads, args.steps, args.warmup)
    sec1, parts1, measured1, desc1 = run_steps(impl, BOX, FREQ, 1, 1, 0, rows=(8, 8))
    v = 1.0 / sec
    m = impl.mesh(BOX)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "solves/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": measured * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "n_unknowns": m.n_edges + m.n_nodes, "Ne": m.n_edges,
                       "Nv": m.n_nodes, "frequency_hz": FREQ, "parallelism": "cpu (%d threads)" % threads,
                       "note": "each step: one bounded sample (ms_per_step is its measured wall time), "
                               "extrapolated to one full solve (value = 1 / median extrapolated seconds)"},
            "solve_seconds_extrapolated": sec, "setup_seconds": setup_s,
            "cpu_baseline": {"value": v, "unit": "solves/s", "cores": threads, "kind": impl.kind,
                             "library": os.path.relpath(impl.path, REPO), "sample": desc,
                             "phase_seconds": {k: round(x, 3) for k, x in parts.items()},
                             "one_thread": {"value": 1.0 / sec1, "unit": "solves/s", "cores": 1,
                                            "solve_seconds_extrapolated": sec1,
                                            "phase_seconds": {k: round(x, 3) for k, x in parts1.items()},
                                            "sample": desc1, "sample_seconds": measured1}},
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--box", default=None, help="lx,ly,lz,nx,ny,nz (default: the 5 cm box)")
    ap.add_argument("--transient-steps", type=int, default=4096)
    ap.add_argument("--no-retarded", action="store_true")
    ap.add_argument("--serve-window", type=float, default=0.2, help="seconds of Poisson arrivals (0: skip)")
    ap.add_argument("--serve-workers", type=int, default=8)
    ap.add_argument("--batch", default="12x64",
                    help="meshes x frequencies of the batched leg, the config-4 sweep on fewer meshes (0: skip)")
    ap.add_argument("--config4", default=None,
                    help="only the batched sweep, meshes x frequencies (e.g. 48x64): sweep graphs vs plain FP64 LU")
    ap.add_argument("--config4-plain-stride", type=int, default=4,
                    help="the plain arm of the sweep legs solves every k-th frequency (throughput over those)")
    ap.add_argument("--config4-workers", type=int, default=32, help="host threads (streams) of both config-4 arms")
    ap.add_argument("--config3-box", default="2.0,1.0,0.5,80,40,20",
                    help="lx,ly,lz,nx,ny,nz of --config3 (a smaller box for profiling runs)")
    ap.add_argument("--config3-rhs", type=int, default=720)
    ap.add_argument("--no-far", action="store_true", help="skip the far-rule precision leg")
    ap.add_argument("--config3", action="store_true",
                    help="only the 2.5 cm retarded box (33602 unknowns): mixed solve + FP64 LU reference")
    args = ap.parse_args()
    if args.box:
        set_box(args.box)
    rank, world, local = dist_env()
    dist = None
    if world > 1:
        import torch.distributed as dist_mod
        dist_mod.init_process_group("gloo")
        dist = dist_mod
    if args.impl == "reference":
        run_reference(args, rank, world)
        if dist:
            dist.barrier()
            dist.destroy_process_group()
        return
    os.environ.setdefault("CUDA_VISIBLE_DEVICES", str(local))
    # the serving and sweep legs run up to 32 host threads, one stream each:
    # as many hardware work queues, so independent streams do not share one
    # (read when the CUDA context is created)
    os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
    from peeeeeeeeeeeeeeeeeeec_gb300 import abi
    lib = abi.load_gpu_lib()
    if not lib.peec_gb300_device_ready():
        raise RuntimeError("no CUDA device")
    if args.config3:
        if rank == 0:
            v = args.config3_box.split(",")
            config3(lib, args.config3_rhs, (float(v[0]), float(v[1]), float(v[2]), int(v[3]), int(v[4]), int(v[5])))
        return
    if args.config4:
        if rank == 0:
            nm, nf = (int(v) for v in args.config4.split("x"))
            res = config4(lib, nm, nf, workers=args.config4_workers, plain_stride=args.config4_plain_stride)
            print(json.dumps({"metric": "config 4 batched sweep: systems/s at <=1e-10 backward error",
                              "value": res["mixed"]["value"], "unit": "systems/s", "batched": res,
                              "data": "synthetic (seeded meshes and plane waves)"}), flush=True)
        return
    m = make_mesh()
    ds = DeviceSolve(lib, m)
    for _ in range(args.warmup):
        be = ds.step()
        assert be <= 1e-10, "backward error %g above the gate" % be
    ds.phase_ms = {}
    clocks = ClockSampler(local)
    if dist:
        dist.barrier()
    lib.peec_gb300_synchronize()
    launches0 = lib.peec_gb300_launch_count()
    clocks.start()
    e0 = lib.peec_gb300_event_record()
    bes = []
    for _ in range(args.steps):
        bes.append(ds.step())
    e1 = lib.peec_gb300_event_record()
    lib.peec_gb300_synchronize()
    clk = clocks.stop()
    total_ms = lib.peec_gb300_event_elapsed_ms(e0, e1)
    launches = lib.peec_gb300_launch_count() - launches0
    if dist:
        import torch
        t = torch.tensor([total_ms], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    assert max(bes) <= 1e-10, "backward error above the gate"
    ms_step = total_ms / args.steps
    value = world * args.steps / (total_ms / 1e3)
    phases = {k: statistics.median(v) for k, v in ds.phase_ms.items()}
    # end to end through the drop-in ABI, host buffers: the same workload,
    # measured next to the device-timed steps (before the other legs)
    e2e = None
    if not args.no_e2e:
        b_host = plane_wave(m)
        edges = m.edges()
        drop_in_solve(lib, m, b_host, edges)  # warm (registry, pools)
        ts = []
        for _ in range(max(1, min(args.steps, 2))):
            t = time.perf_counter()
            be, h2d, d2h = drop_in_solve(lib, m, b_host, edges)
            ts.append(time.perf_counter() - t)
            assert be <= 1e-10
        e2e = {"value": world / statistics.median(ts), "unit": "solves/s", "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "backward_error": be}
    # mixed-precision path on the same system (CUDA-event timed, same gate)
    mixed = None
    if not args.no_mixed:
        for _ in range(args.warmup):
            ds.step_mixed()
        ds.phase_ms_mixed = {}
        msteps = max(args.steps, 10)  # 0.15 s a solve: ten or more steps steady the mean
        lib.peec_gb300_synchronize()
        marks = [lib.peec_gb300_event_record()]
        mbes = []
        for _ in range(msteps):
            mbes.append(ds.step_mixed())
            marks.append(lib.peec_gb300_event_record())
        each = [lib.peec_gb300_event_elapsed_ms(marks[i], marks[i + 1]) for i in range(msteps)]
        mixed_ms = lib.peec_gb300_event_elapsed_ms(marks[0], marks[-1]) / msteps
        split_terms = lib.peec_gb300_mixed_split_terms()
        for e in marks:
            lib.peec_gb300_event_destroy(e)
        # one more mixed solve with the factorisation's phase timing on
        lib.peec_gb300_lu_timing_enable(1)
        ds.step_mixed()
        mt = [C.c_double() for _ in range(4)]
        lib.peec_gb300_lu_timing(*[C.byref(x) for x in mt])
        tt = [C.c_double() for _ in range(2)]
        lib.peec_gb300_lu_timing_trailing(*[C.byref(x) for x in tt])
        lib.peec_gb300_lu_timing_enable(0)
        mixed_lu = {"panel_ms": mt[0].value, "swap_trsm_split_ms": mt[1].value, "tc_update_ms": mt[2].value,
                    "tc_update_issued_bf16_flops": mt[3].value, "trailing_gemm_ms": tt[0].value,
                    "trailing_gemm_issued_bf16_flops": tt[1].value}
        mixed = {"value": world * 1000.0 / mixed_ms, "unit": "solves/s", "ms_per_step": mixed_ms, "steps": msteps,
                 "ms_per_step_min": min(each), "ms_per_step_median": statistics.median(each),
                 "vs_plain_fp64_gpu": (1000.0 / mixed_ms) / (1000.0 / ms_step),
                 "backward_error": max(mbes), "refinement_iterations": ds.mixed_iters,
                 "split_bf16_terms": split_terms, "lu_phases": mixed_lu,
                 "phase_ms": {k: statistics.median(v) for k, v in ds.phase_ms_mixed.items()},
                 "precision": "FP32 far field (near field FP64), FP32 LU with split-BF16x3 tcgen05 trailing "
                              "update (FP32 accumulation; BF16x6 when refinement stalls), FP64 iterative "
                              "refinement"}
    # keep the mixed solution for the RCS comparison
    x_mixed = None
    if mixed is not None:
        x_mixed = lib.peec_gb300_device_alloc(2 * ds.n * 16)
        lib.peec_gb300_copy_device(x_mixed, ds.dx, ds.n * 16)
    # one more solve, outside the timed region, with the LU phase timing on
    lib.peec_gb300_lu_timing_enable(1)
    ds.step()
    lu_t = [C.c_double() for _ in range(4)]
    lib.peec_gb300_lu_timing(*[C.byref(x) for x in lu_t])
    lib.peec_gb300_lu_timing_enable(0)
    lu_phases = {"panel_ms": lu_t[0].value, "swap_trsm_ms": lu_t[1].value, "update_ms": lu_t[2].value,
                 "update_flops": lu_t[3].value}
    rcs = None
    if x_mixed:
        rcs = rcs_leg(lib, ds, x_mixed)
        lib.peec_gb300_device_free(x_mixed)
    incidence = incidence_leg(lib, ds)
    p64, p32 = C.c_double(), C.c_double()
    lib.peec_gb300_pipe_peaks(C.byref(p64), C.byref(p32))
    transient = transient_leg(lib, ds, args.transient_steps) if args.transient_steps > 0 else None
    retarded = None if args.no_retarded else retarded_leg(lib, ds)
    if retarded is not None:
        retarded["plain_fp64_solve"] = retarded_plain_leg(lib, ds)
    far_precision = None if args.no_far else far_precision_leg(lib, ds)
    ds.free()
    serving = serving_leg(lib, args.serve_window, args.serve_workers) if args.serve_window > 0 else None
    batched = None
    if args.batch not in ("0", ""):
        bm, bf = (int(v) for v in args.batch.split("x"))
        batched = config4(lib, bm, bf, workers=args.config4_workers, plain_stride=args.config4_plain_stride)


    cpu = None
    if rank == 0 and not args.no_cpu:
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        from cpu_baseline import run_steps
        impl = cpu_reference()
        sec, parts, measured, desc = run_steps(impl, BOX, FREQ, os.cpu_count(), 1, 0)
        cpu = {"value": 1.0 / sec, "unit": "solves/s", "cores": os.cpu_count(), "kind": impl.kind,
               "library": os.path.relpath(impl.path, REPO), "sample": desc,
               "sample_seconds": round(measured, 2),
               "phase_seconds": {k: round(v, 2) for k, v in parts.items()}}

    roofs = roofline(phases, lu_phases, m, p64.value, p32.value, ds.work)
    if mixed and mixed["lu_phases"].get("tc_update_ms"):
        ml = mixed["lu_phases"]
        bf16 = 1933.8
        try:
            with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
                bf16 = json.load(f).get("bf16_tflops", bf16)
        except Exception:
            pass
        if ml.get("trailing_gemm_ms"):
            a = ml["trailing_gemm_issued_bf16_flops"] / (ml["trailing_gemm_ms"] * 1e-3) / 1e12
            roofs.append({"kernel": "k_tc_gemm_cplx_persistent (mixed LU outer-block trailing update, tcgen05 "
                                    "split-BF16x3)",
                          "bound": "tensor", "achieved": a, "peak": bf16, "unit": "TFLOP/s", "frac": a / bf16,
                          "ms": ml["trailing_gemm_ms"], "traffic": load_traffic().get("k_tc_gemm_cplx_persistent"),
                          "peak_source": "measured (MEASURED_PEAKS.json, cuBLAS BF16 burst)",
                          "note": "CUDA events around the 32 outer-block trailing GEMM launches of one factorisation; "
                                  "issued BF16 flops 2 accumulators x 2 x m x n x 1536 each"})
        a = ml["tc_update_issued_bf16_flops"] / (ml["tc_update_ms"] * 1e-3) / 1e12
        roofs.append({"kernel": "all tensor-core updates of the mixed LU (panel-internal K = 192 updates, U12, "
                                "trailing; with their BF16 operand splits)",
                      "bound": "tensor", "achieved": a, "peak": bf16, "unit": "TFLOP/s", "frac": a / bf16,
                      "ms": ml["tc_update_ms"], "traffic": None,
                      "peak_source": "measured (MEASURED_PEAKS.json, cuBLAS BF16 burst)",
                      "note": "issued BF16 flops: 2 accumulators x 2 x m x n x 6 x (block width)"})
    if mixed and mixed.get("phase_ms"):
        # the mixed path's FP32 far rule against the issue bound of its point
        # loop: 7.25 warp instructions per 32 point pairs (a shared-memory
        # broadcast, an add, three FMAs, the reciprocal square root, the
        # weighted FMA, a quarter of the weights' load) at one warp
        # instruction per clock per SM sub-partition (the FP32 FMA probe's
        # rate / 32 lanes); ncu shows the MUFU pipe at a quarter of its peak
        for tag in ("Lp", "P"):
            ms = mixed["phase_ms"].get(tag + "_far")
            pairs = ds.work.get(tag + "_far_point_pairs")
            if ms and pairs and p32.value:
                a = pairs / (ms * 1e-3) / 1e9
                pk = p32.value * 1e12 / 2 / 32 * (32 / 7.25) / 1e9
                roofs.append({"kernel": "k_assemble_tiles far rule, %s (FP32, mixed path)" % tag, "bound": "issue",
                              "achieved": a, "peak": pk, "unit": "Gpoint-pairs/s", "frac": a / pk, "ms": ms,
                              "traffic": None,
                              "peak_source": "measured FP32 FMA rate / 2 / 32 lanes x 32 / 7.25 point pairs per "
                                             "warp instruction (the point loop's instruction count)"})
    if transient and transient.get("ms_per_step"):
        ne_, nv_ = m.n_edges, m.n_nodes
        nt_ = ne_ + nv_
        # M^-1 as float pairs (8 B) once, its high parts (4 B) once; Lp and
        # A S as float pairs twice
        b = 12.0 * nt_ * nt_ + 16.0 * (ne_ * ne_ + ne_ * nv_)
        a = b / (transient["ms_per_step"] * 1e-3) / 1e9
        hbm_pk = 6800.0
        try:
            with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
                hbm_pk = json.load(f).get("hbm_gbs", hbm_pk)
        except Exception:
            pass
        roofs.append({"kernel": "transient step (k_transient_rhs, 2 x k_minv_apply, k_transient_resid)",
                      "bound": "hbm", "achieved": a, "peak": hbm_pk, "unit": "GB/s", "frac": a / hbm_pk,
                      "ms": transient["ms_per_step"], "traffic": load_traffic().get("k_minv_apply"),
                      "peak_source": "measured (MEASURED_PEAKS.json)",
                      "note": "algorithmic bytes per step: 12 N^2 (M^-1 as float pairs, then its high parts) + "
                              "16 (Ne^2 + Ne Nv) (Lp, A S as float pairs, twice)"})
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": WORKLOAD, "n_unknowns": m.n_edges + m.n_nodes, "Ne": m.n_edges,
                           "Nv": m.n_nodes, "frequency_hz": FREQ, "parallelism": "replicas" if world > 1 else "1gpu",
                           "l2": "inputs larger than L2 (Z is %.2f GB)" % ((m.n_edges + m.n_nodes) ** 2 * 16 / 1e9),
                           "retardation": "none on the headline (quasi-static, as the reference); "
                                          "the retarded kernel is the 'retarded' leg"},
                "phase_ms": phases, "work": ds.work, "backward_error": max(bes), "gpu_launches": int(launches),
                "clocks": clk, "e2e": e2e, "cpu_baseline": cpu,
                "lu_phases": lu_phases, "mixed": mixed, "serving": serving, "batched": batched, "transient": transient, "retarded": retarded,
                "rcs": rcs, "incidence": incidence, "far_precision": far_precision,
                "pipe_peaks_tflops": {"fp64": p64.value, "fp32": p32.value,
                                      "how": "FMA loops on this GPU (the pool's measured peaks cover HBM and BF16)"},
                "rooflines": roofs, "roofline": max(roofs, key=lambda r: r["ms"]) if roofs else None}
        print(json.dumps(line))
    if dist:
        dist.barrier()
        dist.destroy_process_group()


DF_FP32_INSTR_PER_PAIR = 106  # double-float far rule: FP32 instructions per point pair (csrc/assembly.cu)


def load_traffic():
    """DRAM bytes per launch of the profiled kernels, from the committed ncu
    summary (profiles/traffic.json), or {} if absent."""
    path = os.path.join(REPO, "profiles", "traffic.json")
    try:
        with open(path) as f:
            return json.load(f)
    except Exception:
        return {}


def roofline(phases, lu, m, fp64_peak, fp32_peak, work):
    """The dominant kernel of the step against the pipe that bounds it, plus
    the other phases.  Peaks: HBM from MEASURED_PEAKS.json, FP64/FP32 pipes
    measured by bench.py's own FMA loops on the same GPU."""
    peaks = {}
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except Exception:
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    ne, nv = m.n_edges, m.n_nodes
    n = ne + nv
    traffic = load_traffic()
    out = []
    if lu.get("update_ms"):
        a = lu["update_flops"] / (lu["update_ms"] * 1e-3) / 1e12
        out.append({"kernel": "k_gemm_cplx (complex LU trailing update, FP64 FMA)", "bound": "fp64",
                    "achieved": a, "peak": fp64_peak, "unit": "TFLOP/s", "frac": a / fp64_peak if fp64_peak else None,
                    "ms": lu["update_ms"], "traffic": traffic.get("k_gemm_cplx"),
                    "peak_source": "measured (bench FMA loop)"})
    far_pairs = {"Lp": work.get("Lp_far_point_pairs", 0), "P": work.get("P_far_point_pairs", 0)}
    for tag in ("Lp", "P"):
        ms = phases.get(tag + "_far")
        if ms:
            a = far_pairs[tag] / (ms * 1e-3) / 1e9
            pk = fp32_peak * 1e12 / 2 / DF_FP32_INSTR_PER_PAIR / 1e9
            out.append({"kernel": "k_assemble_tiles far rule, %s (double-float on the FP32 pipe)" % tag,
                        "bound": "fp32", "achieved": a, "peak": pk, "unit": "Gpoint-pairs/s", "frac": a / pk,
                        "ms": ms, "traffic": traffic.get("k_assemble_tiles"),
                        "peak_source": "measured FP32 FMA rate / %d FP32 instructions per point pair"
                                       % DF_FP32_INSTR_PER_PAIR})
    if phases.get("mna_fill"):
        b = 16.0 * n * n + 8.0 * ne * ne + 8.0 * nv * nv  # Z written, Lp read, P read (its rows gathered)
        a = b / (phases["mna_fill"] * 1e-3) / 1e9
        out.append({"kernel": "k_harmonic_fill (MNA matrix Z)", "bound": "hbm", "achieved": a, "peak": hbm,
                    "unit": "GB/s", "frac": a / hbm, "ms": phases["mna_fill"], "traffic": traffic.get("k_harmonic_fill"),
                    "peak_source": "measured (MEASURED_PEAKS.json)"})
    if phases.get("backward_error"):
        b = 16.0 * n * n
        a = b / (phases["backward_error"] * 1e-3) / 1e9
        out.append({"kernel": "k_backward_error (FP64 residual, one pass over Z)", "bound": "hbm", "achieved": a,
                    "peak": hbm, "unit": "GB/s", "frac": a / hbm, "ms": phases["backward_error"],
                    "traffic": traffic.get("k_backward_error"), "peak_source": "measured (MEASURED_PEAKS.json)"})
    return out


if __name__ == "__main__":
    main()
