"""Seeded synthetic workloads (the reference publishes no dataset; meshes are
built by the library's own generator, whose topology and dual patches are the
reference's).

* LIGHTNING_10_350: the 10/350 us first-stroke current with a 100 kA peak as
  the reference's double-exponential waveform K (exp(-alpha t) - exp(-beta t))
  (lightning.c:184-212).  alpha and beta were fitted so that the front time
  T1 = 1.25 (t90 - t10) is 10 us and the time from the virtual origin
  O1 = t10 - 0.1 T1 to the half value on the tail is 350 us; K scales the
  peak (at 19.5 us) to 100 kA.  waveform_times() recomputes those figures.
* serving_meshes: boxes with sides U(0.2, 2.0) m or flat plates, the cell
  size chosen so that the unknown count N = Ne + Nv is near a U(lo, hi) draw.
* harmonic_requests: frequency U(1, 100) MHz, 1-64 plane waves with random
  directions and transverse polarisations, Poisson arrival times.
* batch_systems: every mesh of a pool at log-spaced frequencies with a
  fixed number of plane waves (the many-meshes x many-frequencies sweep).
* serving_mix: the two request types of the serving workload on one Poisson
  arrival stream: a fraction of lightning runs (a seeded strike node on the
  box's top face) and harmonic requests as harmonic_requests draws them.
"""
import numpy as np

from .mesh import SynthMesh

LIGHTNING_10_350 = {"K": 105139.0, "alpha": 2127.18, "beta": 246066.0, "delay": 0.0}


def waveform_times(K, alpha, beta, delay=0.0):
    """(front time T1, half-value time T2, peak time, peak current) of the
    double exponential, from a dense sampling (seconds, amperes)."""
    tp = np.log(beta / alpha) / (beta - alpha)
    t = np.linspace(0.0, 20.0 / alpha, 2_000_001)
    i = K * (np.exp(-alpha * t) - np.exp(-beta * t))
    ip = K * (np.exp(-alpha * tp) - np.exp(-beta * tp))
    rise = t <= tp
    t10 = np.interp(0.1 * ip, i[rise], t[rise])
    t90 = np.interp(0.9 * ip, i[rise], t[rise])
    tail = ~rise
    t50 = np.interp(-0.5 * ip, -i[tail], t[tail])
    T1 = 1.25 * (t90 - t10)
    O1 = t10 - 0.1 * T1
    return T1, t50 - O1, tp + delay, ip


def _box_cells(lx, ly, lz, target):
    # N ~ 3 quads for a closed box: quads = area / h^2
    area = 2.0 * (lx * ly + ly * lz + lz * lx)
    h = np.sqrt(3.0 * area / target)
    return tuple(max(1, int(round(s / h))) for s in (lx, ly, lz))


def _plate_cells(lx, ly, target):
    h = np.sqrt(3.0 * lx * ly / target)
    return tuple(max(1, int(round(s / h))) for s in (lx, ly))


def serving_meshes(seed=5, count=6, lo=500, hi=12000):
    """[(SynthMesh, description)] of `count` seeded boxes or plates."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        target = rng.uniform(lo, hi)
        if rng.random() < 0.5:
            lx, ly, lz = rng.uniform(0.2, 2.0, 3)
            nx, ny, nz = _box_cells(lx, ly, lz, target)
            m = SynthMesh.box(lx, ly, lz, nx, ny, nz)
            desc = "box %.2fx%.2fx%.2f m, %dx%dx%d cells" % (lx, ly, lz, nx, ny, nz)
        else:
            lx, ly = rng.uniform(0.2, 2.0, 2)
            nx, ny = _plate_cells(lx, ly, target)
            m = SynthMesh.plate(lx, ly, nx, ny)
            desc = "plate %.2fx%.2f m, %dx%d cells" % (lx, ly, nx, ny)
        out.append((m, desc))
    return out


def plane_waves(rng, count):
    """Unit propagation directions and transverse unit polarisations."""
    th = np.arccos(rng.uniform(-1.0, 1.0, count))
    ph = rng.uniform(0.0, 2.0 * np.pi, count)
    k = np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], 1)
    a = np.where(np.abs(k[:, 2:3]) < 0.9, [[0.0, 0.0, 1.0]], [[1.0, 0.0, 0.0]])
    e = np.cross(k, a)
    e /= np.linalg.norm(e, axis=1)[:, None]
    return k, e


def harmonic_requests(seed, n_meshes, rate_hz, window_s, max_rhs=64):
    """Poisson arrivals over window_s: [(t_arrival, mesh index, frequency,
    k_hat (q, 3), e_hat (q, 3))]."""
    rng = np.random.default_rng(seed)
    out, t = [], 0.0
    while True:
        t += rng.exponential(1.0 / rate_hz)
        if t > window_s:
            return out
        q = int(rng.integers(1, max_rhs + 1))
        k, e = plane_waves(rng, q)
        out.append((t, int(rng.integers(0, n_meshes)), float(rng.uniform(1e6, 100e6)), k, e))


def batch_systems(seed, n_meshes, n_freqs, f_lo=1e3, f_hi=1e8, nrhs=4):
    """[(mesh index, frequency, k_hat (nrhs, 3), e_hat (nrhs, 3))] for every
    mesh at n_freqs log-spaced frequencies in [f_lo, f_hi]."""
    rng = np.random.default_rng(seed)
    out = []
    for mi in range(n_meshes):
        for f in np.logspace(np.log10(f_lo), np.log10(f_hi), n_freqs):
            k, e = plane_waves(rng, nrhs)
            out.append((mi, float(f), k, e))
    return out


def serving_mix(seed, n_meshes, rate_hz, window_s, top_nodes, lightning_fraction=0.3, max_rhs=64):
    """Poisson arrivals over window_s of both request types:
    [("harmonic", t, mesh index, frequency, k_hat, e_hat)] and
    [("lightning", t, strike node)] merged in arrival order; each arrival
    is a lightning run with probability lightning_fraction."""
    rng = np.random.default_rng(seed)
    out, t = [], 0.0
    top_nodes = np.asarray(top_nodes)
    while True:
        t += rng.exponential(1.0 / rate_hz)
        if t > window_s:
            return out
        if rng.random() < lightning_fraction:
            out.append(("lightning", t, int(rng.choice(top_nodes))))
            continue
        q = int(rng.integers(1, max_rhs + 1))
        k, e = plane_waves(rng, q)
        out.append(("harmonic", t, int(rng.integers(0, n_meshes)), float(rng.uniform(1e6, 100e6)), k, e))
