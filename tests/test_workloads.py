"""The seeded synthetic workloads the bench and the serving tests use."""
import numpy as np

from peeeeeeeeeeeeeeeeeeec_gb300 import workloads as W


def test_lightning_waveform_is_10_350_us_100_kA():
    T1, T2, tp, ip = W.waveform_times(**W.LIGHTNING_10_350)
    assert abs(T1 / 10e-6 - 1) < 1e-3
    assert abs(T2 / 350e-6 - 1) < 1e-3
    assert abs(ip / 100e3 - 1) < 1e-3
    assert 15e-6 < tp < 25e-6
    # the reference's default waveform (lightning.c:13-64) for comparison
    T1d, T2d, _, ipd = W.waveform_times(102900.0, 1500.0, 1.0e6)
    assert T1d < 5e-6 and T2d > 400e-6 and 90e3 < ipd < 110e3


def test_serving_meshes_are_seeded_and_sized():
    a = W.serving_meshes(seed=5, count=4, lo=300, hi=1500)
    b = W.serving_meshes(seed=5, count=4, lo=300, hi=1500)
    try:
        for (ma, da), (mb, db) in zip(a, b):
            assert da == db
            n = ma.n_edges + ma.n_nodes
            assert n == mb.n_edges + mb.n_nodes
            assert 150 <= n <= 2500  # rounding of the cell counts keeps N near the draw
    finally:
        for m, _ in a + b:
            m.close()


def test_harmonic_requests():
    r1 = W.harmonic_requests(seed=7, n_meshes=6, rate_hz=200.0, window_s=1.0)
    r2 = W.harmonic_requests(seed=7, n_meshes=6, rate_hz=200.0, window_s=1.0)
    assert len(r1) == len(r2) and 140 < len(r1) < 260  # Poisson(200)
    t = np.array([x[0] for x in r1])
    assert np.all(np.diff(t) > 0) and t[-1] <= 1.0
    for (ta, mi, f, k, e), (tb, mj, g, k2, e2) in zip(r1, r2):
        assert ta == tb and mi == mj and f == g and np.array_equal(k, k2)
        assert 0 <= mi < 6 and 1e6 <= f <= 100e6 and 1 <= len(k) <= 64
        assert np.allclose(np.linalg.norm(k, axis=1), 1) and np.allclose(np.linalg.norm(e, axis=1), 1)
        assert np.allclose(np.sum(k * e, axis=1), 0, atol=1e-12)
