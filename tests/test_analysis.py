"""Host-side analysis helpers: force statistics and the resolution-independent wake
vorticity spectrum."""

import numpy as np


def test_spectrum_is_resolution_independent(pkg):
    chord = 20.0
    res = []
    for n in (200, 400):
        x = np.arange(n) * (200.0 / n)           # the same physical segment, two spacings
        wz = np.sin(2 * np.pi * 0.5 * x / chord)[:, None] * np.ones((1, 8))
        k, p = pkg.analysis.wake_vorticity_spectrum(wz, chord * n / 200.0, 0)
        res.append((k, p))
    (k1, p1), (k2, p2) = res
    i1, i2 = np.argmax(p1), np.argmax(p2)
    assert abs(k1[i1] - 0.5) < 1e-9 and abs(k2[i2] - 0.5) < 1e-9
    assert abs(p1[i1] / p2[i2] - 1.0) < 1e-2   # Hann window end points: O(1/n)
    # identical spectra are at distance zero
    assert pkg.analysis.spectrum_distance(k1, p1, k1, p1, k_max=3.0) == 0.0


def test_force_statistics(pkg):
    t = np.arange(1000)
    coeffs = dict(cl=1.0 + 0.5 * np.sin(2 * np.pi * t / 100), cd=0.2 + 0 * t)
    st = pkg.analysis.force_statistics(coeffs, start=200)
    assert abs(st["cl_mean"] - 1.0) < 1e-9 and abs(st["cl_rms"] - 0.5 / np.sqrt(2)) < 1e-6
    assert st["cd_rms"] == 0.0
