"""Flow analysis on the host: statistics of the lift/drag histories and the mid-span
vorticity spectrum used to compare runs at different resolutions.

The reference only renders the mid-span vorticity (render_2d.py:272-275); the spectrum is
this project's own definition: the power of the z-vorticity along x over the wake
(x from the trailing edge region to the outlet), averaged over y, as a function of the
wavenumber in cycles per chord, so lattices of different resolution compare directly.
"""

import numpy as np


def force_statistics(coeffs, start=0):
    """Mean and RMS (about the mean) of C_L and C_D from `start` on."""
    cl = np.asarray(coeffs["cl"])[start:]
    cd = np.asarray(coeffs["cd"])[start:]
    return dict(cl_mean=float(cl.mean()), cl_rms=float(cl.std()), cd_mean=float(cd.mean()),
                cd_rms=float(cd.std()))


def wake_vorticity_spectrum(wz, chord, x_start, x_stop=None):
    """Power spectrum of wz (Nx, Ny) along x over [x_start, x_stop), mean over y.
    Returns (k, power) with k in cycles per chord. The power of a bin is the squared
    amplitude it holds (|FFT|^2 / n^2 with a Hann window), so the same physical segment
    sampled at different resolutions gives the same values on the same wavenumber bins."""
    seg = np.asarray(wz, np.float64)[int(x_start):(None if x_stop is None else int(x_stop))]
    seg = seg - seg.mean(axis=0, keepdims=True)
    n = seg.shape[0]
    win = np.hanning(n)[:, None]
    spec = np.abs(np.fft.rfft(seg * win, axis=0)) ** 2
    power = spec.mean(axis=1) / max(n, 1) ** 2
    k = np.fft.rfftfreq(n, d=1.0) * chord
    return k, power


def spectrum_distance(k_a, p_a, k_b, p_b, k_max):
    """Relative L2 distance of two spectra on the common band k <= k_max (log power,
    interpolated onto the coarser wavenumber grid)."""
    grid = k_a if len(k_a) <= len(k_b) else k_b
    grid = grid[(grid > 0) & (grid <= k_max)]
    la = np.interp(grid, k_a, np.log10(p_a + 1e-30))
    lb = np.interp(grid, k_b, np.log10(p_b + 1e-30))
    return float(np.linalg.norm(la - lb) / max(np.linalg.norm(lb), 1e-30))
