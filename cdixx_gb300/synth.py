"""Seeded synthetic CDI inputs (the forward model used by tests and the bench).

No reference counterpart: the reference simulates from image files
(src/post_gpu/cdi.cc:161-200) that are not available here.  Objects are
centred in the field; the pattern is I = |FFT(rho)|^2 scaled to a total
photon count and Poisson-sampled, returned in FFT (unshifted) order as the
reference keeps patternData.  Generation runs on the host with NumPy; it is
input preparation, outside the timed phase-retrieval path.
"""
from __future__ import annotations

import numpy as np
from scipy import ndimage


def _rng(seed, pattern=0):
    return np.random.default_rng([int(seed), int(pattern), 0x5C41])


def blob_object(n, seed, pattern=0, nblobs=8, disk_frac=0.25, sig=(2.0, 6.0), amp=(0.3, 1.0), m=None):
    """Sum of `nblobs` Gaussian blobs (sigma U[sig], amplitude U[amp]), real
    positive, centres inside a centred disk of diameter disk_frac*n; masked to
    that disk.  Returns (object complex128, support mask)."""
    m = n if m is None else m
    g = _rng(seed, pattern)
    r = disk_frac * min(n, m) / 2
    yy, xx = np.mgrid[0:n, 0:m]
    cx, cy = n / 2, m / 2
    obj = np.zeros((n, m))
    for _ in range(nblobs):
        while True:
            dx, dy = g.uniform(-r, r, 2)
            if dx * dx + dy * dy <= r * r:
                break
        s = g.uniform(*sig)
        a = g.uniform(*amp)
        obj += a * np.exp(-((yy - cx - dx) ** 2 + (xx - cy - dy) ** 2) / (2 * s * s))
    disk = (yy - cx) ** 2 + (xx - cy) ** 2 <= r * r
    obj *= disk
    return obj.astype(np.complex128), disk


def phase_object(n, seed, pattern=0, diameter=512, smooth=4.0):
    """Amplitude U[0.5,1] and phase in [0, pi] from Gaussian-smoothed white
    noise (sigma = `smooth` px) inside a `diameter`-px support whose radius is
    modulated by a random smooth boundary (low-order Fourier series)."""
    g = _rng(seed, pattern)
    yy, xx = np.mgrid[0:n, 0:n]
    c = n / 2
    th = np.arctan2(yy - c, xx - c)
    rr = np.hypot(yy - c, xx - c)
    r0 = diameter / 2
    rb = np.full_like(th, r0)
    for k in range(1, 6):
        a, b = g.normal(0, 0.03 * r0 / k, 2)
        rb += a * np.cos(k * th) + b * np.sin(k * th)
    sup = rr <= rb
    noise_a = ndimage.gaussian_filter(g.standard_normal((n, n)), smooth, mode="wrap")
    noise_p = ndimage.gaussian_filter(g.standard_normal((n, n)), smooth, mode="wrap")
    na = (noise_a - noise_a.min()) / max(np.ptp(noise_a), 1e-30)
    npf = (noise_p - noise_p.min()) / max(np.ptp(noise_p), 1e-30)
    amp = 0.5 + 0.5 * na
    ph = np.pi * npf
    obj = np.where(sup, amp * np.exp(1j * ph), 0)
    return obj.astype(np.complex128), sup


def pattern_from_object(obj, photons, seed, pattern=0, poisson=True):
    """I = |FFT(obj)|^2 scaled to `photons` total counts, Poisson-sampled,
    float32 in FFT order."""
    F = np.fft.fft2(obj)
    I = np.abs(F) ** 2
    I *= photons / I.sum()
    if poisson:
        g = _rng(seed, pattern + 1_000_003)
        I = g.poisson(I).astype(np.float64)
    return I.astype(np.float32)


def random_phase_start(intensity, seed, pattern=0):
    """Psi0 = sqrt(I) e^{i pi b}, b a fair coin per pixel (binary random phase of
    applyRandomPhase, src/gpu/cdi.cu:486-502), complex64."""
    g = _rng(seed, pattern + 2_000_003)
    b = g.random(intensity.shape) > 0.5
    a = np.sqrt(np.maximum(intensity.astype(np.float64), 0))
    return np.where(b, -a, a).astype(np.complex64)


def config0_case(seed=20260101, n=256, photons=1e6, pattern=0):
    obj, sup = blob_object(n, seed, pattern)
    I = pattern_from_object(obj, photons, seed, pattern)
    return obj, sup, I


def config1_case(seed=20260101, n=2048, photons=1e9, pattern=0, diameter=512):
    obj, sup = phase_object(n, seed, pattern, diameter=diameter)
    I = pattern_from_object(obj, photons, seed, pattern)
    return obj, sup, I
