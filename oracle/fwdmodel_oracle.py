"""NumPy restatement of the GPU forward model (cdixx_gb300/csrc/cdx_fwdmodel.cu).

Test infrastructure only.  Same counter-based random numbers (SplitMix64
finaliser over (seed, pattern, stream, index)), same blob parameters and
rendering, same |FFT|^2 scaling; the Poisson step is checked statistically.
No reference counterpart (the reference simulates from image files,
src/post_gpu/cdi.cc:161-200).
"""
from __future__ import annotations

import numpy as np

M64 = (1 << 64) - 1
S_POS, S_SIG, S_AMP, S_NOISE = 1, 2, 3, 4
BLOBS = 8


def mix64(z):
    z &= M64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
    return z ^ (z >> 31)


def key4(seed, pat, stream, i):
    h = mix64(seed + 0x9E3779B97F4A7C15)
    h = mix64(h ^ ((pat * 0xD1B54A32D192ED03 + 0x8CB92BA72F3D8DD7) & M64))
    h = mix64(h ^ ((stream * 0xAEF17502108EF2D9 + 0x4F1BBCDCBFA53E0B) & M64))
    return mix64(h ^ ((i * 0x9E3779B97F4A7C15 + 0x2545F4914F6CDD1D) & M64))


def unif(seed, pat, stream, i):
    return ((key4(seed, pat, stream, i) >> 11) + 0.5) * (1.0 / 9007199254740992.0)


def blob_params(n, seed, pat):
    r = 0.25 * n / 2.0
    out = []
    for k in range(BLOBS):
        dx = dy = 0.0
        for t in range(64):
            x = (2.0 * unif(seed, pat, S_POS, k * 128 + 2 * t) - 1.0) * r
            y = (2.0 * unif(seed, pat, S_POS, k * 128 + 2 * t + 1) - 1.0) * r
            if x * x + y * y <= r * r:
                dx, dy = x, y
                break
        out.append((dx, dy, 2.0 + 4.0 * unif(seed, pat, S_SIG, k), 0.3 + 0.7 * unif(seed, pat, S_AMP, k)))
    return out


def render(n, seed, pat):
    """(object amplitude, support target) of pattern `pat`, centred, float64."""
    c, r = n / 2.0, 0.25 * n / 2.0
    yy, xx = np.mgrid[0:n, 0:n].astype(np.float64)
    v = np.zeros((n, n))
    for dx, dy, s, a in blob_params(n, seed, pat):
        v += a * np.exp(-((yy - c - dx) ** 2 + (xx - c - dy) ** 2) / (2.0 * s * s))
    v *= (yy - c) ** 2 + (xx - c) ** 2 <= r * r
    return v, (v > 1e-3).astype(np.float64)


def expected_intensity(n, seed, pat, photons):
    """The Poisson mean lambda = |FFT(rho)|^2 * photons / sum|FFT(rho)|^2 (FFT order)."""
    v, _ = render(n, seed, pat)
    F = np.abs(np.fft.fft2(v)) ** 2
    return F * photons / F.sum()
