"""Evaluation metrics of reconstructions (host-side, NumPy; no reference
counterpart -- the reference's PSNR/SSIM script needs image files that are
not available).

error_vs_truth: the normalised error of Fienup, min over the twin image,
integer translations (peak of the FFT cross-correlation, as in Guizar-Sicairos
et al., Opt. Lett. 33, 156 (2008), without sub-pixel refinement) and a global
complex factor:  min || c * g - truth || / || truth ||  with
c = <g, truth> / <g, g>.
"""
from __future__ import annotations

import numpy as np


def _register(g, truth):
    F = np.fft.fft2(truth) * np.conj(np.fft.fft2(g))
    cc = np.fft.ifft2(F)
    k = np.unravel_index(np.argmax(np.abs(cc)), cc.shape)
    gs = np.roll(g, shift=k, axis=(0, 1))
    c = np.vdot(gs, truth) / max(np.vdot(gs, gs).real, 1e-300)
    return np.linalg.norm(c * gs - truth) / max(np.linalg.norm(truth), 1e-300)


def error_vs_truth(rho, truth) -> float:
    """Registered relative error of `rho` against `truth` (both complex)."""
    g = np.asarray(rho, np.complex128)
    t = np.asarray(truth, np.complex128)
    twin = np.conj(np.roll(g[::-1, ::-1], shift=(1, 1), axis=(0, 1)))   # conj(rho(-x, -y)), periodic
    return float(min(_register(g, t), _register(twin, t)))


def r_factor(psi, intensity, mask=None) -> float:
    """sum | |Psi| - sqrt(I) | / sum sqrt(I) over measured pixels (float64)."""
    a = np.abs(np.asarray(psi, np.complex128))
    s = np.sqrt(np.maximum(np.asarray(intensity, np.float64), 0))
    if mask is not None:
        a, s = a[mask], s[mask]
    return float(np.sum(np.abs(a - s)) / max(np.sum(s), 1e-300))
