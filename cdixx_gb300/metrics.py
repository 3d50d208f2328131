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


def _register_t(g, t):
    import torch
    b, n, m = g.shape
    cc = torch.fft.ifft2(torch.fft.fft2(t) * torch.conj(torch.fft.fft2(g))).abs()
    k = torch.argmax(cc.reshape(b, -1), dim=1)
    kx, ky = k // m, k % m
    ix = (torch.arange(n, device=g.device)[None, :, None] - kx[:, None, None]) % n
    iy = (torch.arange(m, device=g.device)[None, None, :] - ky[:, None, None]) % m
    gs = g[torch.arange(b, device=g.device)[:, None, None], ix, iy]          # np.roll(g, (kx, ky))
    c = (torch.conj(gs) * t).sum(dim=(1, 2)) / torch.clamp((gs.abs() ** 2).sum(dim=(1, 2)), min=1e-300)
    num = torch.linalg.vector_norm((c[:, None, None] * gs - t).reshape(b, -1), dim=1)
    return num / torch.clamp(torch.linalg.vector_norm(t.reshape(b, -1), dim=1), min=1e-300)


def error_vs_truth_batch(rho, truth, chunk=64):
    """error_vs_truth of every pattern of a batch, on torch tensors [b, n, m]
    (complex, any device; computed in complex128): returns a float64 NumPy
    array.  Same definition as error_vs_truth, for evaluating thousands of
    reconstructions without a host round trip per pattern."""
    import torch
    out = []
    for s in range(0, rho.shape[0], chunk):
        g = rho[s:s + chunk].to(torch.complex128)
        t = truth[s:s + chunk].to(torch.complex128)
        twin = torch.conj(torch.roll(torch.flip(g, dims=(1, 2)), shifts=(1, 1), dims=(1, 2)))
        out.append(torch.minimum(_register_t(g, t), _register_t(twin, t)).cpu())
    return torch.cat(out).numpy()
