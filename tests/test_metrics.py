"""Registered error against the known object (CPU)."""
import numpy as np

from cdixx_gb300 import metrics, synth


def test_error_vs_truth_invariances():
    obj, sup = synth.blob_object(64, 3)
    obj = obj * np.exp(0.3j * np.linspace(0, 1, 64))[None, :]
    assert metrics.error_vs_truth(obj, obj) < 1e-12
    shifted = np.roll(obj, (5, -7), axis=(0, 1)) * np.exp(1.1j) * 2.5
    assert metrics.error_vs_truth(shifted, obj) < 1e-12
    twin = np.conj(np.roll(obj[::-1, ::-1], (1, 1), axis=(0, 1)))
    assert metrics.error_vs_truth(np.roll(twin, (3, 4), axis=(0, 1)), obj) < 1e-12
    noisy = obj + 0.05 * np.abs(obj).max() * np.random.default_rng(0).standard_normal(obj.shape)
    e = metrics.error_vs_truth(noisy, obj)
    assert 0.01 < e < 0.5


def test_r_factor_zero_for_exact_modulus():
    obj, _ = synth.blob_object(32, 1)
    F = np.fft.fft2(obj)
    assert metrics.r_factor(F, np.abs(F) ** 2) < 1e-12


def test_batched_error_matches_host_error():
    import torch
    from cdixx_gb300 import metrics as M
    g = np.random.default_rng(3)
    truth = (g.random((5, 32, 48)) + 1j * g.random((5, 32, 48))) * (g.random((5, 32, 48)) > 0.6)
    rho = np.stack([np.roll(np.conj(t[::-1, ::-1]), (3 + i, -2), axis=(0, 1)) * np.exp(0.7j) for i, t in
                    enumerate(truth)])
    rho[1] = truth[1] + 0.3 * g.standard_normal((32, 48))
    rho[2] = g.standard_normal((32, 48))
    got = M.error_vs_truth_batch(torch.from_numpy(rho), torch.from_numpy(truth), chunk=2)
    want = np.array([M.error_vs_truth(r, t) for r, t in zip(rho, truth)])
    assert np.allclose(got, want, rtol=1e-10, atol=1e-12)
    assert got[0] < 1e-12
