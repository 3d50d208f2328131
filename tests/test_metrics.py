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
