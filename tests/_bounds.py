"""Tolerances for comparing iterates of the FP32 path with references.

Per iterate (one step from the same state): relative L2 1e-5.  Measured: the
CUDA path's one step differs from the reference's own step by 1.2e-7 .. 3.2e-7
(tests/test_golden.py::test_cuda_one_step_matches_reference).

Along a trajectory (k steps from Psi0) HIO/RAAR/POSHIO amplify rounding: on
the Poisson patterns of these tests a relative 1e-7 perturbation of Psi0 grows
to ~1e-4 within ten HIO steps, and POSHIO (a sign test on rho'.x, and an
imaginary part that always takes the HIO update) turns float32 rounding into
1e-2 differences.  Two float32 implementations (this path with its FFT, the
reference with cuFFT) can therefore not be held to 1e-5 along a trajectory.
The bound is TRAJ_FACTOR (4) times the larger of two sensitivity estimates of the
same run in float64:
  * the divergence when every step adds noise of relative size STEP_NOISE
    times the RMS of rho (the one-step difference measured above), and
  * the distance of the oracle run in float32 from the float64 run,
and never below 1e-5.
"""
import numpy as np

from oracle import cdi_oracle as O

STEP_TOL = 1e-5
STEP_NOISE = 3e-7
TRAJ_FACTOR = 4.0


def rel_l2(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def trajectory_bound(psi0, intensity, algorithm, seed=0, **kw):
    """(float64 oracle state, bound) for `algorithm` run from psi0."""
    a = O.phase_retrieve(psi0, intensity, algorithm, **kw)
    sens = rel_l2(O.phase_retrieve(psi0, intensity, algorithm, dtype=np.complex64, **kw).rho, a.rho)
    for s in range(2):
        b = O.phase_retrieve(psi0, intensity, algorithm, step_noise=(STEP_NOISE, seed + s), **kw)
        sens = max(sens, rel_l2(b.rho, a.rho))
    return a, max(STEP_TOL, TRAJ_FACTOR * sens)
