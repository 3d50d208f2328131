"""The oracle and the CUDA path against the reference's own CDI::phaseRetrieve
at 256 x 256, the plain CDI configuration's size (tests/golden/make_golden.py
--256: 8 blobs in a 64-px disk, 1e6 photons, oversampling 4 so the rect
support is rows/cols 95..160, shrinkThreshold 0.1, beta_HIO 1).

  * step_k (k = 1, 5, 10): one HIO step from the reference's own state after
    k-1 steps -- relative L2 <= 1e-5 per iterate;
  * sw_step: one HIO step and one shrinkwrap from the reference's state after 9
    steps -- the blurred support field within 1e-5, the threshold within
    1e-5 relative, >= 99.9 % of the mask;
  * sw_traj: 2*(10*HIO+1*shrinkWrap)+4*ER from Psi0 -- the object within the
    trajectory bound of tests/_bounds.py, >= 99.9 % of the final mask.
"""
from pathlib import Path

import numpy as np
import pytest

from oracle import cdi_oracle as O
from tests._bounds import STEP_TOL, rel_l2 as rel, trajectory_bound

Z = np.load(Path(__file__).resolve().parent / "golden" / "reference_cases_256.npz")
STEPS = sorted(int(k.split("/")[0][5:]) for k in Z.files if k.startswith("step_") and k.endswith("/rho"))
KW = dict(oversampling_spt=4.0, shrink_threshold=0.1)


def test_fixture_holds_the_config0_cases():
    assert Z["intensity"].shape == (256, 256) and STEPS == [1, 5, 10]


# ------------------------------------------------------------------ oracle (CPU)
@pytest.mark.parametrize("k", STEPS)
def test_oracle_one_step_matches_reference_256(k):
    st = O.phase_retrieve(Z[f"step_{k}/psi_in"], Z["intensity"], "1*HIO", **KW)
    assert rel(st.rho, Z[f"step_{k}/rho"]) <= STEP_TOL


def test_oracle_shrinkwrap_step_matches_reference_256():
    st = O.phase_retrieve(Z["sw_step/psi_in"], Z["intensity"], "1*HIO+1*shrinkWrap", **KW)
    thr = Z["sw_step/scalars"][0]
    assert rel(st.rho, Z["sw_step/rho"]) <= STEP_TOL
    assert rel(st.support, Z["sw_step/support"]) <= STEP_TOL
    assert abs(st.threshold - thr) <= 1e-5 * abs(thr)
    assert np.mean((st.support > st.threshold) == (Z["sw_step/support"] > thr)) >= 0.999


def test_oracle_shrinkwrap_trajectory_matches_reference_256():
    alg = str(Z["sw_traj/algorithm"])
    st, tol = trajectory_bound(Z["psi0"], Z["intensity"], alg, **KW)
    assert rel(st.rho, Z["sw_traj/rho"]) <= tol
    ref_mask = np.unpackbits(Z["sw_traj/support_mask"])[:256 * 256].reshape(256, 256).astype(bool)
    assert np.mean((st.support > st.threshold) == ref_mask) >= 0.999


# ------------------------------------------------------------------ CUDA path
def run_gpu(cdx, psi_in, alg):
    I = Z["intensity"]
    p = cdx.default_params(256, 256, **KW)
    with cdx.Context(p) as ctx:
        ctx.set_pattern(0, I)
        ctx.set_initial(0, np.asarray(psi_in, np.complex64))
        s = ctx.run(alg)
        return s, ctx.get_object(0), ctx.get_support(0)


@pytest.mark.gpu
@pytest.mark.parametrize("k", STEPS)
def test_cuda_one_step_matches_reference_256(cdx, k):
    _, rho, _ = run_gpu(cdx, Z[f"step_{k}/psi_in"], "1*HIO")
    e = rel(rho, Z[f"step_{k}/rho"])
    print(f"256^2 step {k}: rho rel L2 vs the reference's own step {e:.2e}")
    assert e <= STEP_TOL


@pytest.mark.gpu
def test_cuda_shrinkwrap_step_matches_reference_256(cdx):
    s, rho, spt = run_gpu(cdx, Z["sw_step/psi_in"], "1*HIO+1*shrinkWrap")
    thr = Z["sw_step/scalars"][0]
    e_rho, e_spt = rel(rho, Z["sw_step/rho"]), rel(spt, Z["sw_step/support"])
    agree = np.mean((spt > s["threshold"]) == (Z["sw_step/support"] > thr))
    print(f"256^2 shrinkwrap step: rho {e_rho:.2e} support {e_spt:.2e} thr {s['threshold']:.7g}/{thr:.7g} "
          f"mask {agree:.5f}")
    assert e_rho <= STEP_TOL and e_spt <= STEP_TOL
    assert abs(s["threshold"] - thr) <= 1e-5 * abs(thr)
    assert agree >= 0.999


@pytest.mark.gpu
def test_cuda_shrinkwrap_trajectory_matches_reference_256(cdx):
    alg = str(Z["sw_traj/algorithm"])
    s, rho, spt = run_gpu(cdx, Z["psi0"], alg)
    _, tol = trajectory_bound(Z["psi0"], Z["intensity"], alg, **KW)
    ref_mask = np.unpackbits(Z["sw_traj/support_mask"])[:256 * 256].reshape(256, 256).astype(bool)
    e = rel(rho, Z["sw_traj/rho"])
    agree = np.mean((spt > s["threshold"]) == ref_mask)
    print(f"256^2 {alg}: rho {e:.2e} (bound {tol:.1e}) mask {agree:.5f}")
    assert e <= tol and agree >= 0.999
