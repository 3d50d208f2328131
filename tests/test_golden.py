"""The oracle and the CUDA path against golden vectors produced by the
reference's own CDI::phaseRetrieve (built from the reference sources as host
code; tests/golden/make_golden.py).

Two levels (tests/_bounds.py):
  * step_k: one HIO step from the reference's own state after k-1 steps,
    for k = 1..10 -- relative L2 <= 1e-5 per iterate;
  * trajectory cases (hio_k, raar_er, mixed, shrinkwrap, ccd, ...): k steps
    from Psi0, bounded by the divergence a 1e-7 perturbation of Psi0 produces
    over the same steps (never below 1e-5); shrinkwrap masks agree >= 99.9 %.
"""
from pathlib import Path

import numpy as np
import pytest

from oracle import cdi_oracle as O
from tests._bounds import STEP_TOL, rel_l2 as rel, trajectory_bound

GOLDEN = Path(__file__).resolve().parent / "golden" / "reference_cases.npz"
Z = np.load(GOLDEN)
CASES = sorted({k.split("/")[0] for k in Z.files if "/" in k and not k.startswith("step_")})
STEPS = list(range(1, 11))


def case(name):
    spt, thr, exposure, ccd, noise = Z[f"{name}/params"]
    return dict(alg=str(Z[f"{name}/algorithm"]), kw=dict(oversampling_spt=float(spt), shrink_threshold=float(thr),
                                                         exposure=float(exposure), sim_ccd_bit=bool(ccd),
                                                         noise_level=int(noise)))


def step_input(k):
    return Z["psi0"] if k == 1 else Z[f"hio_{k - 1}/psi"]


# ------------------------------------------------------------------ oracle (CPU)
@pytest.mark.parametrize("k", STEPS)
def test_oracle_one_step_matches_reference(k):
    st = O.phase_retrieve(step_input(k), Z["intensity"], "1*HIO", oversampling_spt=2.0)
    assert rel(st.rho, Z[f"step_{k}/rho"]) <= STEP_TOL


@pytest.mark.parametrize("name", CASES)
def test_oracle_trajectory_matches_reference(name):
    c = case(name)
    st, tol = trajectory_bound(Z["psi0"], Z["intensity"], c["alg"], **c["kw"])
    assert rel(st.rho, Z[f"{name}/rho"]) <= tol
    assert rel(st.psi, Z[f"{name}/psi"]) <= tol
    thr, res = Z[f"{name}/scalars"]
    assert abs(st.threshold - thr) <= 1e-5 * abs(thr)
    assert abs(st.residual - res) <= 2 * tol * abs(res)   # quadratic in Psi
    if "shrinkWrap" in c["alg"]:
        assert rel(st.support, Z[f"{name}/support"]) <= tol
        assert np.mean((st.support > st.threshold) == (Z[f"{name}/support"] > thr)) >= 0.999


# ------------------------------------------------------------------ CUDA path
def run_gpu(cdx, psi_in, alg, kw):
    I = Z["intensity"]
    n = I.shape[0]
    p = cdx.default_params(n, n, oversampling_spt=kw["oversampling_spt"], shrink_threshold=kw["shrink_threshold"],
                           exposure=kw["exposure"], sim_ccd_bit=int(kw["sim_ccd_bit"]), noise_level=kw["noise_level"])
    with cdx.Context(p) as ctx:
        ctx.set_pattern(0, I)
        ctx.set_initial(0, np.asarray(psi_in, np.complex64))
        s = ctx.run(alg)
        return s, ctx.get_object(0), ctx.get_fourier(0), ctx.get_support(0)


@pytest.mark.gpu
@pytest.mark.parametrize("k", STEPS)
def test_cuda_one_step_matches_reference(cdx, k):
    kw = dict(oversampling_spt=2.0, shrink_threshold=0.1, exposure=1.0, sim_ccd_bit=False, noise_level=0)
    s, rho, psi, spt = run_gpu(cdx, step_input(k), "1*HIO", kw)
    e = rel(rho, Z[f"step_{k}/rho"])
    print(f"step {k}: rho rel L2 vs the reference's own step {e:.2e}")
    assert e <= STEP_TOL


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_cuda_trajectory_matches_reference(cdx, name):
    c = case(name)
    s, rho, psi, spt = run_gpu(cdx, Z["psi0"], c["alg"], c["kw"])
    _, tol = trajectory_bound(Z["psi0"], Z["intensity"], c["alg"], **c["kw"])
    thr, res = Z[f"{name}/scalars"]
    e_rho, e_psi = rel(rho, Z[f"{name}/rho"]), rel(psi, Z[f"{name}/psi"])
    print(f"{name}: rho {e_rho:.2e} psi {e_psi:.2e} (bound {tol:.1e}) thr {s['threshold']:.7g}/{thr:.7g}")
    assert e_rho <= tol and e_psi <= tol
    assert abs(s["threshold"] - thr) <= 1e-5 * abs(thr)
    assert abs(s["residual"] - res) <= max(1e-4, 2 * tol) * abs(res)
    if "shrinkWrap" in c["alg"]:
        ref = Z[f"{name}/support"]
        assert np.mean((spt > s["threshold"]) == (ref > thr)) >= 0.999
