"""The whole plain-CDI job (256 x 256, 8 blobs in a 64-px disk, 1e6 photons,
oversampling 4, binary random-phase start from the seed, HIO beta 0.9 x180
then ER x20 with a shrinkwrap every 20 iterations, 1000 iterations) on the GPU
against the oracle run from the same seeded Psi0.

Why not "within 1 % per run": HIO with shrinkwrap is chaotic.  The oracle run
in float32 and in float64 from the same Psi0 -- the same algorithm, rounding
changed only -- ends with final errors against the true object that differ by
a factor of up to two on single seeds (median over 16 seeds 0.46 vs 0.40) and
final masks that agree on only ~97 % of the pixels.  No float32
implementation, the reference's included, can hold a single run to 1 % of
another's.  So the job is compared
  * in distribution over 32 seeds: a two-sided sign test (the GPU's final
    error is above the float64 oracle's on 8..24 of the 32 seeds, p ~ 0.007),
    the median final error within 1 % plus three bootstrap standard errors of
    the float32-vs-float64 median difference, and the median mask agreement
    with the float64 oracle no worse than the float32 oracle's own, less 1 %;
  * and from the same state at the end of the job: the final 20 ER
    iterations from the oracle's state after 980 iterations (its Psi and mask)
    end with an error against the true object within 1 % of the oracle's and
    an object within the trajectory bound of tests/_bounds.py.
"""
import multiprocessing as mp
import os

import numpy as np
import pytest

from cdixx_gb300 import metrics, synth
from tests._bounds import rel_l2, trajectory_bound

pytestmark = pytest.mark.gpu

N = 256
PHOTONS = 1e6
SEEDS = list(range(100, 132))
BETA = 0.9
ALG = "5*(" + "+".join(["20*HIO+1*shrinkWrap"] * 9) + "+20*ER+1*shrinkWrap)"
STEPS_BEFORE_LAST_ER = 4 * 210 + 189   # steps (shrinkwraps included) before the job's last 20*ER
KW = dict(oversampling_spt=4.0, beta=BETA, shrink_threshold=0.1)


def _case(seed):
    obj, _, I = synth.config0_case(seed=seed, n=N, photons=PHOTONS)
    return obj, I, synth.random_phase_start(I, seed)


def _oracle_job(seed):
    """(seed, error f64, error f32, mask f64, mask f32, Psi and mask after 980 iterations)."""
    from oracle import cdi_oracle as O
    O.set_fft_workers(1)
    obj, I, psi0 = _case(seed)
    out = [seed]
    masks = []
    for dt in (np.complex128, np.complex64):
        st = O.phase_retrieve(psi0, I, ALG, dtype=dt, **KW)
        out.append(metrics.error_vs_truth(st.rho, obj))
        masks.append(st.support > st.threshold)
    mid = O.phase_retrieve(psi0, I, ALG, max_steps=STEPS_BEFORE_LAST_ER, **KW)
    return out + masks + [mid.psi.astype(np.complex64), (mid.support > mid.threshold).astype(np.float32)]


@pytest.fixture(scope="module")
def oracle_runs():
    # spawn: the workers start clean, without the parent's CUDA context
    with mp.get_context("spawn").Pool(min(len(SEEDS), os.cpu_count() or 1)) as pool:
        return {r[0]: r for r in pool.map(_oracle_job, SEEDS)}


def _boot_se(a, b, reps=2000, seed=0):
    g = np.random.default_rng(seed)
    a, b = np.asarray(a), np.asarray(b)
    idx = g.integers(0, len(a), (reps, len(a)))
    return float(np.std(np.median(a[idx], axis=1) - np.median(b[idx], axis=1)))


def test_config0_job_matches_oracle_in_distribution(cdx, oracle_runs):
    p = cdx.default_params(N, N, batch=len(SEEDS), **KW)
    with cdx.Context(p) as ctx:
        cases = [_case(s) for s in SEEDS]
        for i, (_, I, psi0) in enumerate(cases):
            ctx.set_pattern(i, I)
            ctx.set_initial(i, psi0)
        st = ctx.run(ALG)
        assert st["iterations"] == 1000 and st["shrinkwraps"] == 50
        e_gpu, agree_gpu = [], []
        for i, s in enumerate(SEEDS):
            e_gpu.append(metrics.error_vs_truth(ctx.get_object(i), cases[i][0]))
            mask = ctx.get_support(i) > ctx.stats(i)["threshold"]
            agree_gpu.append(float(np.mean(mask == oracle_runs[s][3])))
    e64 = np.array([oracle_runs[s][1] for s in SEEDS])
    e32 = np.array([oracle_runs[s][2] for s in SEEDS])
    agree32 = np.array([np.mean(oracle_runs[s][3] == oracle_runs[s][4]) for s in SEEDS])
    e_gpu = np.array(e_gpu)
    m64, m32, mg = np.median(e64), np.median(e32), np.median(e_gpu)
    se = _boot_se(e32, e64)
    above = int(np.sum(e_gpu > e64))
    msg = (f"median error vs truth: GPU {mg:.4f}, oracle f64 {m64:.4f}, oracle f32 {m32:.4f} (bootstrap SE {se:.4f}); "
           f"GPU above f64 on {above}/{len(SEEDS)}; median mask agreement with f64: GPU {np.median(agree_gpu):.4f}, "
           f"f32 {np.median(agree32):.4f}")
    print(msg)
    assert 8 <= above <= 24, msg
    assert abs(mg - m64) <= 0.01 * m64 + 3 * se, msg
    assert np.median(agree_gpu) >= np.median(agree32) - 0.01, msg


@pytest.mark.parametrize("seed", SEEDS[:4])
def test_config0_final_er_block_from_the_same_state(cdx, oracle_runs, seed):
    obj, I, _ = _case(seed)
    psi, mask = oracle_runs[seed][5], oracle_runs[seed][6]
    ref, tol = trajectory_bound(psi, I, "20*ER", support=mask, **KW)
    p = cdx.default_params(N, N, **KW)
    with cdx.Context(p) as ctx:
        ctx.set_pattern(0, I)
        ctx.set_initial(0, psi)
        ctx.set_support(0, mask)       # 0/1 field against the initial threshold 0.5
        ctx.run("20*ER")
        rho = ctx.get_object(0)
    e_gpu, e_ref = metrics.error_vs_truth(rho, obj), metrics.error_vs_truth(ref.rho, obj)
    d = rel_l2(rho, ref.rho)
    print(f"seed {seed}: final error vs truth GPU {e_gpu:.5f} oracle {e_ref:.5f}; rho {d:.2e} (bound {tol:.1e})")
    assert abs(e_gpu - e_ref) <= 0.01 * e_ref
    assert d <= tol
