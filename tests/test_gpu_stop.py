"""In-loop stops of a batch: a per-pattern stop R-factor (cdx_set_stop_rfactor)
and the R-factor plateau (plateau_iters / plateau_tol).  A frozen pattern keeps
the state of the iteration it stopped in, so it must equal a run of exactly
that many iterations; the others must not notice it."""
import numpy as np
import pytest

from cdixx_gb300 import synth
from tests._bounds import rel_l2

pytestmark = pytest.mark.gpu

N = 128
RF = 5


def _case(seed=11):
    _, _, I = synth.config0_case(seed=seed, n=N, photons=1e6)
    return I, synth.random_phase_start(I, seed)


def _run(cdx, I, psi0, iters, batch=1, **kw):
    p = cdx.default_params(N, N, batch=batch, oversampling_spt=2.0, beta=0.9, rf_every=RF, **kw)
    ctx = cdx.Context(p)
    for i in range(batch):
        ctx.set_pattern(i, I)
        ctx.set_initial(i, psi0)
    return ctx


def test_per_pattern_stop_freezes_only_that_pattern(cdx):
    I, psi0 = _case()
    with _run(cdx, I, psi0, 40, batch=3) as ctx:
        ctx.set_stop_rfactor(0, 1e9)     # reached at the first check (iteration RF)
        ctx.set_stop_rfactor(2, 1e-12)   # never
        ctx.run("40*HIO")
        s = [ctx.stats(i) for i in range(3)]
        rho = [ctx.get_object(i) for i in range(3)]
    assert s[0]["converged_iter"] == RF + 1 and s[0]["flags"] & 2
    assert s[1]["converged_iter"] == -1 and s[2]["converged_iter"] == -1
    with _run(cdx, I, psi0, 40) as ctx:
        ctx.run(f"{RF + 1}*HIO")
        short = ctx.get_object(0)
    with _run(cdx, I, psi0, 40) as ctx:
        ctx.run("40*HIO")
        full = ctx.get_object(0)
    assert rel_l2(rho[0], short) <= 1e-6
    assert rel_l2(rho[1], full) <= 1e-6 and rel_l2(rho[2], full) <= 1e-6
    assert np.isfinite(s[1]["rfactor_min"]) and s[1]["rfactor_min"] <= s[1]["rfactor"] * 10


def test_plateau_stop(cdx):
    I, psi0 = _case(12)
    plateau = 3 * RF
    # a tolerance of 0.99 counts nothing after the first check as an improvement
    with _run(cdx, I, psi0, 60, batch=1, plateau_iters=plateau, plateau_tol=0.99) as ctx:
        ctx.run("60*HIO")
        s = ctx.stats(0)
        rho = ctx.get_object(0)
    assert s["converged_iter"] == RF + plateau + 1
    assert s["flags"] & 8
    with _run(cdx, I, psi0, 60) as ctx:
        ctx.run(f"{RF + plateau + 1}*HIO")
        short = ctx.get_object(0)
    assert rel_l2(rho, short) <= 1e-6
    # tolerance 0: any decrease counts; the plateau cannot end a run shorter than the window
    with _run(cdx, I, psi0, 60, batch=1, plateau_iters=100, plateau_tol=0.0) as ctx:
        ctx.run("60*HIO")
        assert ctx.stats(0)["converged_iter"] == -1


def test_plateau_arguments_are_checked(cdx):
    with pytest.raises(Exception):
        cdx.Context(cdx.default_params(N, N, plateau_iters=-1))
    with pytest.raises(Exception):
        cdx.Context(cdx.default_params(N, N, plateau_tol=1.5))
