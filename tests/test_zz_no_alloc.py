"""cdx_iterate_noalloc, the entry point that allocates no device memory.

Some callers of this library cannot allocate device memory: an acquisition
loop that cannot take the device-wide synchronisation cudaMalloc/cudaFree
bring between detector frames, or a plugin whose host application owns the
whole device-memory budget.  cdx_iterate_noalloc gives them the fused
iteration with its scratch in a static device array of the library; they pass
only their own input and output buffers.

Here it is called through the C ABI, twice in a row on the same inputs, and
each call is checked
  * against the oracle (the CPU restatement of phaseRetrieve, pinned against
    the reference's own step): relative L2 within the trajectory bound of
    tests/_bounds.py (1e-5 for one step, the float32 sensitivity of the run
    for longer ones), and
  * against the context path (cdx_set_pattern / cdx_set_initial /
    cdx_set_support / cdx_run) within the per-iterate tolerance 1e-5,
at the largest size its static array admits (512 x 512) among others, with
no iteration at all, and for the arguments it must refuse.  The file name
sorts last so that a run stopping at its first failure has already run every
other test.
"""
import ctypes

import numpy as np
import pytest

from cdixx_gb300 import synth
from tests._bounds import STEP_TOL, rel_l2, trajectory_bound

pytestmark = pytest.mark.gpu


def _ptr(t, byte_offset=0):
    return ctypes.c_void_p(t.data_ptr() + byte_offset)


def _case(rows, cols, seed=31):
    n = max(rows, cols)
    obj, sup, I_full = synth.config0_case(seed=seed, n=n, photons=1e6)
    I = np.ascontiguousarray(I_full[:rows, :cols])
    psi0 = synth.random_phase_start(I, seed)
    spt = np.zeros((rows, cols), np.float32)
    spt[rows // 4: 3 * rows // 4, cols // 4: 3 * cols // 4] = 1.0
    return I, psi0, spt


def _call(cdx, torch, rows, cols, algo, beta, iters, d_int, d_spt, d_psi0):
    rho = torch.full((rows, cols), float("nan"), dtype=torch.complex64, device="cuda")
    psi = torch.full_like(rho, float("nan"))
    lib = cdx.lib()
    rc = lib.cdx_iterate_noalloc(rows, cols, algo, beta, iters, _ptr(d_int), _ptr(d_spt), 0.5, _ptr(d_psi0),
                                 _ptr(rho), _ptr(psi), None)
    assert rc == 0, lib.cdx_last_error()
    torch.cuda.synchronize()
    return rho.cpu().numpy(), psi.cpu().numpy()


@pytest.mark.parametrize("rows,cols", [(256, 256), (192, 384), (512, 512)])
def test_noalloc_matches_oracle_and_context_on_two_calls(cdx, torch_cuda, rows, cols):
    torch = torch_cuda
    I, psi0, spt = _case(rows, cols)
    d_int = torch.from_numpy(I).cuda()
    d_spt = torch.from_numpy(spt).cuda()
    d_psi0 = torch.from_numpy(psi0).cuda()
    for algo, name, beta, iters in [(cdx.HIO, "HIO", 0.9, 6), (cdx.RAAR, "RAAR", 0.9, 4), (cdx.ER, "ER", 1.0, 1)]:
        alg = f"{iters}*{name}"
        ref, bound = trajectory_bound(psi0, I, alg, support=spt, beta=beta)
        p = cdx.default_params(rows, cols, beta=beta)
        with cdx.Context(p) as ctx:
            ctx.set_pattern(0, I)
            ctx.set_initial(0, psi0)
            ctx.set_support(0, spt)          # threshold 0.5, the initial vars.threshold
            ctx.run(alg)
            ctx_rho, ctx_psi = ctx.get_object(0), ctx.get_fourier(0)
        outs = [_call(cdx, torch, rows, cols, algo, beta, iters, d_int, d_spt, d_psi0) for _ in range(2)]
        for call, (rho, psi) in enumerate(outs):
            e_rho, e_psi = rel_l2(rho, ref.rho), rel_l2(psi, ref.psi)
            assert e_rho <= bound and e_psi <= bound, (name, call, "oracle", e_rho, e_psi, bound)
            c_rho, c_psi = rel_l2(rho, ctx_rho), rel_l2(psi, ctx_psi)
            assert c_rho <= STEP_TOL and c_psi <= STEP_TOL, (name, call, "context", c_rho, c_psi)
        # the second call starts from the first call's leftovers in the shared array
        assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1]), name


def test_noalloc_zero_iterations_is_the_restart_object(cdx, torch_cuda):
    """iterations = 0: rho = IFFT(Psi0)/sqrt(N) as prepareIter leaves it
    (scaled back by phaseRetrieve's sqrt(N)), Psi = Psi0; also with psi_out
    being psi0 itself."""
    torch = torch_cuda
    rows, cols = 256, 256
    I, psi0, spt = _case(rows, cols, seed=5)
    d_int = torch.from_numpy(I).cuda()
    d_spt = torch.from_numpy(spt).cuda()
    d_psi0 = torch.from_numpy(psi0).cuda()
    ref, _ = trajectory_bound(psi0, I, "1*HIO", support=spt, max_steps=0)
    for _ in range(2):
        rho, psi = _call(cdx, torch, rows, cols, cdx.HIO, 1.0, 0, d_int, d_spt, d_psi0)
        assert rel_l2(rho, ref.rho) <= STEP_TOL
        assert np.array_equal(psi, psi0)
    rho = torch.empty((rows, cols), dtype=torch.complex64, device="cuda")
    lib = cdx.lib()
    rc = lib.cdx_iterate_noalloc(rows, cols, cdx.HIO, 1.0, 0, _ptr(d_int), _ptr(d_spt), 0.5, _ptr(d_psi0), _ptr(rho),
                                 _ptr(d_psi0), None)
    assert rc == 0, lib.cdx_last_error()
    torch.cuda.synchronize()
    assert rel_l2(rho.cpu().numpy(), ref.rho) <= STEP_TOL
    assert np.array_equal(d_psi0.cpu().numpy(), psi0)


def test_noalloc_rejects_what_it_cannot_run(cdx, torch_cuda):
    """Refused before any work is queued: sizes beyond the static array,
    shrinkwrap, buffers off a 16-byte boundary, outputs that alias inputs."""
    torch = torch_cuda
    lib = cdx.lib()
    n = 1024   # 1024 x 1024 > CDX_NOALLOC_MAX_PIXELS
    a = torch.zeros((n, n), dtype=torch.float32, device="cuda")
    z = torch.zeros((n, n), dtype=torch.complex64, device="cuda")
    w = torch.zeros((n, n), dtype=torch.complex64, device="cuda")
    for r, c in [(1024, 1024), (512, 768)]:
        rc = lib.cdx_iterate_noalloc(r, c, cdx.HIO, 1.0, 1, _ptr(a), _ptr(a), 0.5, _ptr(z), _ptr(w), _ptr(z), None)
        assert rc == cdx.CDX_ERR_SIZE
        assert b"CDX_NOALLOC_MAX_PIXELS" in lib.cdx_last_error()
    rc = lib.cdx_iterate_noalloc(256, 256, cdx.SHRINKWRAP, 1.0, 1, _ptr(a), _ptr(a), 0.5, _ptr(z), _ptr(w), _ptr(z),
                                 None)
    assert rc == cdx.CDX_ERR_ALGO
    # a complex view one element in: 8-byte aligned, not 16
    rc = lib.cdx_iterate_noalloc(256, 256, cdx.HIO, 1.0, 1, _ptr(a), _ptr(a), 0.5, _ptr(z), _ptr(w, 8), _ptr(z),
                                 None)
    assert rc == cdx.CDX_ERR_ARG and b"16-byte" in lib.cdx_last_error()
    # rho_out on top of psi0
    rc = lib.cdx_iterate_noalloc(256, 256, cdx.HIO, 1.0, 1, _ptr(a), _ptr(a), 0.5, _ptr(z), _ptr(z), _ptr(w), None)
    assert rc == cdx.CDX_ERR_ARG and b"overlap" in lib.cdx_last_error()
    # psi_out overlapping psi0 without being psi0
    rc = lib.cdx_iterate_noalloc(256, 256, cdx.HIO, 1.0, 1, _ptr(a), _ptr(a), 0.5, _ptr(z), _ptr(w), _ptr(z, 4096),
                                 None)
    assert rc == cdx.CDX_ERR_ARG and b"overlap" in lib.cdx_last_error()
