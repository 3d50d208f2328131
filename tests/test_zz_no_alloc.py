"""cdx_iterate_noalloc, the entry point that allocates no device memory.

Some callers of this library cannot allocate device memory: an acquisition
loop that cannot take the device-wide synchronisation cudaMalloc/cudaFree
bring between detector frames, or a plugin whose host application owns the
whole device-memory budget.  cdx_iterate_noalloc gives them the fused
iteration with its scratch in a static device array of the library; they pass
only their own input and output buffers.

Here it is called through the C ABI and checked, on two calls in a row,
against the context path (cdx_set_pattern / cdx_set_initial /
cdx_set_support / cdx_run) within the per-iterate tolerance of the parity
tests (relative L2 1e-5).  The file name sorts last so that a run stopping at
its first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from cdixx_gb300 import synth

pytestmark = pytest.mark.gpu

TOL = 1e-5


def rel_l2(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.mark.parametrize("rows,cols", [(256, 256), (192, 384)])
def test_noalloc_matches_context_path_on_two_calls(cdx, torch_cuda, rows, cols):
    torch = torch_cuda
    n = max(rows, cols)
    obj, sup, I_full = synth.config0_case(seed=31, n=n, photons=1e6)
    I = np.ascontiguousarray(I_full[:rows, :cols])
    psi0 = synth.random_phase_start(I, 31)
    spt = np.zeros((rows, cols), np.float32)
    spt[rows // 4: 3 * rows // 4, cols // 4: 3 * cols // 4] = 1.0
    d_int = torch.from_numpy(I).cuda()
    d_spt = torch.from_numpy(spt).cuda()
    d_psi0 = torch.from_numpy(psi0).cuda()
    rho = torch.empty((rows, cols), dtype=torch.complex64, device="cuda")
    psi = torch.empty_like(rho)
    lib = cdx.lib()
    for algo, name, beta, iters in [(cdx.HIO, "HIO", 0.9, 12), (cdx.RAAR, "RAAR", 0.9, 7), (cdx.ER, "ER", 1.0, 3)]:
        p = cdx.default_params(rows, cols, beta=beta)
        with cdx.Context(p) as ctx:
            ctx.set_pattern(0, I)
            ctx.set_initial(0, psi0)
            ctx.set_support(0, spt)          # threshold 0.5, the initial vars.threshold
            ctx.run(f"{iters}*{name}")
            ref_rho, ref_psi = ctx.get_object(0), ctx.get_fourier(0)
        for call in range(2):
            rho.fill_(float("nan"))
            psi.fill_(float("nan"))
            rc = lib.cdx_iterate_noalloc(rows, cols, algo, beta, iters, _ptr(d_int), _ptr(d_spt), 0.5, _ptr(d_psi0),
                                         _ptr(rho), _ptr(psi), None)
            assert rc == 0, lib.cdx_last_error()
            torch.cuda.synchronize()
            e_rho = rel_l2(rho.cpu().numpy(), ref_rho)
            e_psi = rel_l2(psi.cpu().numpy(), ref_psi)
            assert e_rho <= TOL and e_psi <= TOL, (name, call, e_rho, e_psi)


def test_noalloc_rejects_sizes_beyond_its_scratch(cdx, torch_cuda):
    torch = torch_cuda
    lib = cdx.lib()
    n = 1024   # 1024 x 1024 > CDX_NOALLOC_MAX_PIXELS
    a = torch.zeros((n, n), dtype=torch.float32, device="cuda")
    z = torch.zeros((n, n), dtype=torch.complex64, device="cuda")
    rc = lib.cdx_iterate_noalloc(n, n, cdx.HIO, 1.0, 1, _ptr(a), _ptr(a), 0.5, _ptr(z), _ptr(z), _ptr(z), None)
    assert rc == cdx.CDX_ERR_SIZE
    assert b"CDX_NOALLOC_MAX_PIXELS" in lib.cdx_last_error()
    rc = lib.cdx_iterate_noalloc(256, 256, cdx.SHRINKWRAP, 1.0, 1, _ptr(a), _ptr(a), 0.5, _ptr(z), _ptr(z), _ptr(z),
                                 None)
    assert rc == cdx.CDX_ERR_ALGO
