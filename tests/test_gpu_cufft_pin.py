"""The FP32 path against cuFFT, the FFT library the reference calls
(myFFT / myIFFT, src/gpu/cudaConfig.cu:175-180).

The oracle restates cuFFT as the exact DFT, so its own rounding is not part
of the host-built golden vectors.  Here the GPU run pins it:
  * every supported length: this library's 2-D FFT against cuFFT (through
    torch.fft, which calls it) on the same input, relative L2 <= 5e-7 (two
    float32 FFTs each ~1e-7 from the exact transform);
  * one HIO step from the same Psi0 against the reference's iteration
    structure on cuFFT -- applyModAbs, cufftExecC2C inverse, applyNorm,
    ApplyHIOSupport, cufftExecC2C forward (the bench's comparator library,
    cdixx_gb300/csrc/cufft_cmp.cu) -- relative L2 <= 1e-5 per iterate.
"""
import ctypes
from pathlib import Path

import numpy as np
import pytest

from cdixx_gb300 import synth
from tests._bounds import STEP_TOL, rel_l2

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
LENGTHS = [16, 24, 32, 48, 64, 96, 128, 192, 256, 384, 512, 768, 1024, 1536, 2048, 3072, 4096]


@pytest.mark.parametrize("n", LENGTHS)
def test_fft_matches_cufft(cdx, torch_cuda, n):
    torch = torch_cuda
    rng = np.random.default_rng(7 + n)
    x = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))).astype(np.complex64)
    xd = torch.from_numpy(x).cuda()
    out = torch.empty_like(xd)
    for inverse in (False, True):
        cdx.fft2(xd, out, inverse=inverse)
        ref = torch.fft.ifft2(xd) * (n * n) if inverse else torch.fft.fft2(xd)   # cuFFT, unnormalised
        torch.cuda.synchronize()
        e = rel_l2(out.cpu().numpy(), ref.cpu().numpy())
        assert e <= 5e-7, (n, inverse, e)


def _cmp_lib():
    lib = ctypes.CDLL(str(ROOT / "cdixx_gb300" / "_lib" / "libcdx_cufft_cmp.so"))
    lib.cmp_iterate.argtypes = [ctypes.c_int] * 4 + [ctypes.c_void_p] * 5 + [ctypes.c_float, ctypes.c_float,
                                                                              ctypes.c_void_p]
    return lib


@pytest.mark.parametrize("n", [256, 2048])
def test_one_hio_step_matches_the_reference_structure_on_cufft(cdx, torch_cuda, n):
    torch = torch_cuda
    obj, sup, I = synth.config0_case(seed=17, n=n, photons=1e8)
    psi0 = synth.random_phase_start(I, 17)
    p = cdx.default_params(n, n, oversampling_spt=4.0, beta=0.9)
    with cdx.Context(p) as ctx:
        ctx.set_pattern(0, I)
        ctx.set_initial(0, psi0)
        spt = ctx.get_support(0)
        ctx.run("1*HIO")
        rho_ours = ctx.get_object(0)
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    d_I = torch.from_numpy(I).cuda()
    d_spt = torch.from_numpy(spt).cuda()
    psi = torch.from_numpy(psi0).cuda()
    rho = torch.fft.ifft2(psi)                   # prepareIter: IFFT(Psi0)/sqrt(N), then /sqrt(N)
    rhop = torch.empty_like(rho)
    torch.cuda.synchronize()
    rc = _cmp_lib().cmp_iterate(n, n, 1, 1, P(psi), P(rho), P(rhop), P(d_I), P(d_spt), 0.5, 0.9, None)
    assert rc == 0
    torch.cuda.synchronize()
    rho_ref = rho.cpu().numpy() * np.float32(n)  # phaseRetrieve leaves rho scaled by sqrt(N)
    e = rel_l2(rho_ours, rho_ref)
    print(f"{n}^2 one HIO step against the cuFFT structure: {e:.2e}")
    assert e <= STEP_TOL
