"""Tensor-core FFT modes against the FP64 oracle: FFT_TC_BF16 (the radix-16
passes as tcgen05 MMAs, accumulator in TMEM) and FFT_TC_MMA (the same product
on warp-level mma.sync m16n8k16).

The radix-16 passes run as BF16 MMAs on a two-term split of each operand
(x = hi + lo, both BF16; three products, FP32 accumulate), the other passes
stay on the FP32 SIMT path.  The split keeps about 16 mantissa bits
of each operand, so the error per radix-16 pass is ~2^-17 relative instead of
FP32's 2^-24.  Stated tolerances:
  * 2-D FFT: relative L2 <= 5e-5 against float64 (measured ~1e-5),
  * one iterate from the oracle's state: relative L2 <= 1e-4,
  * full reconstructions of 8 patterns reach the same median error against
    the true object and R-factor as the FP32 mode (within 15 %, or 0.01).
"""
import numpy as np
import pytest

from cdixx_gb300 import metrics, synth
from oracle import cdi_oracle as O

pytestmark = pytest.mark.gpu

TC_FFT_TOL = 5e-5
TC_STEP_TOL = 1e-4


def rel_l2(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


SIZES = [16, 32, 48, 64, 96, 128, 256, 384, 512, 768, 1024, 1536, 2048, 3072, 4096]
MODES = ["tcgen05", "mma"]


def mode_of(cdx, name):
    return cdx.FFT_TC_BF16 if name == "tcgen05" else cdx.FFT_TC_MMA


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("n", SIZES)
def test_tc_fft2_square(cdx, torch_cuda, n, mode):
    torch = torch_cuda
    rng = np.random.default_rng(100 + n)
    batch = 2 if n <= 1024 else 1
    x = (rng.standard_normal((batch, n, n)) + 1j * rng.standard_normal((batch, n, n))).astype(np.complex64)
    xd = torch.from_numpy(x).cuda()
    out = torch.empty_like(xd)
    m = mode_of(cdx, mode)
    cdx.fft2(xd, out, inverse=False, fft_mode=m)
    torch.cuda.synchronize()
    e_f = rel_l2(out.cpu().numpy(), np.fft.fft2(x.astype(np.complex128)))
    cdx.fft2(xd, out, inverse=True, fft_mode=m)
    torch.cuda.synchronize()
    e_i = rel_l2(out.cpu().numpy(), np.fft.ifft2(x.astype(np.complex128)) * n * n)
    print(f"{mode} fft2 {n}x{n}: rel L2 vs float64 fwd {e_f:.3e} inv {e_i:.3e}")
    assert e_f < TC_FFT_TOL and e_i < TC_FFT_TOL


@pytest.mark.parametrize("shape", [(128, 256), (512, 2048), (2048, 512)])
def test_tc_fft2_rect_in_place(cdx, torch_cuda, shape):
    torch = torch_cuda
    rng = np.random.default_rng(5)
    x = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
    xd = torch.from_numpy(x).cuda()
    cdx.fft2(xd, xd, fft_mode=cdx.FFT_TC_BF16)
    torch.cuda.synchronize()
    assert rel_l2(xd.cpu().numpy(), np.fft.fft2(x.astype(np.complex128))) < TC_FFT_TOL


def test_tc_fft2_dynamic_range(cdx, torch_cuda):
    """A diffraction-like field (values spanning 1e6): the split keeps the
    error relative to the field's norm, not to each element."""
    torch = torch_cuda
    obj, sup, I = synth.config0_case(seed=3, n=512, photons=1e9)
    x = synth.random_phase_start(I, 3).astype(np.complex64)
    xd = torch.from_numpy(x).cuda()
    out = torch.empty_like(xd)
    cdx.fft2(xd, out, inverse=True, fft_mode=cdx.FFT_TC_BF16)
    torch.cuda.synchronize()
    ref = np.fft.ifft2(x.astype(np.complex128)) * x.size
    e = rel_l2(out.cpu().numpy(), ref)
    print(f"tc ifft2 of a pattern: {e:.3e}")
    assert e < TC_FFT_TOL


def test_unknown_fft_mode_is_an_error(cdx, torch_cuda):
    torch = torch_cuda
    xd = torch.zeros((64, 64), dtype=torch.complex64, device="cuda")
    with pytest.raises(cdx.CdxError):
        cdx.fft2(xd, xd, fft_mode=7)
    with pytest.raises(cdx.CdxError):
        cdx.Context(cdx.default_params(64, 64, fft_mode=7))


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("algo,beta", [("HIO", 1.0), ("RAAR", 0.9), ("ER", 1.0)])
def test_tc_one_step_per_iterate(cdx, algo, beta, mode):
    """From the FP64 oracle's state after k-1 steps, one TC step gives rho_k
    within relative L2 1e-4 of the oracle's."""
    obj, sup, I = synth.config0_case(seed=11, n=256, photons=1e6)
    psi0 = synth.random_phase_start(I, 11)
    steps = 6
    ref = O.phase_retrieve(psi0, I, f"{steps}*{algo}", oversampling_spt=4.0, beta=beta, record=set(range(steps)))
    p = cdx.default_params(256, 256, oversampling_spt=4.0, beta=beta, fft_mode=mode_of(cdx, mode))
    worst = 0.0
    with cdx.Context(p) as ctx:
        ctx.set_pattern(0, I)
        state = psi0.astype(np.complex128)
        for k in range(steps):
            ctx.set_initial(0, state.astype(np.complex64))
            ctx.run(f"1*{algo}")
            rho_k, psi_k = ref.history[k][0], ref.history[k][1]
            e = rel_l2(ctx.get_object(0), rho_k * 256.0)
            worst = max(worst, e)
            assert e <= TC_STEP_TOL, (algo, k + 1, e)
            state = psi_k
    print(f"{mode} {algo}: worst one-step rel L2 {worst:.3e}")


def test_tc_reconstruction_quality_matches_fp32(cdx):
    """Full reconstructions with shrinkwrap of 8 patterns: both FFT modes reach
    the same error against the true object and the same R-factor (medians
    within 15 %, or 0.01 absolute: single trajectories are chaotic, and the two
    modes round differently from the first step)."""
    n, count = 256, 8
    cases = [synth.config0_case(seed=21 + k, n=n, photons=1e7) for k in range(count)]
    alg = "100*RAAR+1*shrinkWrap+100*RAAR+1*shrinkWrap+100*HIO+1*shrinkWrap+50*ER"
    res = {}
    for mode in (cdx.FFT_FP32, cdx.FFT_TC_BF16):
        p = cdx.default_params(n, n, batch=count, oversampling_spt=2.0, beta=0.9, shrink_threshold=0.15,
                               fft_mode=mode)
        with cdx.Context(p) as ctx:
            for k, (obj, sup, I) in enumerate(cases):
                ctx.set_pattern(k, I)
                ctx.set_initial(k, synth.random_phase_start(I, 21 + k))
            ctx.run(alg)
            e = [metrics.error_vs_truth(ctx.get_object(k), cases[k][0]) for k in range(count)]
            r = [ctx.stats(k)["rfactor"] for k in range(count)]
        res[mode] = (float(np.median(e)), float(np.median(r)))
    (e32, r32), (etc, rtc) = res[cdx.FFT_FP32], res[cdx.FFT_TC_BF16]
    print(f"median error vs truth: fp32 {e32:.4f} (R {r32:.4f}), tc {etc:.4f} (R {rtc:.4f})")
    assert etc <= max(1.15 * e32, e32 + 0.01)
    assert rtc <= max(1.15 * r32, r32 + 0.01)


def test_tc_batch_matches_single(cdx):
    """The TC mode gives identical bits whether a pattern runs alone or in a batch."""
    cases = [synth.config0_case(seed=s, n=128)[2] for s in (1, 2)]
    starts = [synth.random_phase_start(I, s) for I, s in zip(cases, (1, 2))]
    alg = "6*HIO+1*shrinkWrap+3*ER"
    p = cdx.default_params(128, 128, batch=2, oversampling_spt=2.0, shrink_threshold=0.1,
                           fft_mode=cdx.FFT_TC_BF16)
    with cdx.Context(p) as ctx:
        for i in range(2):
            ctx.set_pattern(i, cases[i])
            ctx.set_initial(i, starts[i])
        ctx.run(alg)
        both = [ctx.get_object(i) for i in range(2)]
    for i in range(2):
        q = cdx.default_params(128, 128, oversampling_spt=2.0, shrink_threshold=0.1, fft_mode=cdx.FFT_TC_BF16)
        with cdx.Context(q) as ctx:
            ctx.set_pattern(0, cases[i])
            ctx.set_initial(0, starts[i])
            ctx.run(alg)
            assert np.array_equal(ctx.get_object(0), both[i])
