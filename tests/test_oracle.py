"""CPU tests of the oracle (the NumPy restatement of the reference path)."""
import math

import numpy as np
import pytest

from oracle import cdi_oracle as O


def test_algoparser_reference_configs():
    # html/cdi.cfg:28 and html/default/cdi.cfg:29, html/default/pulse.cfg:27
    s = O.AlgoParser("100*(3*POSHIO+20*RAAR+1*POSHIO+1*shrinkWrap)+20*RAAR+1*ER").expand()
    unit = [O.POSHIO] * 3 + [O.RAAR] * 20 + [O.POSHIO, O.SHRINKWRAP]
    assert s == unit * 100 + [O.RAAR] * 20 + [O.ER]
    s = O.AlgoParser("200*(20*POSHIO+1*POSHIO+1*shrinkWrap)+100*POSHIO").expand()
    assert s == ([O.POSHIO] * 21 + [O.SHRINKWRAP]) * 200 + [O.POSHIO] * 100
    assert O.AlgoParser("3000*RAAR+20*ER").expand() == [O.RAAR] * 3000 + [O.ER] * 20
    assert O.AlgoParser(" 2 * HIO + 1 * ER ").expand() == [O.HIO, O.HIO, O.ER]


def test_algoparser_sequential_groups_and_default_branch():
    s = O.AlgoParser("2*(1*HIO+1*ER)+3*(1*RAAR)").expand()
    assert s == [O.HIO, O.ER, O.HIO, O.ER, O.RAAR, O.RAAR, O.RAAR]
    assert O.AlgoParser("1*KKT+1*XCORRELATION+1*FHIO").expand() == [O.KKT, O.XCORRELATION, O.FHIO]


def test_algoparser_reference_rejects_nested_groups():
    # readConfig.cc:97-108 cuts a group at the first ')', leaving "shrinkWrap)".
    with pytest.raises(O.AlgoParseError, match=r"shrinkWrap\)"):
        O.AlgoParser("5*(9*(20*HIO+1*shrinkWrap)+20*ER+1*shrinkWrap)").expand()
    with pytest.raises(O.AlgoParseError):
        O.AlgoParser("10*BOGUS").expand()


def test_fft_convention():
    x = np.zeros((8, 8), complex)
    x[1, 2] = 1
    F = O.fft2_u(x)
    kx, ky = np.meshgrid(np.arange(8), np.arange(8), indexing="ij")
    assert np.allclose(F, np.exp(-2j * np.pi * (kx * 1 + ky * 2) / 8))
    assert np.allclose(O.ifft2_u(F), 64 * x)


def test_mod_abs_edges():
    psi = np.array([3 + 4j, 0j, 1 + 1j, -2 + 0j], np.complex64)
    I = np.array([25.0, 9.0, -1.0, np.nan], np.float32)
    out = O.apply_mod_abs(psi, I)
    assert out[0] == pytest.approx(3 + 4j)
    assert out[1] == 3 + 0j            # |psi| == 0 -> sqrt(I) + 0i
    assert out[2] == 0                 # I <= 0 -> 0
    assert out[3] == 0                 # NaN fails I > 0 -> 0


def test_support_updates():
    rho = np.array([1 + 1j, 1 + 1j, 2 - 1j, 2 - 1j], np.complex128)
    rp = np.array([0.5 + 0.25j, 0.5 + 0.25j, -1 + 1j, -1 + 1j])
    spt = np.array([1.0, 0.5, 1.0, 0.0])   # 0.5 is NOT > 0.5
    hio = O.apply_support(rho, rp, spt, 0.5, O.HIO, beta=0.9)
    assert hio[0] == rp[0] and hio[1] == rho[1] - 0.9 * rp[1]
    er = O.apply_support(rho, rp, spt, 0.5, O.ER)
    assert er[0] == pytest.approx(rho[0] + 1.9 * (rp[0] - rho[0])) and er[1] == 0
    raar = O.apply_support(rho, rp, spt, 0.5, O.RAAR, beta=0.9)
    assert raar[3] == pytest.approx(0.9 * rho[3] + (1 - 1.8) * rp[3])
    poser = O.apply_support(rho, rp, spt, 0.5, O.POSER)
    assert poser[0] == rp[0] and poser[2] == 0          # rho'.x <= 0 -> 0
    ph = O.apply_support(rho, rp, spt, 0.5, O.POSHIO, beta=1.0)
    assert ph[2] == pytest.approx((2 - (-1)) + (-1 - 1) * 1j)
    f = O.apply_support(rho, rp, spt, 0.5, O.KKT)       # default branch = FHIO
    assert f[1] == pytest.approx(rho[1] - 1.2 * rp[1])


def test_rect_support_matches_reference_geometry():
    s = O.rect_support(256, 256, 4.0)
    rows = np.where(s.any(1))[0]
    assert rows[0] == 95 and rows[-1] == 160          # [95, 161)
    s2 = O.rect_support(256, 256, 2.0)
    r2 = np.where(s2.any(1))[0]
    assert r2[0] == 63 and r2[-1] == 192


def test_shrink_kernel_equals_fourier_multiply():
    # |IFFT(G . FFT(rho))|^2 == |N (k_x (x) k_y) * rho|^2 with the periodic kernels
    rng = np.random.default_rng(1)
    n = 64
    rho = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    sf = (n >> 2) / 3.0
    a = O.ifft2_u(O.gauss_mult_freq(O.fft2_u(rho), sf))
    kx = O.shrink_kernel_1d(n, sf)
    conv = np.fft.ifft2(np.fft.fft2(rho) * np.outer(np.fft.fft(kx), np.fft.fft(kx))) * n * n
    assert np.abs(a - conv).max() / np.abs(a).max() < 1e-6


def test_phase_retrieve_fp32_tracks_fp64():
    rng = np.random.default_rng(3)
    n = 32
    I = rng.random((n, n)).astype(np.float32) * 100
    psi0 = (np.sqrt(I) * np.where(rng.random((n, n)) > 0.5, -1, 1)).astype(np.complex64)
    a = O.phase_retrieve(psi0, I, "5*HIO", oversampling_spt=2.0, dtype=np.complex128)
    b = O.phase_retrieve(psi0, I, "5*HIO", oversampling_spt=2.0, dtype=np.complex64)
    assert np.linalg.norm(a.rho - b.rho) / np.linalg.norm(a.rho) < 1e-5


def test_er_fixed_point_of_consistent_object():
    # an object inside the support whose pattern is exact is a fixed point of HIO
    n = 32
    obj = np.zeros((n, n), complex)
    obj[12:20, 13:19] = np.arange(48).reshape(8, 6) + 1.0
    I = np.abs(O.fft2_u(obj)) ** 2
    spt = np.zeros((n, n))
    spt[10:22, 10:22] = 1
    st = O.phase_retrieve(O.fft2_u(obj), I, "3*HIO", support=spt)
    # phaseRetrieve hands rho back scaled by sqrt(N) (cdi.cc:406)
    assert np.allclose(st.rho / n, obj, atol=1e-9)
    assert st.residual < 1e-12 * (I ** 2).sum()


def test_bin_roundtrip(tmp_path):
    a = (np.arange(12).reshape(3, 4) + 1j).astype(np.complex64)
    O.write_bin(tmp_path / "a.bin", a)
    assert (tmp_path / "a.bin").stat().st_size == 20 + 12 * 8
    assert np.array_equal(O.read_bin(tmp_path / "a.bin"), a)


def test_residual_ignores_overexposed():
    psi = np.array([[2 + 0j, 1 + 0j]])
    I = np.array([[0.5, 1.5]])
    assert O.residual(psi, I) == pytest.approx((4 - 0.5) ** 2)


def test_threshold_state_across_shrinkwraps():
    rng = np.random.default_rng(5)
    n = 32
    I = rng.random((n, n)) * 10
    psi0 = np.sqrt(I).astype(np.complex128)
    st = O.phase_retrieve(psi0, I, "2*HIO+1*shrinkWrap+2*HIO+1*shrinkWrap", oversampling_spt=2.0,
                          shrink_threshold=0.1)
    assert st.avg > 0
    assert st.gauss_sigma == pytest.approx(float(np.float64(np.float64(3 * 0.99) * 0.99)), rel=1e-12)
    assert math.isfinite(st.threshold) and st.threshold > 0
