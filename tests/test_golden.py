"""The oracle and the CUDA path against golden vectors produced by the
reference's own CDI::phaseRetrieve (built from the reference sources as host
code; tests/golden/make_golden.py).

Two levels (tests/_bounds.py):
  * step_k: one HIO step from the reference's own state after k-1 steps,
    for k = 1..10 -- relative L2 <= 1e-5 per iterate;
  * trajectory cases (hio_k, raar_er, mixed, shrinkwrap, ccd, ...): k steps
    from Psi0, bounded by the divergence a 1e-7 perturbation of Psi0 produces
    over the same steps (never below 1e-5); shrinkwrap masks agree >= 99.9 %.
  * PRTF cases: the reference's prtf.txt column (printed with 6 decimals),
    within the trajectory bound of the run plus the print resolution;
  * saveState: the reference's centroid ("mid=" line), the object cropped
    about it and the autocorrelation FFT(|Psi|^2), as its plotter received them.
"""
from pathlib import Path

import numpy as np
import pytest

from oracle import cdi_oracle as O
from oracle import ptycho_oracle as PO
from tests._bounds import STEP_TOL, rel_l2 as rel, trajectory_bound

GOLDEN = Path(__file__).resolve().parent / "golden" / "reference_cases.npz"
Z = np.load(GOLDEN)
CASES = sorted({k.split("/")[0] for k in Z.files
                if "/" in k and not k.startswith(("step_", "prtf_", "savestate", "sim/", "simf/"))})
PRTF_CASES = sorted({k.split("/")[0] for k in Z.files if k.startswith("prtf_")})
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


# ------------------------------------------------------------------ PRTF
def prtf_bound(name):
    alg = str(Z[f"{name}/algorithm"])
    _, tol = trajectory_bound(Z["psi0"], Z["intensity"], alg, oversampling_spt=2.0, shrink_threshold=0.1)
    return 4 * tol


@pytest.mark.parametrize("name", PRTF_CASES)
def test_oracle_prtf_matches_reference(name):
    alg, k = str(Z[f"{name}/algorithm"]), int(Z[f"{name}/prtf_iter"])
    st = O.phase_retrieve(Z["psi0"], Z["intensity"], alg, oversampling_spt=2.0, shrink_threshold=0.1, prtf_iter=k)
    ref = Z[f"{name}/prtf"]
    assert st.prtf.shape == ref.shape
    assert np.max(np.abs(st.prtf - ref)) <= prtf_bound(name) * np.max(np.abs(ref)) + 1e-6


@pytest.mark.gpu
@pytest.mark.parametrize("name", PRTF_CASES)
def test_cuda_prtf_matches_reference(cdx, name):
    alg, k = str(Z[f"{name}/algorithm"]), int(Z[f"{name}/prtf_iter"])
    I = Z["intensity"]
    n = I.shape[0]
    p = cdx.default_params(n, n, oversampling_spt=2.0, shrink_threshold=0.1, prtf_iter=k)
    with cdx.Context(p) as ctx:
        ctx.set_pattern(0, I)
        ctx.set_initial(0, np.asarray(Z["psi0"], np.complex64))
        ctx.run(alg)
        got = ctx.get_prtf(0)
    ref = Z[f"{name}/prtf"]
    e = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
    print(f"{name}: PRTF max rel diff vs the reference {e:.2e}")
    assert np.max(np.abs(got - ref)) <= prtf_bound(name) * np.max(np.abs(ref)) + 1e-6


# ------------------------------------------------------------------ saveState
def test_oracle_savestate_matches_reference():
    """find_middle, crop_about and the autocorrelation applied to the reference's
    own support, object and Psi reproduce what its saveState computed; the
    oracle's run reaches the same object."""
    mid = Z["savestate/mid"]
    spt, rho, psi = Z["savestate/support"], Z["savestate/rho"], Z["savestate/psi"]
    mx, my = O.find_middle(spt)
    assert abs(mx - mid[0]) <= 1e-6 and abs(my - mid[1]) <= 1e-6     # printed with 6 decimals
    wave = Z["savestate/wave"]
    assert np.array_equal(O.crop_about(rho, wave.shape[0], wave.shape[1], mid[0], mid[1]), wave)
    ac = np.fft.fft2(np.abs(psi.astype(np.complex128)) ** 2)
    assert rel(Z["savestate/autocorrelation"], ac) <= 1e-6
    # checkAutoCorrelation: R2C of the pattern, filled to the Hermitian spectrum, / sqrt(N)
    I = Z["intensity"].astype(np.float64)
    assert rel(Z["savestate/check_autocorrelation"], np.fft.fft2(I) / np.sqrt(I.size)) <= 1e-6
    alg = str(Z["savestate/algorithm"])
    st, tol = trajectory_bound(Z["psi0"], Z["intensity"], alg, oversampling_spt=2.0, shrink_threshold=0.1)
    assert rel(st.rho, rho) <= tol


@pytest.mark.gpu
def test_cdi_run_savestate_matches_reference(cdx, tmp_path):
    """cdi_run (the config-driven C++ entry) on the same inputs: its saveState
    dumps against the reference's (nIter = 0: no restart passes after the first
    reconstruction, util/cdi.cpp:35-46)."""
    import subprocess
    lib = Path(__file__).resolve().parents[1] / "cdixx_gb300" / "_lib"
    I = Z["intensity"]
    O.write_bin(tmp_path / "pattern.bin", np.fft.fftshift(I))
    O.write_bin(tmp_path / "restart.bin", Z["psi0"])
    alg = str(Z["savestate/algorithm"])
    (tmp_path / "cdi.cfg").write_text(f"""
InputImages = {{ default = {{ Pattern = "pattern.bin"; restart = "restart.bin"; }}; }};
Job = {{
  algorithm = "{alg}";
  oversampling_spt = 2.;
  shrinkThreshold = 0.1;
  exposure = 1.;
  nIter = 0;
  doIteration = True;
  restart = True;
  outputDir = "./";
}};
""")
    r = subprocess.run([str(lib / "cdi_run"), "cdi.cfg"], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    _, tol = trajectory_bound(Z["psi0"], I, alg, oversampling_spt=2.0, shrink_threshold=0.1)
    mid = [float(v) for v in r.stdout.split("mid=")[1].split()[0].split(",")]
    spt = O.read_bin(tmp_path / "support.bin")
    assert np.mean(spt == Z["savestate/support"]) >= 0.999
    assert np.max(np.abs(np.array(mid) - Z["savestate/mid"])) <= 2e-3
    wave = O.read_bin(tmp_path / "recon_wave.bin")
    assert wave.shape == Z["savestate/wave"].shape
    if np.allclose(mid, Z["savestate/mid"], atol=1e-6):   # same crop window: same pixels
        assert rel(wave, Z["savestate/wave"]) <= tol
    ac = O.read_bin(tmp_path / "autocorrelation_recon.bin")
    assert rel(ac, Z["savestate/autocorrelation"]) <= 2 * tol
    ac = O.read_bin(tmp_path / "autocorrelation.bin")          # checkAutoCorrelation
    assert rel(ac, Z["savestate/check_autocorrelation"]) <= 1e-5


@pytest.mark.gpu
def test_cdi_run_savestate_fresnel_removed_phase(cdx, tmp_path):
    """With isFresnel, saveState also dumps the object's phase with the Fresnel phase
    removed (cdi.cc:285-288): the phase of recon_object times the inverse Fresnel phase."""
    import subprocess
    lib = Path(__file__).resolve().parents[1] / "cdixx_gb300" / "_lib"
    I = Z["intensity"]
    O.write_bin(tmp_path / "pattern.bin", np.fft.fftshift(I))
    O.write_bin(tmp_path / "restart.bin", Z["psi0"])
    (tmp_path / "cdi.cfg").write_text("""
InputImages = { default = { Pattern = "pattern.bin"; restart = "restart.bin"; }; };
Job = {
  algorithm = "20*HIO+5*ER";
  oversampling_spt = 2.;
  exposure = 1.;
  nIter = 0;
  doIteration = True;
  restart = True;
  isFresnel = True;
  lambda = 0.6328;
  d = 2e4;
  pixelsize = 13.;
  outputDir = "./";
};
""")
    r = subprocess.run([str(lib / "cdi_run"), "cdi.cfg"], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    rho = O.read_bin(tmp_path / "recon_object.bin")
    ph = O.read_bin(tmp_path / "recon_phase_fresnelRemoved.bin")
    f = PO.fresnel_factor(0.6328, 2e4, 13.0, I.shape[0], remove=True)
    want = np.angle(PO.fresnel_phase(rho.astype(np.complex64), f))
    live = np.abs(rho) > 1e-3 * np.abs(rho).max()
    d = np.angle(np.exp(1j * (ph[live] - want[live])))
    assert np.max(np.abs(d)) < 1e-4


# ------------------------------------------------------------------ runSim
def test_oracle_sim_pattern_matches_reference():
    """The noise-free runSim pattern of the reference (readObjectWave + prepareIter)."""
    os_, pm, _ex = Z["sim/params"]
    got = O.sim_pattern(Z["sim/intensity"], Z["sim/phase"], float(os_), float(pm))
    assert rel(got, Z["sim/pattern"]) <= 1e-6
    # isFresnel: the object takes the Fresnel phase of the runSim distance first
    lam, px, bss, ospt = Z["simf/optics"]
    rows = int(Z["sim/intensity"].shape[0] * os_)
    f = PO.fresnel_factor(lam, ospt * px * bss / lam, px, rows)
    got = O.sim_pattern(Z["sim/intensity"], Z["sim/phase"], float(os_), float(pm), fresnel=f)
    assert rel(got, Z["simf/pattern"]) <= 1e-6
    assert rel(Z["sim/pattern"], Z["simf/pattern"]) > 0.1


@pytest.mark.gpu
@pytest.mark.parametrize("fresnel", [False, True])
def test_cpp_runsim_pattern_matches_reference(cdx, tmp_path, fresnel):
    """The C++ CDI layer's runSim set-up (cdi_shim readObjectWave) on the same images,
    with and without isFresnel."""
    import subprocess
    root = Path(__file__).resolve().parents[1]
    lib = root / "cdixx_gb300" / "_lib"
    exe = tmp_path / "sim_dump"
    subprocess.run(["g++", "-std=c++17", "-O1", f"-I{root / 'include'}", "-I/usr/local/cuda/include",
                    str(root / "tests" / "cpp" / "sim_dump.cc"), "-o", str(exe), f"-L{lib}", "-lcdx",
                    "-L/usr/local/cuda/lib64", "-lcudart", f"-Wl,-rpath,{lib}"], check=True)
    O.write_bin(tmp_path / "i.bin", Z["sim/intensity"])
    O.write_bin(tmp_path / "p.bin", Z["sim/phase"])
    os_, pm, ex = Z["sim/params"]
    lam, px, bss, ospt = Z["simf/optics"]
    optics = (f"lambda = {float(lam)!r}; pixelsize = {float(px)!r}; beamspotsize = {float(bss)!r}; isFresnel = True;"
              if fresnel else "")
    (tmp_path / "sim.cfg").write_text(f"""
InputImages = {{ default = {{ Intensity = "i.bin"; Phase = "p.bin"; }}; }};
Job = {{
  runSim = True;
  oversampling = {float(os_)};
  phaseModulation = {float(pm)};
  exposure = {float(ex)};
  oversampling_spt = {float(ospt)};
  {optics}
  outputDir = "./";
}};
""")
    r = subprocess.run([str(exe), "sim.cfg", "sim_out.bin"], cwd=tmp_path, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    got = O.read_bin(tmp_path / "sim_out.bin")
    ref = Z["simf/pattern" if fresnel else "sim/pattern"]
    assert got.shape == ref.shape
    assert rel(got, ref) <= 2e-6
