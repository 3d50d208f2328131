"""The C++ drop-in layer: readConfig / AlgoParser (CPU) and cdi_run, the
config-driven entry point, end to end on the GPU against the oracle."""
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import cdi_oracle as O

ROOT = Path(__file__).resolve().parents[1]
LIBDIR = ROOT / "cdixx_gb300" / "_lib"


@pytest.fixture(scope="module")
def config_dump(cdx, tmp_path_factory):
    exe = tmp_path_factory.mktemp("cpp") / "config_dump"
    cmd = ["g++", "-std=c++17", "-O1", f"-I{ROOT / 'include'}", str(ROOT / "tests" / "cpp" / "config_dump.cc"),
           "-o", str(exe), f"-L{LIBDIR}", "-lcdx", f"-Wl,-rpath,{LIBDIR}"]
    subprocess.run(cmd, check=True)
    return exe


def parse_dump(out):
    return dict(line.split("=", 1) for line in out.strip().splitlines() if "=" in line)


def test_readconfig_parses_libconfig_subset(config_dump):
    cfg = ROOT / "tests" / "golden" / "cdi_example.cfg"
    r = subprocess.run([str(config_dump), str(cfg)], capture_output=True, text=True, check=True)
    d = parse_dump(r.stdout)
    assert d["Pattern"] == "pattern.bin" and d["restart"] == "restart.bin" and d["Intensity"] == "sample.bin"
    assert d["pupilPattern"] == "pupil.bin"
    assert float(d["oversampling"]) == 2.0 and float(d["oversampling_spt"]) == 4.0
    assert float(d["shrinkThreshold"]) == 0.15 and float(d["exposure"]) == 1.0 and float(d["lambda"]) == 2e-3
    assert int(d["beamStopSize"]) == 7 and int(d["nIter"]) == 0 and int(d["prtfIter"]) == 4401
    assert int(d["noiseLevel"]) == 24 and int(d["verbose"]) == 1
    assert d["simCCDbit"] == "1" and d["useBS"] == "0" and d["doIteration"] == "1" and d["restartFlag"] == "1"
    assert d["intensityModulation"] == "0" and d["runSim"] == "0"
    assert float(d["beta"]) == 0.9 and float(d["stepSize"]) == 32 and float(d["photoncount"]) == 1e9
    alg = d["algorithm"]
    ref = O.AlgoParser(alg).expand()
    assert int(d["steps"]) == len(ref) == 10 * 25 + 21
    assert [int(x) for x in d["first"].strip(",").split(",")] == ref[:8]


def test_readconfig_reports_syntax_errors(config_dump, tmp_path):
    bad = tmp_path / "bad.cfg"
    bad.write_text('Job = { algorithm = "10*HIO" ; oversampling = ; };\n')
    r = subprocess.run([str(config_dump), str(bad)], capture_output=True, text=True)
    assert r.returncode != 0 and "line 1" in r.stderr
    missing = subprocess.run([str(config_dump), str(tmp_path / "nope.cfg")], capture_output=True, text=True)
    assert missing.returncode != 0


def test_algoparser_unknown_token_exits_like_reference(config_dump, tmp_path):
    cfg = tmp_path / "a.cfg"
    cfg.write_text('Job = { algorithm = "10*HIO+5*BOGUS"; };\n')
    r = subprocess.run([str(config_dump), str(cfg)], capture_output=True, text=True)
    assert r.returncode == 0 and "Algorithm BOGUS not found" in r.stdout and "steps=" not in r.stdout


@pytest.mark.gpu
def test_cdi_run_end_to_end_matches_oracle(cdx, tmp_path):
    """cdi_run on a config: restart from a .bin Psi0, centred .bin pattern scaled
    by 1/exposure (cdi.cc:105-106), HIO + shrinkwrap + ER; the restart file it
    writes back (Psi) and the object dump agree with the oracle."""
    from cdixx_gb300 import synth
    n = 128
    obj, sup, I = synth.config0_case(seed=3, n=n, photons=1e6)
    psi0 = synth.random_phase_start(I, 3)
    exposure = 0.5
    O.write_bin(tmp_path / "pattern.bin", np.fft.fftshift(I) * exposure)   # centred, like a detector image
    O.write_bin(tmp_path / "restart.bin", psi0)
    alg = "2*(10*HIO+1*shrinkWrap)+4*ER"
    (tmp_path / "cdi.cfg").write_text(f"""
InputImages = {{ default = {{ Pattern = "pattern.bin"; restart = "restart.bin"; }}; }};
Job = {{
  algorithm = "{alg}";
  oversampling_spt = 2.;
  shrinkThreshold = 0.1;
  exposure = {exposure};
  nIter = 0;
  doIteration = True;
  restart = True;
  outputDir = "./";
}};
""")
    r = subprocess.run([str(LIBDIR / "cdi_run"), "cdi.cfg"], cwd=tmp_path, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "residual=" in r.stdout
    psi = O.read_bin(tmp_path / "restart.bin")
    rho = O.read_bin(tmp_path / "recon_object.bin")
    from tests._bounds import rel_l2, trajectory_bound
    ref, tol = trajectory_bound(psi0, I.astype(np.float32), alg, oversampling_spt=2.0, shrink_threshold=0.1)
    err = rel_l2(rho, ref.rho)
    assert err <= tol, (err, tol)
    assert rel_l2(psi, ref.psi) <= tol
    res = float(r.stdout.split("residual=")[1].split()[0])
    assert abs(res - ref.residual) <= max(1e-3, 2 * tol) * ref.residual
    assert (tmp_path / "support.bin").exists() and (tmp_path / "autocorrelation.bin").exists()
    # saveState post-processing (cdi.cc:266-292): centroid, crop, autocorrelation
    spt = O.read_bin(tmp_path / "support.bin")
    midx, midy = O.find_middle(spt)
    got_mid = [float(v) for v in r.stdout.split("mid=")[1].split()[0].split(",")]
    assert abs(got_mid[0] - midx) < 2e-6 and abs(got_mid[1] - midy) < 2e-6   # printed with 6 decimals
    wave = O.read_bin(tmp_path / "recon_wave.bin")
    assert wave.shape == (n // 2, n // 2)
    assert np.array_equal(wave, O.crop_about(rho, n // 2, n // 2, got_mid[0], got_mid[1]))
    ac = O.read_bin(tmp_path / "autocorrelation_recon.bin")
    assert rel_l2(ac, np.fft.fft2(np.abs(psi.astype(np.complex128)) ** 2)) < 1e-5
