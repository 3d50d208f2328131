"""Generate the golden fixtures of the CDI path from the reference's own code.

Builds the reference's hot-path sources (src/gpu/cdi.cu, cudaConfig.cu,
cub_wrap.cu, src/post_gpu/cdi.cc, readConfig.cc, memManager.cc) as host code
with oracle/build_ref.sh, runs CDI::phaseRetrieve from a restart iterate on
seeded synthetic 64x64 patterns, and stores inputs and outputs in
tests/golden/reference_cases.npz; a smaller set at 256x256 (the plain CDI
configuration's size: 8 blobs in a 64-px disk, 1e6 photons, oversampling 4)
goes to tests/golden/reference_cases_256.npz.  Needs the reference checkout
(default /root/reference) and g++; run it in the container that has them:

    python tests/golden/make_golden.py [/path/to/reference]

The reference's cuFFT calls run as the exact DFT in double precision
(oracle/refshim/cufft.h) and its CUB reductions as left folds; everything
else is the reference's code.
"""
import os
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from cdixx_gb300 import synth  # noqa: E402
from oracle import cdi_oracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent / "reference_cases.npz"
OUT256 = Path(__file__).resolve().parent / "reference_cases_256.npz"
N = 64
# 256x256: one HIO step from the reference's own state after k-1 steps for these k
# (stored inputs Psi_{k-1} and outputs rho_k only for them, to keep the file small),
# one HIO step + shrinkwrap from its state after 9 steps, and a shrinkwrap trajectory
STEPS_256 = (1, 5, 10)
SW_TRAJ_256 = "2*(10*HIO+1*shrinkWrap)+4*ER"

# (name, algorithm, oversampling_spt, shrinkThreshold, exposure, simCCDbit, noiseLevel)
CASES = [(f"hio_{k}", f"{k}*HIO", 2.0, 0.1, 1.0, 0, 0) for k in range(1, 11)] + [
    ("raar_er", "6*RAAR+3*ER", 2.0, 0.1, 1.0, 0, 0),
    ("mixed", "2*POSHIO+2*FHIO+2*POSER+1*KKT+1*XCORRELATION", 2.0, 0.1, 1.0, 0, 0),
    ("shrinkwrap", "3*(6*HIO+1*shrinkWrap)+4*ER", 2.0, 0.1, 1.0, 0, 0),
    ("shrink_first", "1*shrinkWrap+4*HIO", 2.0, 0.05, 1.0, 0, 0),
    ("ccd", "6*HIO+2*ER", 2.0, 0.1, 0.5, 1, 3),
    ("spt4", "2*(4*RAAR+1*shrinkWrap)", 4.0, 0.2, 1.0, 0, 0),
]


# (name, algorithm, prtfIter): spt 2, shrinkThreshold 0.1, exposure 1, beta_HIO 1
PRTF_CASES = [("prtf_er", "30*ER", 10), ("prtf_hio", "12*HIO+10*ER", 6)]
SAVE_ALGO = "2*(10*HIO+1*shrinkWrap)+4*ER"
SIM_OVERSAMPLING, SIM_PHASEMOD, SIM_EXPOSURE = 2.0, 0.7, 0.5
SIM_FRESNEL_OPTICS = (0.6328, 13.0, 300.0, 2.0)   # lambda, pixelsize, beamspotsize, oversampling_spt


def main(ref=None):
    ref = ref or os.environ.get("CDX_REFERENCE", "/root/reference")
    subprocess.run([str(ROOT / "oracle" / "build_ref.sh"), ref], check=True)
    exe = ROOT / "oracle" / "_ref" / "ref_harness"
    obj, sup, I = synth.config0_case(seed=5, n=N, photons=1e6)
    psi0 = synth.random_phase_start(I, 5)
    data = {"intensity": I, "psi0": psi0}
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        for name, alg, spt, thr, exposure, ccd, noise in CASES:
            # readPattern centres nothing: the file holds the centred pattern times
            # the exposure, cudaConvertFO and 1/exposure bring it back (cdi.cc:105-106)
            O.write_bin(td / "pattern.bin", np.fft.fftshift(I) * np.float32(exposure))
            O.write_bin(td / "restart.bin", psi0)
            subprocess.run([str(exe), "pattern.bin", "restart.bin", alg, str(spt), str(thr), str(exposure), str(ccd),
                            str(noise), "out"], cwd=td, check=True, capture_output=True)
            sc = dict(line.split() for line in open(td / "out_scalars.txt"))
            data[f"{name}/rho"] = O.read_bin(td / "out_rho.bin")
            data[f"{name}/psi"] = O.read_bin(td / "out_psi.bin")
            if "shrinkWrap" in alg:
                data[f"{name}/support"] = O.read_bin(td / "out_support.bin")
            data[f"{name}/scalars"] = np.array([float(sc["threshold"]), float(sc["residual"])])
            data[f"{name}/params"] = np.array([spt, thr, exposure, ccd, noise])
            data[f"{name}/algorithm"] = np.array(alg)
        # PRTF from prtfIter on: the reference writes prtf.txt ("i, prtf[i]/weights[i]")
        for name, alg, prtf_iter in PRTF_CASES:
            O.write_bin(td / "pattern.bin", np.fft.fftshift(I))
            O.write_bin(td / "restart.bin", psi0)
            subprocess.run([str(exe), "pattern.bin", "restart.bin", alg, "2.0", "0.1", "1.0", "0", "0", "out",
                            str(prtf_iter)], cwd=td, check=True, capture_output=True)
            rows = [ln.split(",") for ln in open(td / "prtf.txt") if ln.strip()]
            data[f"{name}/prtf"] = np.array([float(r[1]) for r in rows], np.float64)
            data[f"{name}/rho"] = O.read_bin(td / "out_rho.bin")
            data[f"{name}/algorithm"] = np.array(alg)
            data[f"{name}/prtf_iter"] = np.array(prtf_iter)
        # saveState after a run with shrinkwraps: the plotted fields are dumped raw
        # (CDXREF_PLOT_DUMP), the centroid is printed as "mid= x,y"
        plots = td / "plots"
        plots.mkdir()
        O.write_bin(td / "pattern.bin", np.fft.fftshift(I))
        O.write_bin(td / "restart.bin", psi0)
        r = subprocess.run([str(exe), "pattern.bin", "restart.bin", SAVE_ALGO, "2.0", "0.1", "1.0", "0", "0", "out",
                            str(1 << 30), "1"], cwd=td, check=True, capture_output=True, text=True,
                           env={**os.environ, "CDXREF_PLOT_DUMP": str(plots)})
        mid = [float(v) for v in r.stdout.split("mid=")[1].split()[0].split(",")]
        data["savestate/algorithm"] = np.array(SAVE_ALGO)
        data["savestate/mid"] = np.array(mid)
        data["savestate/rho"] = O.read_bin(td / "out_rho_before_save.bin")
        data["savestate/psi"] = O.read_bin(td / "restart.bin")          # saveState writes Psi there
        data["savestate/support"] = O.read_bin(plots / "support.bin")   # after bitMap
        data["savestate/wave"] = O.read_bin(plots / "recon_wave.bin")   # object cropped about mid
        data["savestate/autocorrelation"] = O.read_bin(plots / "autocorrelation_recon.bin")
        data["savestate/check_autocorrelation"] = O.read_bin(plots / "autocorrelation.bin")   # checkAutoCorrelation
        # the noise-free runSim simulation (readObjectWave + prepareIter, cdi.cc:62-82, 161-200)
        rng = np.random.default_rng(11)
        m = 32
        x = np.linspace(-1, 1, m)[:, None]
        y = np.linspace(-1, 1, m)[None, :]
        inten = ((x ** 2 + y ** 2) < 0.8) * (0.5 + 0.5 * rng.random((m, m)))
        phase = rng.random((m, m))
        O.write_bin(td / "sim_i.bin", inten.astype(np.float32))
        O.write_bin(td / "sim_p.bin", phase.astype(np.float32))
        subprocess.run([str(exe), "--sim", "sim_i.bin", "sim_p.bin", str(SIM_OVERSAMPLING), str(SIM_PHASEMOD),
                        str(SIM_EXPOSURE), "sim_out.bin"], cwd=td, check=True, capture_output=True)
        data["sim/intensity"] = inten.astype(np.float32)
        data["sim/phase"] = phase.astype(np.float32)
        data["sim/params"] = np.array([SIM_OVERSAMPLING, SIM_PHASEMOD, SIM_EXPOSURE])
        data["sim/pattern"] = O.read_bin(td / "sim_out.bin")
        # the same with isFresnel: the distance of runSim (cdi.cc:39) and the object's Fresnel phase
        subprocess.run([str(exe), "--sim", "sim_i.bin", "sim_p.bin", str(SIM_OVERSAMPLING), str(SIM_PHASEMOD),
                        str(SIM_EXPOSURE), "simf_out.bin", *[str(v) for v in SIM_FRESNEL_OPTICS], "1"],
                       cwd=td, check=True, capture_output=True)
        data["simf/optics"] = np.array(SIM_FRESNEL_OPTICS)
        data["simf/pattern"] = O.read_bin(td / "simf_out.bin")
        # one step from the reference's own state after k-1 HIO steps: restart from
        # its Psi_{k-1} (prepareIter recomputes rho_{k-1} = IFFT(Psi_{k-1})/N)
        prev = psi0
        for k in range(1, 11):
            O.write_bin(td / "pattern.bin", np.fft.fftshift(I))
            O.write_bin(td / "restart.bin", prev)
            subprocess.run([str(exe), "pattern.bin", "restart.bin", "1*HIO", "2.0", "0.1", "1.0", "0", "0", "out"],
                           cwd=td, check=True, capture_output=True)
            data[f"step_{k}/rho"] = O.read_bin(td / "out_rho.bin")   # input: psi0 or hio_{k-1}/psi
            prev = data[f"hio_{k}/psi"]
    np.savez_compressed(OUT, **data)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes, {len(CASES)} cases)")
    main256(exe)


def main256(exe):
    """The 256x256 set: oversampling 4 (rect rows/cols 95..160), shrinkThreshold 0.1,
    beta_HIO 1 (the reference's fixed value)."""
    n = 256
    obj, sup, I = synth.config0_case(seed=5, n=n, photons=1e6)
    psi0 = synth.random_phase_start(I, 5)
    data = {"intensity": I, "psi0": psi0}

    def run(td, psi_in, alg):
        O.write_bin(td / "pattern.bin", np.fft.fftshift(I))
        O.write_bin(td / "restart.bin", np.asarray(psi_in, np.complex64))
        subprocess.run([str(exe), "pattern.bin", "restart.bin", alg, "4.0", "0.1", "1.0", "0", "0", "out"], cwd=td,
                       check=True, capture_output=True)
        sc = dict(line.split() for line in open(td / "out_scalars.txt"))
        return (O.read_bin(td / "out_rho.bin"), O.read_bin(td / "out_psi.bin"),
                O.read_bin(td / "out_support.bin") if "shrinkWrap" in alg else None,
                np.array([float(sc["threshold"]), float(sc["residual"])]))

    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        prev = psi0
        for k in range(1, max(STEPS_256) + 1):
            rho, psi, _, _ = run(td, prev, "1*HIO")
            if k in STEPS_256:
                data[f"step_{k}/psi_in"] = np.asarray(prev, np.complex64)
                data[f"step_{k}/rho"] = rho
            if k == 9:
                rho_s, _, spt_s, sc_s = run(td, psi, "1*HIO+1*shrinkWrap")
                data["sw_step/psi_in"] = psi
                data["sw_step/rho"] = rho_s
                data["sw_step/support"] = spt_s
                data["sw_step/scalars"] = sc_s
            prev = psi
        rho, psi, spt, sc = run(td, psi0, SW_TRAJ_256)
        data["sw_traj/algorithm"] = np.array(SW_TRAJ_256)
        data["sw_traj/rho"] = rho
        data["sw_traj/support_mask"] = np.packbits(spt > sc[0])
        data["sw_traj/scalars"] = sc
    np.savez_compressed(OUT256, **data)
    print(f"wrote {OUT256} ({OUT256.stat().st_size} bytes)")


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "--256":
        ref = sys.argv[2] if len(sys.argv) > 2 else os.environ.get("CDX_REFERENCE", "/root/reference")
        subprocess.run([str(ROOT / "oracle" / "build_ref.sh"), ref], check=True)
        main256(ROOT / "oracle" / "_ref" / "ref_harness")
    else:
        main(sys.argv[1] if len(sys.argv) > 1 else None)
