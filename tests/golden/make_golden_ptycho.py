"""Generate the golden fixtures of the ptychography path from the reference's own code.

Builds the reference's ptychography driver (util/ptycho.cpp with
src/gpu/ptycho.cu, beamDecomposition.cu, cudaConfig.cu, cdi.cu,
src/post_gpu/propagator.cc, FISTA.cc, misc.cc)
as host code with oracle/build_ref.sh, runs ptycho::iterate on seeded
synthetic 32x32-probe / 64x64-object cases (inputs made by the oracle's
restatement of pupilFunc, the angular-spectrum propagator and the noise-free
createPattern), and stores inputs and outputs in tests/golden/ptycho_cases.npz.
Needs the reference checkout (default /root/reference) and g++:

    python tests/golden/make_golden_ptycho.py [/path/to/reference]

The reference's cuFFT calls run as the exact DFT in double precision
(oracle/refshim/cufft.h) and its CUB reductions as left folds; everything
else is the reference's code.  The scan order of each sweep is the
reference's rand() shuffle after srand(seed); the orders are stored too.
"""
import os
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle import ptycho_oracle as PO  # noqa: E402
from oracle.cdi_oracle import read_bin, write_bin  # noqa: E402

OUT = Path(__file__).resolve().parent / "ptycho_cases.npz"
R, RO = 32, 64

# name, n_iter, mPIE, useBS, beamStopSize, exposure, pattern scale, scan layout, seed
CASES = [
    ("obj3", 3, 1, 0, 5, 1.0, 40.0, "grid", 7),
    ("obj20_nompie", 20, 0, 0, 5, 1.0, 40.0, "grid", 11),
    ("obj30", 30, 1, 0, 5, 1.0, 40.0, "grid", 3),
    ("beamstop", 6, 1, 1, 3, 1.0, 40.0, "grid", 5),
    ("saturated", 6, 1, 0, 5, 2.0, 200.0, "grid", 9),
    ("offedge", 6, 1, 0, 5, 1.0, 40.0, "edge", 13),
    ("probe402", 402, 1, 0, 5, 1.0, 40.0, "grid", 7),
    ("refine520", 520, 0, 0, 5, 1.0, 40.0, "grid", 7),
    ("noise2003", 2003, 0, 0, 5, 1.0, 40.0, "grid", 7),
    ("fista45", 45, 1, 0, 5, 1.0, 40.0, "grid", 7),
    ("fista405", 405, 0, 0, 5, 1.0, 40.0, "grid", 3),
    ("zernike412", 412, 0, 0, 5, 1.0, 40.0, "grid", 3),
    ("zernike412_mpie", 412, 1, 0, 5, 1.0, 40.0, "grid", 7),
    ("fresnel30", 30, 1, 0, 5, 1.0, 40.0, "grid", 5),
    ("fresnel405", 405, 0, 0, 5, 1.0, 40.0, "grid", 3),
    ("posref541", 541, 0, 0, 5, 1.0, 40.0, "grid", 7),
]
NOISE_LEVEL = {"noise2003": 20}
# FISTA object step (and the probe momentum every 10); from 400 the Zernike pupil fit every 10
ZERNIKE_ITER = {"fista45": 35, "fista405": 300, "zernike412": 1200, "zernike412_mpie": 1200}
FRESNEL = {"fresnel30", "fresnel405"}   # isFresnel: the exit waves take the Fresnel phase of distance d
# positionUncertainty: the scan-position refinement every 20 sweeps from 500; the patterns are
# simulated at positions off the nominal ones by whole pixels
UNCERTAINTY = {"posref541": 2.0}
TRUE_OFFSETS = {"posref541": ([1, -1, 0, 2, 0, -1, 1, 0, -2], [0, 1, -1, 0, 2, 0, -1, 1, 0])}
OPTICS = dict(lam=0.5, d=2e4, dpupil=1e3, pixelsize=20.0, pupil_size=16.0)


def scan(layout):
    if layout == "grid":   # 3 x 3 with fractional offsets (round vs truncation differ)
        xs = [4 + 12 * i + 0.3 * j for i in range(3) for j in range(3)]
        ys = [4 + 12 * j + 0.6 * i for i in range(3) for j in range(3)]
    else:                  # windows hanging over every edge of the object
        xs = [-6.0, -3.4, 20.0, 38.5, 41.0, 10.0, 30.2]
        ys = [-5.0, 40.6, -2.5, 20.0, 39.0, 16.0, 8.7]
    return np.array(xs, np.float32), np.array(ys, np.float32)


def truth_object(rng):
    x = np.linspace(-1, 1, RO)[:, None]
    y = np.linspace(-1, 1, RO)[None, :]
    a, b = rng.uniform(1, 4, 2)
    amp = 0.6 + 0.4 * np.cos(a * x) * np.sin(b * y)
    ph = 1.2 * np.sin(2 * x + y * a)
    return (amp * np.exp(1j * ph)).astype(np.complex64)


def main(ref=None):
    ref = ref or os.environ.get("CDX_REFERENCE", "/root/reference")
    subprocess.run(["sh", str(ROOT / "oracle" / "build_ref.sh"), ref], check=True, stdout=subprocess.DEVNULL)
    harness = ROOT / "oracle" / "_ref" / "pty_harness"
    prm0 = PO.PtyParams(**OPTICS)
    res = prm0.resolution(R)
    data = {}
    with tempfile.TemporaryDirectory() as d:
        for (name, n_iter, mpie, use_bs, bss, expo, pscale, layout, seed) in CASES:
            rng = np.random.default_rng(seed)
            sx, sy = scan(layout)
            probe_t = PO.angular_spectrum(PO.pupil_func(R, R, OPTICS["pupil_size"]), OPTICS["lam"],
                                          OPTICS["dpupil"], res)
            fres = PO.fresnel_factor(OPTICS["lam"], OPTICS["d"], OPTICS["pixelsize"], R) if name in FRESNEL else 0.0
            ox, oy = (np.array(v, np.float32) for v in TRUE_OFFSETS.get(name, (np.zeros(len(sx)), np.zeros(len(sy)))))
            pats = PO.simulate_patterns(truth_object(rng), probe_t, sx + ox, sy + oy, 1.0, fresnel=fres)
            pats = (pats / pats.max() * np.float32(pscale / expo)).astype(np.float32)
            obj0 = np.exp(2j * np.pi * rng.random((RO, RO))).astype(np.complex64)
            probe0 = PO.angular_spectrum(PO.pupil_func(R, R, OPTICS["pupil_size"]), OPTICS["lam"],
                                         OPTICS["dpupil"], res)
            write_bin(f"{d}/obj.bin", obj0)
            write_bin(f"{d}/probe.bin", probe0)
            write_bin(f"{d}/pats.bin", pats.reshape(-1, R))
            with open(f"{d}/scan.txt", "w") as f:
                for a, b in zip(sx, sy):
                    f.write(f"{float(a)!r} {float(b)!r}\n")
            cmd = [str(harness), f"{d}/obj.bin", f"{d}/probe.bin", f"{d}/pats.bin", f"{d}/scan.txt", str(n_iter),
                   str(mpie), str(OPTICS["lam"]), str(OPTICS["d"]), str(OPTICS["dpupil"]), str(OPTICS["pixelsize"]),
                   str(OPTICS["pupil_size"]), str(expo), str(use_bs), str(bss), str(seed), f"{d}/out",
                   str(NOISE_LEVEL.get(name, 0)), str(ZERNIKE_ITER.get(name, 0)), str(int(name in FRESNEL)),
                   str(UNCERTAINTY.get(name, 0.0))]
            subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL)
            p = f"{name}/"
            data[p + "obj0"] = obj0
            data[p + "probe0"] = probe0
            data[p + "pats"] = pats
            data[p + "scanx"] = sx
            data[p + "scany"] = sy
            data[p + "orders"] = PO.scan_orders(len(sx), n_iter, seed)
            data[p + "cfg"] = np.array([n_iter, mpie, use_bs, bss, seed, NOISE_LEVEL.get(name, 0),
                                        ZERNIKE_ITER.get(name, 0), int(name in FRESNEL)], np.int64)
            data[p + "exposure"] = np.float64(expo)
            data[p + "uncertainty"] = np.float64(UNCERTAINTY.get(name, 0.0))
            data[p + "ref_object"] = read_bin(f"{d}/out_object.bin").copy()
            data[p + "ref_pupil"] = read_bin(f"{d}/out_pupil.bin").copy()
            print(name, "done")
    data["optics"] = np.array([OPTICS[k] for k in ("lam", "d", "dpupil", "pixelsize", "pupil_size")], np.float64)
    np.savez_compressed(OUT, **data)
    print("wrote", OUT)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
