"""Self-checking ptychography workload for kernel captures, e.g.

    python -m cdixx_gb300.ptycho_profile --probe 512 --object 1280 --sweeps 10

Simulates noise-free patterns of a smooth object on the triangle scan of the
reference's driver (optics of its default ptychography configuration), runs
rPIE + mPIE sweeps from the random initial object and exits non-zero when the
object is not finite or the far-field error did not fall.  Prints the mean
sweep time measured with CUDA events.
"""
from __future__ import annotations

import argparse
import sys

import numpy as np


def main(argv=None):
    from cdixx_gb300 import ptycho as PT
    ap = argparse.ArgumentParser()
    ap.add_argument("--probe", type=int, default=512)
    ap.add_argument("--object", type=int, default=1280)
    ap.add_argument("--sweeps", type=int, default=10)
    ap.add_argument("--step", type=float, default=250.0)
    ap.add_argument("--first", type=int, default=0, help="iteration index of the first sweep (400+: probe phase)")
    ap.add_argument("--zernike-iter", type=int, default=0,
                    help="zernikeIter (the reference's ptycho.cfg: 1200): FISTA step, probe momentum, Zernike fit")
    a = ap.parse_args(argv)
    R, RO = a.probe, a.object
    sx, sy = PT.scan_triangle(RO, RO, R, R, a.step)
    t = PT.Ptycho(R, R, RO, RO, sx, sy, lam=0.6328, d=125e3, dpupil=6.8e3, pixelsize=13.0,
                  pupil_size=min(335.0083, R * 0.65), exposure=0.01, zernike_iter=a.zernike_iter)
    x = np.linspace(-1, 1, RO, dtype=np.float32)[:, None]
    y = np.linspace(-1, 1, RO, dtype=np.float32)[None, :]
    truth = ((0.6 + 0.4 * np.cos(9 * x) * np.sin(7 * y)) * np.exp(1.2j * np.sin(5 * x + 3 * y))).astype(np.complex64)
    t.initObject(seed=1)
    obj0 = t.objectWave
    t.objectWave = truth
    t.createPattern()
    pats = t.patterns
    t.objectWave = obj0
    t.iterate(1, first_iter=a.first, seed=3)
    t.objectWave = obj0
    ms = t.iterate(a.sweeps, first_iter=a.first, seed=5)
    obj = t.objectWave
    ok = bool(np.isfinite(obj).all())
    t.objectWave = obj
    t.createPattern()
    sim = t.patterns
    err = float(np.abs(np.sqrt(np.maximum(sim, 0)) - np.sqrt(pats)).sum() / np.sqrt(pats).sum())
    print(f"probe {R} object {RO} positions {len(sx)}: {ms / a.sweeps:.3f} ms/sweep, far-field error {err:.4f}, "
          f"finite={ok}")
    t.close()
    return 0 if ok and err < 1.0 else 1


if __name__ == "__main__":
    sys.exit(main())
