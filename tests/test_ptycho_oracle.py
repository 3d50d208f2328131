"""CPU tests of the ptychography oracle: it reproduces the reference's own
ptycho::iterate (built as host code; tests/golden/ptycho_cases.npz from
tests/golden/make_golden_ptycho.py), and the library's restatement of the C
library's rand() gives the reference's scan orders.  No kernel runs here."""
from pathlib import Path

import numpy as np
import pytest

from oracle import ptycho_oracle as PO

GOLD = Path(__file__).resolve().parent / "golden" / "ptycho_cases.npz"
CASES = ["obj3", "obj20_nompie", "obj30", "beamstop", "saturated", "offedge", "probe402", "refine520", "noise2003",
         "fista45", "fista405", "zernike412", "zernike412_mpie", "fresnel30", "fresnel405", "posref541"]
# Relative L2 bounds of oracle (and GPU) against the reference's run.  Short
# runs agree to float32 rounding; along long runs the rounding differences of
# two FFTs grow (momentum and the probe phase amplify them): measured oracle
# vs reference 2e-7..6e-7 (<= 20 sweeps), 2.1e-5 (30 sweeps with momentum),
# 4.6e-4 object / 3.6e-6 pupil (402 sweeps, two in the probe phase).  The
# long runs go without momentum (with it the probe phase drifts along the
# object/probe ambiguities, a few per cent between any two FFTs by 500 sweeps):
# 520 sweeps across the reference's first position-refinement step (a no-op at
# positionUncertainty = 0) 2.0e-5 / 1.6e-5; 2003 sweeps, the last three with
# the noise-tolerant projection (noiseLevel 20), 1.4e-3 / 9.2e-4.
# With zernikeIter (FISTA object step each sweep, probe momentum every tenth):
# 45 sweeps with momentum 1.1e-6, 405 sweeps without 7.4e-7; 412 sweeps, the Zernike
# pupil fit at 400 and 410, without momentum 4.1e-7 / 6.7e-7, with it 2.1e-6 / 8.2e-7.
# With isFresnel (phases up to 39 rad on the 32^2 frame): one sweep 7.6e-7, then the
# rounding of the phase factors grows along the run without momentum (1.6e-6 after
# 10 sweeps, 8.6e-6 after 50, 1.3e-4 after 200, 2.9e-3 / 5.6e-4 after 405; GPU builds 5e-3 to
# 1.2e-2 there, the drift being chaotic), and
# 1.1e-4 after 30 sweeps with momentum.  Scan-position refinement (positionUncertainty 2,
# patterns taken up to two pixels off the nominal positions, updates at 500, 520, 540):
# 4.7e-6 / 2.5e-6 after 541 sweeps.
OBJ_BOUND = {"obj30": 2e-4, "probe402": 3e-3, "refine520": 2e-4, "noise2003": 5e-3, "fista45": 1e-5,
             "fista405": 1e-5, "fresnel30": 2e-4, "fresnel405": 1e-2, "posref541": 1e-5}
PUPIL_BOUND = {"probe402": 1e-4, "refine520": 2e-4, "noise2003": 5e-3, "fresnel405": 2e-3, "posref541": 5e-6}


def load(name):
    z = np.load(GOLD)
    p = name + "/"
    n_iter, mpie, use_bs, bss, seed, noise, zern, fres = [int(v) for v in z[p + "cfg"]]
    opt = z["optics"]
    prm = PO.PtyParams(lam=opt[0], d=opt[1], dpupil=opt[2], pixelsize=opt[3], pupil_size=opt[4],
                       exposure=float(z[p + "exposure"]), mpie=bool(mpie), use_bs=bool(use_bs),
                       beam_stop_size=bss, noise_level=noise, zernike_iter=zern, is_fresnel=bool(fres),
                       position_uncertainty=float(z[p + "uncertainty"]))
    case = {k: z[p + k] for k in ("obj0", "probe0", "pats", "scanx", "scany", "orders", "ref_object", "ref_pupil")}
    return case, prm, n_iter, seed


def obj_bound(name):
    return OBJ_BOUND.get(name, 5e-6)


def pupil_bound(name):
    return PUPIL_BOUND.get(name, 2e-6)


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_run(name):
    c, prm, n_iter, _ = load(name)
    O, pupil, _P = PO.iterate(c["obj0"], c["probe0"], c["pats"], c["scanx"], c["scany"], n_iter, prm, c["orders"])
    assert PO.rel_err(O, c["ref_object"]) < obj_bound(name)
    assert PO.rel_err(pupil, c["ref_pupil"]) < pupil_bound(name)


def test_oracle_orders_are_glibc_shuffles():
    c, _prm, n_iter, seed = load("obj30")
    assert (PO.scan_orders(len(c["scanx"]), n_iter, seed) == c["orders"]).all()
    for row in c["orders"]:
        assert sorted(row) == list(range(len(c["scanx"])))


def test_library_rand_restatement_matches_reference_orders(cdx):
    from cdixx_gb300 import ptycho as PT
    for name in CASES:
        c, _prm, n_iter, seed = load(name)
        assert (PT.scan_orders(len(c["scanx"]), n_iter, seed) == c["orders"]).all(), name
    for seed in (0, 1, 2, 12345, 2 ** 31 - 1, 2 ** 32 - 1):
        assert (PT.scan_orders(11, 30, seed) == PO.scan_orders(11, 30, seed)).all(), seed


def test_masks_and_helpers():
    # C_circle keeps an int centre: (pd + 1)/2 = 8.5 becomes 8
    m = PO.circle_mask(16, 16, 8.5, 8.5, 8.0)
    assert (m == PO.circle_mask(16, 16, 8, 8, 8.0)).all()
    assert m[4, 15] == 0 and m[8, 1] == 1 and m[8, 0] == 0   # about (8.5, 8.5) pixel (4, 15) would be inside
    # round (window) against truncation (overlap mask)
    assert PO.c_round(2.5) == 3 and PO.c_round(-2.5) == -3 and int(np.float32(-2.5)) == -2
    # the propagator is unitary up to the evanescent cut and reversible
    rng = np.random.default_rng(0)
    f = (rng.standard_normal((32, 32)) + 1j * rng.standard_normal((32, 32))).astype(np.complex64)
    g = PO.angular_spectrum(PO.angular_spectrum(f, 0.5, 1e3, 15.625), 0.5, 1e3, 15.625, reverse=True)
    assert PO.rel_err(g, f) < 5e-3   # a = 2 pi d / lambda ~ 1.3e4 rad carries float rounding


def test_position_refinement_changes_the_run():
    """Without the refinement (positionUncertainty 0) the same run ends 4 % away from the
    reference's refined one; the restated refinement lands on it (the bound above)."""
    c, prm, n_iter, _ = load("posref541")
    prm.position_uncertainty = 0.0
    O, _pupil, _P = PO.iterate(c["obj0"], c["probe0"], c["pats"], c["scanx"], c["scany"], n_iter, prm, c["orders"])
    assert PO.rel_err(O, c["ref_object"]) > 1e-2
