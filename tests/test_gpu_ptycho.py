"""GPU parity of the ptychographic reconstruction (include/cdx_ptycho.h) against
the reference's own ptycho::iterate runs (tests/golden/ptycho_cases.npz) and
against the oracle (oracle/ptycho_oracle.py) one sweep at a time, plus the
set-up steps (initObject, createPattern) and the argument checks."""
import numpy as np
import pytest

from oracle import ptycho_oracle as PO
from tests.test_ptycho_oracle import CASES, load, obj_bound, pupil_bound

pytestmark = pytest.mark.gpu

# One sweep from the same state: float32 rounding of two FFT implementations.
STEP_BOUND = 1e-5


@pytest.fixture(scope="module")
def PT(cdx):
    from cdixx_gb300 import ptycho
    return ptycho


def make(PT, c, prm, rows=None, obj_shape=None):
    rows = rows or c["probe0"].shape[0]
    orow, ocol = obj_shape or c["obj0"].shape
    t = PT.Ptycho(rows, c["probe0"].shape[1], orow, ocol, c["scanx"], c["scany"], lam=prm.lam, d=prm.d,
                  dpupil=prm.dpupil, pixelsize=prm.pixelsize, pupil_size=prm.pupil_size, exposure=prm.exposure,
                  mpie=prm.mpie, use_bs=prm.use_bs, beam_stop_size=prm.beam_stop_size,
                  noise_level=prm.noise_level, position_uncertainty=prm.position_uncertainty,
                  zernike_iter=prm.zernike_iter, is_fresnel=prm.is_fresnel)
    t.objectWave = c["obj0"]
    t.probe = c["probe0"]
    t.patterns = c["pats"]
    return t


@pytest.mark.parametrize("name", CASES)
def test_gpu_matches_reference_run(PT, name):
    c, prm, n_iter, seed = load(name)
    with make(PT, c, prm) as t:
        t.iterate(n_iter, orders=c["orders"])
        assert PO.rel_err(t.objectWave, c["ref_object"]) < 2 * obj_bound(name)
        assert PO.rel_err(t.pupil, c["ref_pupil"]) < 2 * pupil_bound(name)


def test_gpu_draws_the_reference_orders_from_the_seed(PT):
    c, prm, n_iter, seed = load("obj20_nompie")
    with make(PT, c, prm) as a, make(PT, c, prm) as b:
        a.iterate(n_iter, seed=seed)
        b.iterate(n_iter, orders=c["orders"])
        assert np.array_equal(a.objectWave, b.objectWave)


# (first iteration, zernikeIter): FISTA step (and the probe momentum at 10) in the
# object phase; from 400 the pupil disk, or the Zernike pupil fit at 400, 410, 2010
SWEEPS = [(0, 400), (7, 400), (10, 400), (400, 0), (400, 1200), (410, 1200), (411, 1200), (450, 0), (520, 0),
          (2000, 0), (2010, 2100)]


@pytest.mark.parametrize("first,zernike_iter", SWEEPS)
@pytest.mark.parametrize("mpie", [False, True])
def test_one_sweep_matches_oracle(PT, first, zernike_iter, mpie):
    """Per-iterate parity: one sweep (object phase, or probe phase from 400) from
    the same object and probe as the oracle."""
    c, prm, _n, _s = load("obj3")
    prm.mpie = mpie
    prm.noise_level = 20   # the noise-tolerant projection from iteration 2000
    prm.zernike_iter = zernike_iter
    rng = np.random.default_rng(first)
    obj = (c["obj0"] * (0.5 + rng.random(c["obj0"].shape))).astype(np.complex64)
    orders = np.array([rng.permutation(len(c["scanx"]))], np.int32)
    with make(PT, c, prm) as t:
        t.objectWave = obj
        t.iterate(1, first_iter=first, orders=orders)
        O, pupil, P = PO.iterate(obj, c["probe0"], c["pats"], c["scanx"], c["scany"], 1, prm, orders, start_iter=first)
        assert PO.rel_err(t.objectWave, O) < STEP_BOUND
        assert PO.rel_err(t.probe, P) < STEP_BOUND
        assert PO.rel_err(t.pupil, pupil) < STEP_BOUND


def test_large_sweep_matches_oracle_and_reconstructs(PT):
    """256^2 probe on a 640^2 object, 16 positions: one sweep against the oracle,
    then 60 sweeps lower the far-field error of the simulated data."""
    R, RO = 256, 640
    prm = PO.PtyParams(lam=0.5, d=2e5, dpupil=2e3, pixelsize=20.0, pupil_size=160.0, exposure=1.0, mpie=True)
    res = prm.resolution(R)
    rng = np.random.default_rng(3)
    x = np.linspace(-1, 1, RO)[:, None]
    y = np.linspace(-1, 1, RO)[None, :]
    truth = ((0.6 + 0.4 * np.cos(5 * x) * np.sin(3 * y)) * np.exp(1.5j * np.sin(4 * x + 2 * y))).astype(np.complex64)
    probe = PO.angular_spectrum(PO.pupil_func(R, R, prm.pupil_size), prm.lam, prm.dpupil, res)
    sx = np.array([60 + 80 * i + 0.4 * j for i in range(4) for j in range(4)], np.float32)
    sy = np.array([60 + 80 * j + 0.7 * i for i in range(4) for j in range(4)], np.float32)
    pats = PO.simulate_patterns(truth, probe, sx, sy)
    pats = (pats / pats.max() * 0.9).astype(np.float32)
    obj0 = np.exp(2j * np.pi * rng.random((RO, RO))).astype(np.complex64)
    c = {"obj0": obj0, "probe0": probe, "pats": pats, "scanx": sx, "scany": sy}
    orders = PO.scan_orders(16, 1, 5)
    with make(PT, c, prm) as t:
        t.iterate(1, orders=orders)
        O, _pu, _P = PO.iterate(obj0, probe, pats, sx, sy, 1, prm, orders)
        assert PO.rel_err(t.objectWave, O) < STEP_BOUND

        def far_error(obj):
            sim = PO.simulate_patterns(obj, probe, sx, sy)
            return float(np.abs(np.sqrt(sim) - np.sqrt(pats)).sum() / np.sqrt(pats).sum())

        e0 = far_error(t.objectWave)
        t.iterate(60, seed=9)
        e1 = far_error(t.objectWave)
        assert e1 < 0.5 * e0, (e0, e1)


def test_zernike_sweep_at_the_reference_pupil_ratio(PT):
    """One Zernike sweep (iteration 410, zernikeIter 1200, mPIE) on a 128^2 probe with
    an 84-pixel pupil (about the reference configuration's 335 of 512) against the
    oracle, and the fitted pupil differs from the disk-cut one."""
    R, RO = 128, 256
    prm = PO.PtyParams(lam=0.5, d=5e4, dpupil=1e3, pixelsize=20.0, pupil_size=84.0, exposure=1.0, mpie=True,
                       zernike_iter=1200)
    res = prm.resolution(R)
    rng = np.random.default_rng(8)
    x = np.linspace(-1, 1, RO)[:, None]
    y = np.linspace(-1, 1, RO)[None, :]
    truth = ((0.7 + 0.3 * np.cos(4 * x) * np.sin(3 * y)) * np.exp(1j * np.sin(3 * x + y))).astype(np.complex64)
    probe = PO.angular_spectrum(PO.pupil_func(R, R, prm.pupil_size), prm.lam, prm.dpupil, res)
    sx = np.array([30 + 40 * i + 0.4 * j for i in range(3) for j in range(3)], np.float32)
    sy = np.array([30 + 40 * j + 0.7 * i for i in range(3) for j in range(3)], np.float32)
    pats = PO.simulate_patterns(truth, probe, sx, sy)
    pats = (pats / pats.max() * 0.9).astype(np.float32)
    obj0 = (truth * np.exp(0.3j * rng.random((RO, RO)))).astype(np.complex64)
    c = {"obj0": obj0, "probe0": probe, "pats": pats, "scanx": sx, "scany": sy}
    orders = PO.scan_orders(9, 1, 4)
    with make(PT, c, prm) as t:
        t.iterate(1, first_iter=410, orders=orders)
        O, pupil, P = PO.iterate(obj0, probe, pats, sx, sy, 1, prm, orders, start_iter=410)
        assert PO.rel_err(t.objectWave, O) < STEP_BOUND
        assert PO.rel_err(t.probe, P) < STEP_BOUND
        prm.zernike_iter = 0
        _O, _pu, Pdisk = PO.iterate(obj0, probe, pats, sx, sy, 1, prm, orders, start_iter=410)
        assert PO.rel_err(t.probe, Pdisk) > 100 * STEP_BOUND


@pytest.mark.parametrize("first", [0, 400])
@pytest.mark.parametrize("mpie", [False, True])
def test_one_fresnel_sweep_matches_oracle(PT, first, mpie):
    """isFresnel: one sweep with the exit waves' Fresnel phase (object phase, probe
    phase) against the oracle, and createPattern with it."""
    c, prm, _n, _s = load("fresnel30")
    prm.mpie = mpie
    rng = np.random.default_rng(first + 1)
    obj = (c["obj0"] * (0.5 + rng.random(c["obj0"].shape))).astype(np.complex64)
    orders = np.array([rng.permutation(len(c["scanx"]))], np.int32)
    with make(PT, c, prm) as t:
        t.objectWave = obj
        t.iterate(1, first_iter=first, orders=orders)
        O, pupil, P = PO.iterate(obj, c["probe0"], c["pats"], c["scanx"], c["scany"], 1, prm, orders, start_iter=first)
        assert PO.rel_err(t.objectWave, O) < STEP_BOUND
        assert PO.rel_err(t.probe, P) < STEP_BOUND
        t.objectWave = obj
        t.probe = c["probe0"]
        t.createPattern()
        fres = PO.fresnel_factor(prm.lam, prm.d, prm.pixelsize, c["probe0"].shape[0])
        ref = PO.simulate_patterns(obj, c["probe0"], c["scanx"], c["scany"], prm.exposure, fresnel=fres)
        assert np.linalg.norm(t.patterns - ref) / np.linalg.norm(ref) < 2e-6


@pytest.mark.parametrize("first", [500, 520])
@pytest.mark.parametrize("mpie", [False, True])
def test_position_update_sweep_matches_oracle(PT, first, mpie):
    """A sweep with the scan-position refinement (positionUncertainty 2): gradients per
    position, new shifts, the object shifted by their mean; against the oracle."""
    c, prm, _n, _s = load("posref541")
    prm.mpie = mpie
    rng = np.random.default_rng(first)
    obj = (c["obj0"] * (0.5 + rng.random(c["obj0"].shape))).astype(np.complex64)
    orders = np.array([rng.permutation(len(c["scanx"]))], np.int32)
    with make(PT, c, prm) as t:
        t.objectWave = obj
        t.iterate(1, first_iter=first, orders=orders)
        O, pupil, P = PO.iterate(obj, c["probe0"], c["pats"], c["scanx"], c["scany"], 1, prm, orders, start_iter=first)
        assert PO.rel_err(t.objectWave, O) < STEP_BOUND
        assert PO.rel_err(t.probe, P) < STEP_BOUND
        prm.position_uncertainty = 0.0           # without the refinement the sweep ends elsewhere
        O0, _pu, _P = PO.iterate(obj, c["probe0"], c["pats"], c["scanx"], c["scany"], 1, prm, orders, start_iter=first)
        assert PO.rel_err(t.objectWave, O0) > 10 * STEP_BOUND


def test_simulate_ccd_record_statistics(PT):
    """createPattern with simCCDbit: per pixel (Poisson(noiseLevel + rcolor I exposure), clamped
    below rcolor, - noiseLevel) / rcolor / exposure.  Against the noise-free patterns of the
    same context: the mean residual is unbiased and its variance is the Poisson one."""
    c, prm, _n, _s = load("obj3")
    prm.noise_level = 20
    prm.exposure = 1e-3
    with make(PT, c, prm) as t:
        rng = np.random.default_rng(2)
        truth = (np.exp(1j * rng.random(c["obj0"].shape)) * (0.5 + rng.random(c["obj0"].shape))).astype(np.complex64)
        t.objectWave = truth
        t.createPattern()
        clean = t.patterns
        t.createPattern(simCCDbit=True, seed=3)
        noisy = t.patterns
        t.createPattern(simCCDbit=True, seed=4)
        noisy2 = t.patterns
    rc, e, nl = 65535.0, prm.exposure, prm.noise_level
    lam = nl + rc * clean.astype(np.float64) * e
    live = lam < rc - 5 * np.sqrt(rc)                 # away from the clamp
    z = (noisy.astype(np.float64) * rc * e + nl - lam) / np.sqrt(np.maximum(lam, 1e-9))
    assert abs(z[live].mean()) < 0.05
    assert abs(z[live].std() - 1) < 0.05
    assert not np.array_equal(noisy, noisy2)
    assert np.all(noisy * rc * e + nl <= rc - 1 + 1e-2)


def test_simulate_with_beamstop_matches_oracle(PT):
    c, prm, _n, _s = load("beamstop")
    with make(PT, c, prm) as t:
        t.createPattern()
        bs = PO.circle_mask(32, 32, 16, 16, prm.beam_stop_size, True)
        ref = PO.simulate_patterns(c["obj0"], c["probe0"], c["scanx"], c["scany"], prm.exposure, bs=bs)
        assert np.linalg.norm(t.patterns - ref) / np.linalg.norm(ref) < 2e-6


def test_simulate_matches_oracle(PT):
    c, prm, _n, _s = load("offedge")
    with make(PT, c, prm) as t:
        rng = np.random.default_rng(1)
        truth = (np.exp(1j * rng.random(c["obj0"].shape)) * rng.random(c["obj0"].shape)).astype(np.complex64)
        t.objectWave = truth
        t.createPattern()
        ref = PO.simulate_patterns(truth, c["probe0"], c["scanx"], c["scany"], prm.exposure)
        got = t.patterns
        assert got.shape == ref.shape
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 2e-6


def test_init_object_matches_oracle(PT):
    c, prm, _n, _s = load("obj3")
    with make(PT, c, prm) as t:
        t.initObject(seed=4)
        o = t.objectWave
        assert np.allclose(np.abs(o), 1, atol=2e-6)
        ph = np.angle(o)
        assert ph.std() > 1.5   # uniform phase on (-pi, pi]: std pi/sqrt(3)
        ref = PO.angular_spectrum(PO.pupil_func(32, 32, prm.pupil_size), prm.lam, prm.dpupil, prm.resolution(32))
        assert PO.rel_err(t.probe, ref) < 2e-6


def test_argument_checks(PT, cdx):
    c, prm, _n, _s = load("obj3")
    prm.position_uncertainty = 2.0
    with make(PT, c, prm) as t:
        t.iterate(10, first_iter=495)              # position refinement at 500 (64^2 object: FFT size)
    c68 = dict(c, obj0=np.ones((68, 68), np.complex64))
    with make(PT, c68, prm) as t:
        with pytest.raises(cdx.CdxError) as e:
            t.iterate(10, first_iter=495)          # 68 = 4 x 17: no object transform for the shift
        assert e.value.code == cdx.CDX_ERR_SIZE
        t.iterate(5, first_iter=495)               # the run ends before the refinement
    prm.position_uncertainty = 0.0
    prm.zernike_iter = 1200
    with make(PT, c, prm) as t:
        t.iterate(5)                               # FISTA steps in the object phase
        t.iterate(5, first_iter=400)               # the Zernike pupil fit at 400
        bad = c["orders"][:2].copy()
        bad[0, 0] = 99
        with pytest.raises(cdx.CdxError):
            t.iterate(2, orders=bad)
    with pytest.raises(cdx.CdxError) as e:
        PT.Ptycho(40, 40, 64, 64, c["scanx"], c["scany"], lam=0.5, d=2e4, dpupil=1e3, pixelsize=20, pupil_size=16)
    assert e.value.code == cdx.CDX_ERR_SIZE
    with pytest.raises(cdx.CdxError):
        PT.Ptycho(32, 32, 64, 64, c["scanx"], c["scany"], lam=0.5, d=2e4, dpupil=1e3, pixelsize=20, pupil_size=40)


def test_ptycho_run_program(PT, cdx, tmp_path):
    """ptycho_run, the config-driven program: a simulation run (object and pupil
    images, triangle scan, noise-free patterns written as .bin, 30 sweeps) equals
    the same calls made through the library, and a second run reads the
    patterns and scan.txt it wrote (readPattern / readScan)."""
    import subprocess
    from pathlib import Path
    from oracle.cdi_oracle import read_bin, write_bin
    lib = Path(__file__).resolve().parents[1] / "cdixx_gb300" / "_lib"
    R, RO, step = 32, 64, 12.0
    rng = np.random.default_rng(5)
    x = np.linspace(-1, 1, RO)[:, None]
    y = np.linspace(-1, 1, RO)[None, :]
    inten = ((0.6 + 0.4 * np.cos(3 * x) * np.sin(2 * y)) ** 2).astype(np.float32)
    phase = (0.5 + 0.2 * np.sin(2 * x + y)).astype(np.float32)
    pupil_i = PO.pupil_func(R, R, 16).real.astype(np.float32)
    write_bin(tmp_path / "obj_i.bin", inten)
    write_bin(tmp_path / "obj_p.bin", phase)
    write_bin(tmp_path / "pupil_i.bin", pupil_i)
    optics = "lambda = 0.5;\n  d = 2e4;\n  dpupil = 1e3;\n  pixelsize = 20.;\n  pupilSize = 16.;\n  exposure = 1.;"
    (tmp_path / "sim.cfg").write_text(f"""
InputImages = {{ default = {{ Intensity = "obj_i.bin"; Phase = "obj_p.bin"; Pattern = "pat"; }};
                 pupil = {{ Intensity = "pupil_i.bin"; }}; }};
Job = {{
  {optics}
  stepSize = {step};
  nIter = 30;
  seed = 3;
  runSim = True;
  doIteration = True;
  outputDir = "./";
}};
""")
    r = subprocess.run([str(lib / "ptycho_run"), "sim.cfg"], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    obj_prog = read_bin(tmp_path / "ptycho_object.bin")
    assert obj_prog.shape == (RO, RO) and np.isfinite(obj_prog).all()
    # the same through the library
    sx, sy = PT.scan_triangle(RO, RO, R, R, step)
    truth = (np.sqrt(inten) * np.exp(1j * ((phase.astype(np.float64) - 0.5) * 2 * np.pi))).astype(np.complex64)
    with PT.Ptycho(R, R, RO, RO, sx, sy, lam=0.5, d=2e4, dpupil=1e3, pixelsize=20.0, pupil_size=16.0) as t:
        t.objectWave = truth
        t.pupil = np.sqrt(pupil_i).astype(np.complex64)
        t.createPattern()
        pats = t.patterns
        t.initObject(seed=3)
        t.iterate(30, seed=1)
        obj_lib = t.objectWave
    # the program builds the true object in float (cosf/sinf of a float phase), the test in
    # double: patterns 5e-8 apart, 1.2e-5 after 30 sweeps with momentum (6.6e-8 after one)
    assert PO.rel_err(obj_prog, obj_lib) < 1e-4
    saved = read_bin(tmp_path / "pat0.bin")            # centred, times the exposure
    assert PO.rel_err(np.fft.ifftshift(saved), pats[0]) < 1e-6
    # readPattern / readScan mode on what the first run wrote
    (tmp_path / "rec.cfg").write_text(f"""
InputImages = {{ default = {{ Pattern = "pat"; }}; }};
Job = {{
  {optics}
  nIter = 5;
  doIteration = True;
  distFile = "scan.txt";
  outputDir = "./";
}};
""")
    r = subprocess.run([str(lib / "ptycho_run"), "rec.cfg"], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Object image dimension" in r.stdout
    obj2 = read_bin(tmp_path / "ptycho_object.bin")
    assert np.isfinite(obj2).all() and obj2.shape[0] % 4 == 0
