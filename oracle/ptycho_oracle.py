"""CPU oracle for the ptychographic reconstruction (rPIE object and probe updates).

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import this
module.  It is the checker, never the product: the product path lives in
``cdixx_gb300`` (``cdx_pty_*`` in include/cdx_ptycho.h).

NumPy restatement of the reference's ``ptycho::iterate`` (util/ptycho.cpp:429-736)
and the kernels it calls (src/gpu/ptycho.cu, src/gpu/cdi.cu, src/gpu/cudaConfig.cu,
src/post_gpu/propagator.cc, src/post_gpu/misc.cc), in complex64 / float32 with
the reference's scalar types (float parameters; the double literals and double
config fields where the reference has them).  The FFT is the unnormalised DFT
via NumPy (cuFFT's published transform), reductions accumulate in float64.

Scope: the iteration with the FISTA object step, the Zernike pupil fit and the
Fresnel exit-wave phase, without scan-position refinement.  From iteration 500 the reference refines the
positions every 20 sweeps; with positionUncertainty = 0 (its default) that
leaves every shift at zero and the object changed only by the rounding of an
FFT round trip, which is not repeated here; runs with positionUncertainty > 0
past iteration 500 are refused.  It is pinned by the reference's own driver
built as host code (oracle/build_ref.sh -> oracle/_ref/pty_harness).
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass

import numpy as np

F32 = np.float32
C64 = np.complex64

ALPHA = F32(0.1)    # src/gpu/ptycho.cu:5
BETA = F32(0.5)     # src/gpu/ptycho.cu:6
UPDATE_PROBE_ITER = 400      # util/ptycho.cpp:441
POSITION_UPDATE_ITER = 500   # util/ptycho.cpp:442
NOISE_PROJ_ITER = 2000       # applyMod instead of applyModAccurate, util/ptycho.cpp:536-545
RCOLOR = F32(65535)          # include/format.hpp:21


# --------------------------------------------------------------------------- FFT
def fft2_u(a):
    """Unnormalised forward 2-D DFT (myFFT, CUFFT_FORWARD)."""
    return np.fft.fft2(a).astype(C64)


def ifft2_u(a):
    """Unnormalised inverse 2-D DFT (myIFFT, CUFFT_INVERSE)."""
    n = a.shape[0] * a.shape[1]
    return (np.fft.ifft2(a) * n).astype(C64)


def convert_fo(a):
    """cudaConvertFO (src/gpu/cudaConfig.cu:202-212): swap the quadrants
    (an fftshift for the even sizes used here)."""
    return np.fft.fftshift(a)


# ----------------------------------------------------------- rand() and order
class GlibcRand:
    """glibc's rand()/srand() through ctypes: the reference shuffles the scan
    order with rand() (util/ptycho.cpp:28-38) after the process's srand()."""

    def __init__(self, seed: int):
        self.libc = ctypes.CDLL(None)
        self.libc.srand(ctypes.c_uint(seed))

    def rand(self) -> int:
        return int(self.libc.rand())


def shuffle_array(order, rng):
    """shuffle_array (util/ptycho.cpp:28-38): Fisher-Yates from the top with rand() % (i + 1)."""
    n = len(order)
    for i in range(n - 1, 0, -1):
        j = rng.rand() % (i + 1)
        order[i], order[j] = order[j], order[i]


def scan_orders(nscan: int, n_iter: int, seed: int):
    """The scan order of every iteration: iterOrder starts as the identity and
    is shuffled in place once per iteration (util/ptycho.cpp:466-469, 512)."""
    rng = GlibcRand(seed)
    order = list(range(nscan))
    out = []
    for _ in range(n_iter):
        shuffle_array(order, rng)
        out.append(list(order))
    return np.array(out, np.int32).reshape(n_iter, nscan)


# --------------------------------------------------------------------- masks
def circle_mask(rows, cols, x0, y0, r, is_freq=False):
    """createCircleMask (src/post_gpu/misc.cc:161-170) -> createMask<C_circle>
    (src/gpu/cudaConfig.cu:1291-1299, C_circle::isInside 93-97): 1 where
    sqrtf(dx^2 + dy^2) < r, dx = x - x0 in float; the centre is stored in the
    int members of C_circle (include/cudaConfig.hpp:217-221), so a fractional
    x0, y0 is truncated."""
    x = np.arange(rows)[:, None]
    y = np.arange(cols)[None, :]
    if is_freq:
        x = np.where(x >= rows // 2, x - rows // 2, x + rows // 2)
        y = np.where(y >= cols // 2, y - cols // 2, y + cols // 2)
    dx = (x - int(F32(x0))).astype(F32)
    dy = (y - int(F32(y0))).astype(F32)
    dr = np.sqrt((dx * dx + dy * dy).astype(F32))
    return (dr < F32(r)).astype(F32)


def pupil_func(rows, cols, pupilsize):
    """pupilFunc (src/gpu/ptycho.cu:123-130): 1 + 0i inside the disk
    shiftx^2 + shifty^2 <= pupilsize^2 / 4 about (rows/2, cols/2), else 0."""
    sx = np.arange(rows)[:, None] - rows // 2
    sy = np.arange(cols)[None, :] - cols // 2
    ps = F32(pupilsize)
    inside = (sx * sx + sy * sy).astype(F32) <= F32(ps * ps) / F32(4)
    return inside.astype(C64)


def masksum(rows, cols, obj_rows, obj_cols, scanx, scany, pupil_size):
    """The overlap mask of util/ptycho.cpp:470-479: a disk of diameter
    pupilSize at the centre of the probe frame added at every scan position
    (addWindow, src/gpu/ptycho.cu:35-41; the float position is truncated to
    int by the call), then bitMap(> 0.5)."""
    disk = circle_mask(rows, cols, rows >> 1, cols >> 1, F32(np.float64(pupil_size) / 2))
    acc = np.zeros((obj_rows, obj_cols), F32)
    for px, py in zip(scanx, scany):
        sx, sy = int(F32(px)), int(F32(py))
        _add_window(acc, sx, sy, disk)
    return (acc > F32(0.5)).astype(F32)


def _window_ranges(shape_o, sx, sy, rows, cols):
    x0, y0 = max(0, -sx), max(0, -sy)
    x1, y1 = min(rows, shape_o[0] - sx), min(cols, shape_o[1] - sy)
    return x0, x1, y0, y1


def _add_window(obj, sx, sy, win):
    rows, cols = win.shape
    x0, x1, y0, y1 = _window_ranges(obj.shape, sx, sy, rows, cols)
    if x1 > x0 and y1 > y0:
        obj[x0 + sx:x1 + sx, y0 + sy:y1 + sy] = (win[x0:x1, y0:y1] + obj[x0 + sx:x1 + sx, y0 + sy:y1 + sy]).astype(obj.dtype)


def get_window(obj, sx, sy, rows, cols):
    """getWindow (src/gpu/ptycho.cu:18-24): the rows x cols window at (sx, sy),
    zero outside the object."""
    w = np.zeros((rows, cols), obj.dtype)
    x0, x1, y0, y1 = _window_ranges(obj.shape, sx, sy, rows, cols)
    if x1 > x0 and y1 > y0:
        w[x0:x1, y0:y1] = obj[x0 + sx:x1 + sx, y0 + sy:y1 + sy]
    return w


def update_window(obj, sx, sy, win):
    """updateWindow (src/gpu/ptycho.cu:26-30): write the window back inside the object."""
    rows, cols = win.shape
    x0, x1, y0, y1 = _window_ranges(obj.shape, sx, sy, rows, cols)
    if x1 > x0 and y1 > y0:
        obj[x0 + sx:x1 + sx, y0 + sy:y1 + sy] = win[x0:x1, y0:y1]


def c_round(v) -> int:
    """round() of the C library (halves away from zero) as passed to an int parameter."""
    v = float(F32(v))
    return int(math.floor(abs(v) + 0.5)) * (1 if v >= 0 else -1)


# ----------------------------------------------------------------- kernels
def apply_mod_accurate(F, pattern, norm, scale, bs=None):
    """applyModAccurate, 4-argument form (src/gpu/cdi.cu:351-388): F * norm,
    replaced by sqrt(I / |F norm|^2) * F norm except where the beamstop
    blocks (kept scaled), where |F norm| == 0 (left as it was) and where the
    pixel is saturated (I >= 0.95 scale and |F norm|^2 >= I: kept scaled)."""
    mod2 = np.maximum(F32(0), pattern.astype(F32))
    rx = (F.real * F32(norm)).astype(F32) if norm != 1 else F.real.astype(F32)
    ry = (F.imag * F32(norm)).astype(F32) if norm != 1 else F.imag.astype(F32)
    src = (rx * rx + ry * ry).astype(F32)
    maximum = F32(F32(scale) * F32(0.95))
    with np.errstate(divide="ignore", invalid="ignore"):
        s = np.sqrt((mod2 / np.where(src == 0, F32(1), src)).astype(F32))
    keep = (mod2 >= maximum) & (src >= mod2)
    s = np.where(keep, F32(1), s).astype(F32)
    out = ((s * rx).astype(F32) + 1j * (s * ry).astype(F32)).astype(C64)
    out = np.where(src == 0, F, out)
    if bs is not None:
        blocked = bs > F32(0.5)
        out = np.where(blocked, (rx + 1j * ry).astype(C64), out)
    return out.astype(C64)


def apply_mod_noise(F, pattern, norm, scale, noise_level, bs=None):
    """applyMod, 5-argument form with bsnorm (src/gpu/cdi.cu:438-485): the projection
    toward the measured intensity stops a tolerance sqrt(noise + I rcolor/scale)
    scale/rcolor short of it; saturated pixels (I >= 0.95 scale) take max(I, |F|^2)."""
    mod2 = np.maximum(F32(0), pattern.astype(F32))
    rx = (F.real * F32(norm)).astype(F32) if norm != 1 else F.real.astype(F32)
    ry = (F.imag * F32(norm)).astype(F32) if norm != 1 else F.imag.astype(F32)
    src = (rx * rx + ry * ry).astype(F32)
    sc = F32(scale)
    mod2 = np.where(mod2 >= F32(sc * F32(0.95)), np.maximum(mod2, src), mod2).astype(F32)
    tol = (np.sqrt((F32(noise_level) + ((mod2 * RCOLOR).astype(F32) / sc).astype(F32)).astype(F32)) * sc / RCOLOR).astype(F32)
    diff = (mod2 - src).astype(F32)
    val = np.where(diff > tol, mod2 - tol, np.where(diff < -tol, mod2 + tol, mod2)).astype(F32)
    with np.errstate(divide="ignore", invalid="ignore"):
        s = np.sqrt((np.maximum(val, F32(0)) / np.where(src == 0, F32(1), src)).astype(F32)).astype(F32)
    out = ((s * rx).astype(F32) + 1j * (s * ry).astype(F32)).astype(C64)
    out = np.where(src == 0, (val + 0j).astype(C64), out)
    if bs is not None:
        out = np.where(bs > F32(0.5), (rx + 1j * ry).astype(C64), out)
    return out.astype(C64)


def _rpie_denom(source_mod2, maxi, param, stepsize):
    """The denominator of rPIE / rPIE_step (src/gpu/ptycho.cu:55-68):
    stepsize / ((1 - param) |s|^2 + param max(maxi, 1e-5)), the max and the
    sum in double (max(float, double)), the result stored as float."""
    a = ((F32(1) - F32(param)) * source_mod2).astype(F32).astype(np.float64)
    b = np.float64(F32(param)) * max(np.float64(F32(maxi)), 1e-5)
    return (np.float64(stepsize) / (a + b)).astype(F32)


def rpie(target, source, diff, maxi, param, stepsize=1.0):
    """rPIE (src/gpu/ptycho.cu:55-61): target -= conj(source) diff * denom."""
    sx, sy = source.real.astype(F32), source.imag.astype(F32)
    dx, dy = diff.real.astype(F32), diff.imag.astype(F32)
    d = _rpie_denom((sx * sx + sy * sy).astype(F32), maxi, param, stepsize)
    tx = (target.real - ((sx * dx + sy * dy).astype(F32) * d).astype(F32)).astype(F32)
    ty = (target.imag - ((sx * dy - sy * dx).astype(F32) * d).astype(F32)).astype(F32)
    return (tx + 1j * ty).astype(C64)


def rpie_step(source, diff, maxi, param):
    """rPIE_step (src/gpu/ptycho.cu:62-68): -conj(source) diff * denom (stepsize 1)."""
    sx, sy = source.real.astype(F32), source.imag.astype(F32)
    dx, dy = diff.real.astype(F32), diff.imag.astype(F32)
    d = _rpie_denom((sx * sx + sy * sy).astype(F32), maxi, param, 1.0)
    return (-((sx * dx + sy * dy).astype(F32) * d) - 1j * ((sx * dy - sy * dx).astype(F32) * d)).astype(C64)


def angular_spectrum(field, lam, distance, pixelsize, reverse=False):
    """propagator::angularSpectrumPropagate / ...Reverse (src/post_gpu/propagator.cc:31-49)
    with multiplyPropagatePhase (src/gpu/cudaConfig.cu:669-679): FFT, 1/(rows cols),
    centre, multiply by exp(i a sqrt(1 - ((x - r/2)^2 + (y - c/2)^2) b)) (0 where
    the root is imaginary), uncentre, inverse FFT.  The propagator's members are
    float; a = 2 pi distance / lambda is evaluated in double."""
    rows, cols = field.shape
    lam32, dist32, ps32 = F32(lam), F32(distance), F32(pixelsize)
    if not reverse:
        a = F32(2 * math.pi * np.float64(dist32) / np.float64(lam32))
        loi = F32(lam32 / F32(ps32 * F32(rows)))
        b = F32(loi * loi)
    else:
        a = F32(-2 * math.pi * np.float64(dist32) / np.float64(lam32))
        iol = F32(F32(ps32 * F32(rows)) / lam32)
        b = F32(1.0 / np.float64(F32(iol * iol)))
    out = fft2_u(field)
    out = (out * F32(1.0 / (rows * cols))).astype(C64)
    out = convert_fo(out)
    x = np.arange(rows)[:, None] - (rows >> 1)
    y = np.arange(cols)[None, :] - (cols >> 1)
    square = (F32(1) - ((x * x + y * y).astype(F32) * b).astype(F32)).astype(F32)
    ok = square >= 0
    phase = (a * np.sqrt(np.where(ok, square, F32(0))).astype(F32)).astype(F32)
    ph = phase.astype(np.float64)
    fac = (np.cos(ph) + 1j * np.sin(ph)).astype(C64)
    out = np.where(ok, (out * fac).astype(C64), 0).astype(C64)
    out = convert_fo(out)
    return ifft2_u(out)


def fista_step(b, lam=0.01):
    """FISTA_step (src/post_gpu/FISTA.cc:109-135) of the complex object, one TV
    proximal step: o = b * (0.125 / lambda); p, q = forward differences of o along
    x and y (partialx / partialy, src/gpu/cudaConfig.cu:1124-1150: the last row /
    column keeps o itself); each component of (p, q) scaled to modulus <= 1
    (diffMax, 1158-1170); lpq = p + q - p(x-1) - q(y-1) (no wrap, calcLpq
    1180-1188); result b - lambda lpq, all in float."""
    lam = F32(lam)
    s = F32(0.125 / np.float64(lam))
    o = (b.astype(C64) * s).astype(C64)
    ore, oim = o.real.astype(F32), o.imag.astype(F32)

    def parts(a):
        p = a.copy()
        p[:-1, :] = (a[:-1, :] - a[1:, :]).astype(F32)
        q = a.copy()
        q[:, :-1] = (a[:, :-1] - a[:, 1:]).astype(F32)
        mod = np.hypot(p, q).astype(F32)
        big = mod > F32(1)
        safe = np.where(big, mod, F32(1))
        p = np.where(big, (p / safe).astype(F32), p)
        q = np.where(big, (q / safe).astype(F32), q)
        lpq = (p + q).astype(F32)
        lpq[1:, :] = (lpq[1:, :] - p[:-1, :]).astype(F32)
        lpq[:, 1:] = (lpq[:, 1:] - q[:, :-1]).astype(F32)
        return lpq

    lr, li = parts(ore), parts(oim)
    out_r = (b.real.astype(F32) + (lr * -lam).astype(F32)).astype(F32)
    out_i = (b.imag.astype(F32) + (li * -lam).astype(F32)).astype(F32)
    return (out_r + 1j * out_i).astype(C64)


def find_middle(m):
    """findMiddle of a float field (src/post_gpu/misc.cc:27-42) with multiplyx/multiplyy
    (src/gpu/cudaConfig.cu:1427-1437): centroid in units of the size, coordinate
    (x + 0.5)/rows - 0.5 (in double), sums then a float division."""
    rows, cols = m.shape
    m64 = m.astype(np.float64)
    cx = ((np.arange(rows) + 0.5) / rows - 0.5)[:, None]
    cy = ((np.arange(cols) + 0.5) / cols - 0.5)[None, :]
    wx = (m64 * cx).astype(F32).astype(np.float64)
    wy = (m64 * cy).astype(F32).astype(np.float64)
    s = F32(m64.sum())
    return F32(F32(wx.sum()) / s), F32(F32(wy.sum()) / s)


def multiply_shift(wave, shiftx, shifty):
    """multiplyShift (src/gpu/cudaConfig.cu:373-378): wave * exp(-2 pi i (shiftx (x - r/2)/r
    + shifty (y - c/2)/c)), the bracket in float."""
    rows, cols = wave.shape
    x = (np.arange(rows) - rows // 2).astype(F32)[:, None]
    y = (np.arange(cols) - cols // 2).astype(F32)[None, :]
    t = ((F32(shiftx) * x).astype(F32) / F32(rows)).astype(F32) + ((F32(shifty) * y).astype(F32) / F32(cols)).astype(F32)
    ph = (F32(-2 * math.pi) * t.astype(F32)).astype(F32).astype(np.float64)
    return (wave * (np.cos(ph) + 1j * np.sin(ph)).astype(C64)).astype(C64)


def fresnel_factor(lam, distance, pixelsize, rows, remove=False):
    """propagator::multiplyFresnelPhase / removeFresnelPhase (src/post_gpu/propagator.cc:15-20):
    pi lambda distance / (pixelsize rows)^2 of the propagator's float members, in double,
    passed on as float."""
    side = F32(F32(pixelsize) * F32(rows))
    f = math.pi * float(F32(lam)) * float(F32(distance)) / float(F32(side * side))
    return F32(-f if remove else f)


def fresnel_phase(a, factor):
    """multiplyFresnelPhase_Device (src/gpu/cudaConfig.cu:1095-1101): a exp(i factor ((x - rows/2)^2
    + (y - cols/2)^2)) on the entries that are not zero, the squared distance in integers and
    the phase in float."""
    rows, cols = a.shape
    dx = (np.arange(rows) - (rows >> 1))[:, None]
    dy = (np.arange(cols) - (cols >> 1))[None, :]
    ph = (F32(factor) * (dx * dx + dy * dy).astype(F32)).astype(F32).astype(np.float64)
    p = (np.cos(ph) + 1j * np.sin(ph)).astype(C64)
    return np.where(a != 0, (a * p).astype(C64), a).astype(C64)


# ------------------------------------------------------- position refinement
DELTA = F32(1e-3)        # src/gpu/ptycho.cu:7
POSITION_STEP = F32(0.3)  # util/ptycho.cpp:569


def position_gradient(w, P, Fn, pattern, bs=None):
    """ptycho::updatePosition (util/ptycho.cpp:360-385) with calcPartial (src/gpu/ptycho.cu:156-169):
    the window's spectrum, centred and scaled by sqrt(1/n), times (x/rows - 0.5) and
    (y/cols - 0.5), back to FFT order scaled by 1/n, inverse transforms, times the probe,
    forward transforms; per pixel (Fn.x d.y - Fn.y d.x)(1 - sqrt((I + 1e-3)/(|Fn|^2 + 1e-3)))
    (zero under the beamstop) summed.  Fn is the exit wave's transform times 1/sqrt(n).
    Returns (gx, gy)."""
    rows, cols = w.shape
    nrm = F32(1.0 / (rows * cols))
    s1 = F32(math.sqrt(nrm))
    spec = np.fft.fftshift(fft2_u(w.astype(C64))).astype(C64)
    spec = (spec * s1).astype(C64)
    sx = ((np.arange(rows, dtype=F32) * F32(1.0 / rows)).astype(F32) - F32(0.5)).astype(F32)[:, None]
    sy = ((np.arange(cols, dtype=F32) * F32(1.0 / cols)).astype(F32) - F32(0.5)).astype(F32)[None, :]
    fact = np.maximum((pattern.astype(F32) + DELTA).astype(F32), F32(0))
    fm2 = (Fn.real * Fn.real + Fn.imag * Fn.imag).astype(F32)
    k = (F32(1) - np.sqrt((fact / (fm2 + DELTA).astype(F32)).astype(F32)).astype(F32)).astype(F32)
    out = []
    for sc in (sx, sy):
        d = np.fft.ifftshift((spec * sc).astype(C64)).astype(C64)
        d = (d * nrm).astype(C64)
        d = (ifft2_u(d) * P).astype(C64)
        d = fft2_u(d)
        part = ((Fn.real * d.imag).astype(F32) - (Fn.imag * d.real).astype(F32)).astype(F32)
        part = (part * k).astype(F32)
        if bs is not None:
            part = np.where(bs > F32(0.5), F32(0), part)
        out.append(F32(part.astype(np.float64).sum()))
    return out[0], out[1]


def shift_wave(wave, shiftx, shifty):
    """shiftWave (src/post_gpu/misc.cc:97-113): FFT, centre, multiplyShift
    (cudaConfig.cu:373-378) by (shiftx, shifty), back to FFT order, times 1/(rows cols),
    inverse FFT."""
    rows, cols = wave.shape
    spec = np.fft.fftshift(fft2_u(wave.astype(C64))).astype(C64)
    spec = multiply_shift(spec, shiftx, shifty)
    spec = (np.fft.ifftshift(spec) * F32(1.0 / (rows * cols))).astype(C64)
    return ifft2_u(spec).astype(C64)


def add_probability(shifts, grad, sigma):
    """addProbability (cudaConfig.cu:808-817): d + v (v = 0.3 grad), damped by
    exp(-(d + v)^2 / (2 sigma^2)) when the step moves away from zero."""
    out = shifts.astype(F32).copy()
    for j in range(out.size):
        d = F32(out.flat[j])
        v = F32(F32(grad.flat[j]) * POSITION_STEP)
        t = F32(d + v)
        if abs(t) > abs(d):
            g = F32(math.exp(float(-F32(F32(F32(t * t) / F32(2)) / F32(F32(sigma) * F32(sigma))))))
            out.flat[j] = F32(d + F32(v * g))
        else:
            out.flat[j] = t
    return out


# ------------------------------------------------------- Zernike pupil fit
ZERNIKE_MAX_N = 40                      # util/ptycho.cpp:439
ZERNIKE_REG_L, ZERNIKE_REG_M = F32(5e-5), F32(5e-8)   # beamDecomposition.cu:585-588


def pixel_coverage(px, py, r):
    """compute_pixel (src/gpu/beamDecomposition.cu:11-104): the area of the unit
    pixel centred at (px, py) inside the circle of radius r about the origin and
    that area's centroid.  Pixels further than r + sqrt(2) are out, nearer than
    r - sqrt(2) in; a pixel with all four corners in (or out) counts whole (or
    not at all); otherwise the polygon of its inside corners and the circle's
    crossings of its edges (sorted by angle about the pixel centre, shoelace
    area and first moments), plus the circular segment beyond the chord when
    there are two crossings.  Float arithmetic as the reference's."""
    f = F32
    px, py, r = f(px), f(py), f(r)
    r2 = f(r * r)
    d2 = f(f(px * px) + f(py * py))
    s2 = f(math.sqrt(2.0))
    if d2 > f(f(r + s2) * f(r + s2)):
        return f(0), px, py
    if d2 < f(f(r - s2) * f(r - s2)):
        return f(1), px, py
    x0, x1, y0, y1 = f(px - f(0.5)), f(px + f(0.5)), f(py - f(0.5)), f(py + f(0.5))
    inside = [f(f(x0 * x0) + f(y0 * y0)) < r2, f(f(x1 * x1) + f(y0 * y0)) < r2,
              f(f(x1 * x1) + f(y1 * y1)) < r2, f(f(x0 * x0) + f(y1 * y1)) < r2]
    n_in = sum(inside)
    if n_in == 4:
        return f(1), px, py
    if n_in == 0:
        return f(0), px, py
    eps = f(1e-5)
    ints = []

    def dup(x, y):
        return any(abs(f(a - x)) < eps and abs(f(b - y)) < eps for a, b in ints)

    for x in (x0, x1):                   # crossings of the vertical edges
        val = f(f(r - x) * f(r + x))
        if val >= -eps:
            y = f(math.sqrt(max(val, f(0))))
            if f(y0 - eps) <= y <= f(y1 + eps) and not dup(x, y):
                ints.append((x, y))
            if len(ints) < 8 and y > eps and f(y0 - eps) <= -y <= f(y1 + eps) and not dup(x, -y):
                ints.append((x, -y))
    for y in (y0, y1):                   # crossings of the horizontal edges
        val = f(f(r - y) * f(r + y))
        if val >= -eps:
            x = f(math.sqrt(max(val, f(0))))
            if f(x0 - eps) <= x <= f(x1 + eps) and not dup(x, y):
                ints.append((x, y))
            if len(ints) < 8 and x > eps and f(x0 - eps) <= -x <= f(x1 + eps) and not dup(-x, y):
                ints.append((-x, y))
    corners = [(x0, y0), (x1, y0), (x1, y1), (x0, y1)]
    verts = [c for c, k in zip(corners, inside) if k] + ints
    nc = len(verts)
    if nc < 3:
        return f(1 if n_in > 0 else 0), px, py
    idx = list(range(nc))
    ang = [f(math.atan2(f(v[1] - py), f(v[0] - px))) for v in verts]
    for i in range(nc - 1):              # the reference's exchange sort by angle
        for j in range(i + 1, nc):
            if ang[idx[i]] > ang[idx[j]]:
                idx[i], idx[j] = idx[j], idx[i]
    A = Mx = My = f(0)
    for i in range(nc):
        p1, p2 = verts[idx[i]], verts[idx[(i + 1) % nc]]
        cross = float(p1[0]) * float(p2[1]) - float(p2[0]) * float(p1[1])
        A = f(float(A) + cross)
        Mx = f(float(Mx) + float(f(p1[0] + p2[0])) * cross)
        My = f(float(My) + float(f(p1[1] + p2[1])) * cross)
    A, Mx, My = f(A * f(0.5)), f(Mx / f(6)), f(My / f(6))
    if A < 0:
        A, Mx, My = -A, -Mx, -My
    if len(ints) == 2:                   # the circular segment beyond the chord
        mx, my = f(f(ints[0][0] + ints[1][0]) * f(0.5)), f(f(ints[0][1] + ints[1][1]) * f(0.5))
        dxc, dyc = f(ints[0][0] - ints[1][0]), f(ints[0][1] - ints[1][1])
        L = f(math.sqrt(f(f(dxc * dxc) + f(dyc * dyc))))
        h = f(math.sqrt(f(f(mx * mx) + f(my * my))))
        th = f(f(2) * f(math.atan2(f(f(0.5) * L), h)))
        if th < f(1e-4):
            t2 = f(th * th)
            t3 = f(t2 * th)
            t5 = f(t3 * t2)
            tms = f(f(t3 / f(6)) - f(t5 / f(120)))
            sh = f(f(0.5) * th)
            shc = f(f(sh * sh) * sh)
        else:
            tms = f(th - f(math.sin(th)))
            shc = f(f(math.sin(f(f(0.5) * th))) ** 3)
        As = f(f(f(0.5) * r2) * tms)
        ds = f(f(f(f(4) * r) * shc) / f(f(3) * tms)) if tms > f(1e-10) else r
        nrm = h if h > f(1e-9) else f(1)
        ux, uy = f(mx / nrm), f(my / nrm)
        A, Mx, My = f(A + As), f(Mx + f(f(As * ds) * ux)), f(My + f(f(As * ds) * uy))
    if A > f(1e-9):
        return A, f(Mx / A), f(My / A)
    return A, px, py


def zernike_table(pd):
    """Per pixel of the pd x pd crop (x the fast index, y the slow one): the
    covered fraction of the pixel in the disk of radius pd/2 about ((pd-1)/2,
    (pd-1)/2), the centroid's radius over pd/2 (clamped to 1) and its angle
    atan2(dy, dx) (beamDecomposition.cu:356-368, 521-530)."""
    c = F32((pd - 1) / 2)
    rad = F32(pd / 2)
    frac = np.zeros((pd, pd), F32)
    rho = np.ones((pd, pd), F32)
    th = np.zeros((pd, pd), F32)
    for y in range(pd):
        for x in range(pd):
            a, cx, cy = pixel_coverage(F32(x - c), F32(y - c), rad)
            frac[y, x] = a
            if a > F32(2e-20):
                rho[y, x] = min(F32(F32(math.sqrt(F32(F32(cx * cx) + F32(cy * cy)))) / rad), F32(1))
                th[y, x] = F32(math.atan2(cy, cx))
    return frac, rho, th


def zernike_modes(rho, th, weight):
    """The real Zernike basis in the reference's mode order (m = 0 .. maxN, n = m,
    m+2, .. maxN; cos then sin for m > 0): the radial polynomials by the
    three-term recurrence from weight * rho^m, normalised by sqrt(n+1) (m = 0)
    or sqrt(2(n+1)).  Returns an array [nmodes, ...] (float64)."""
    rho = rho.astype(np.float64)
    out = []
    rp = weight.astype(np.float64)
    for m in range(ZERNIKE_MAX_N + 1):
        cm, sm = np.cos(m * th.astype(np.float64)), np.sin(m * th.astype(np.float64))
        r2 = r4 = None
        for n in range(m, ZERNIKE_MAX_N + 1, 2):
            if n == m:
                cur = rp
            elif n == m + 2:
                cur = r2 * ((m + 2) * rho * rho - (m + 1))
            else:
                k1 = 0.5 * (n + m) * (n - m) * (n - 2.0)
                k2 = 2.0 * n * (n - 1.0) * (n - 2.0)
                k3 = -m * m * (n - 1.0) - n * (n - 1.0) * (n - 2.0)
                k4 = -0.5 * n * (n + m - 2.0) * (n - m - 2.0)
                cur = ((k2 * rho * rho + k3) * r2 + k4 * r4) / k1
            r4, r2 = r2, cur
            nz = cur * (math.sqrt(n + 1.0) if m == 0 else math.sqrt(2.0 * (n + 1.0)))
            if m == 0:
                out.append(nz)
            else:
                out.append(nz * cm)
                out.append(nz * sm)
        rp = rp * rho
    return np.stack(out)


def zernike_regularize(coef):
    """regularize_zernike_coefficients (beamDecomposition.cu:480-513) as zernike_compute
    launches it, with max_l = the number of modes (861): modes 0..430 get p = 2 * mode,
    m = 0, modes 431..860 m = 1, p = 1 + 2 ((mode - 431) // 2); each coefficient is
    soft-thresholded by 5e-5 p^2 + 5e-8 m^2 (zero below 1e-9 in modulus)."""
    nm = coef.shape[0]
    out = np.zeros(nm, C64)
    half = nm >> 1
    for mode in range(nm):
        if mode <= half:
            p, m = 2 * mode, 0
        elif nm % 2 == 1 and mode < (nm + 1) * 3 // 2:
            m, p = 1, 1 + (((mode - half - 1) >> 1) << 1)
        else:
            raise ValueError("mode outside the two branches the launch reaches")
        factor = F32(F32(F32(ZERNIKE_REG_L * F32(p)) * F32(p)) + F32(F32(ZERNIKE_REG_M * F32(m)) * F32(m)))
        c = np.complex64(coef[mode])
        mag = F32(abs(c))
        sc = max(F32(0), F32(F32(1) - F32(factor / mag))) if mag > F32(1e-9) else F32(0)
        out[mode] = np.complex64(complex(F32(c.real * sc), F32(c.imag * sc)))
    return out


def zernike_fit(crop):
    """zernike_compute + zernike_reconstruct of util/ptycho.cpp:619-622 on the pd x pd
    crop: coefficients = sum over pixels of crop * coverage * Z_k (at the coverage
    centroid) / (pi (pd/2)^2), regularised, and the crop replaced by sum_k c_k Z_k
    on the pixels the disk touches (zero elsewhere; beamDecomposition.cu:339-608)."""
    pd = crop.shape[0]
    frac, rho, th = zernike_table(pd)
    live = frac > F32(2e-20)
    Z = zernike_modes(np.where(live, rho, 1), th, np.where(live, frac, 0))
    rad = np.float64(F32(pd / 2))
    coef = (Z.reshape(Z.shape[0], -1) @ crop.astype(np.complex128).reshape(-1)) / (math.pi * rad * rad)
    coef = zernike_regularize(coef.astype(C64))
    th0 = np.where(rho > F32(2e-20), th, F32(0))
    B = zernike_modes(rho, th0, np.ones_like(rho))
    rec = np.tensordot(coef.astype(np.complex128), B, axes=1)
    return np.where(frac >= F32(2e-20), rec, 0).astype(C64)


# ------------------------------------------------- ptycho::iterate and set-up
@dataclass
class PtyParams:
    """The config fields ``ptycho::iterate`` reads (include/readConfig.hpp:25-35; REALVAR are double)."""
    lam: float = 0.5
    d: float = 2e4
    dpupil: float = 1e3
    pixelsize: float = 20.0
    pupil_size: float = 32.0
    exposure: float = 1.0
    mpie: bool = True
    use_bs: bool = False
    beam_stop_size: int = 5
    noise_level: int = 0
    position_uncertainty: float = 0.0
    zernike_iter: int = 0
    is_fresnel: bool = False

    def resolution(self, rows):
        """resolution = lambda d / pixelsize / row (util/ptycho.cpp:246), stored as float."""
        return F32(self.lam * self.d / self.pixelsize / rows)


def simulate_patterns(obj, probe, scanx, scany, exposure=1.0, fresnel=0.0, bs=None):
    """The noise-free part of ptycho::createPattern (util/ptycho.cpp:310-359):
    I_i = |FFT(P O_window)|^2 / (rows cols), times exposure then times float(1/exposure);
    with isFresnel (fresnel = the factor) the exit wave takes the Fresnel phase first; with a
    beamstop (useBS) applySupport zeroes the stopped pixels."""
    rows, cols = probe.shape
    out = []
    for px, py in zip(scanx, scany):
        w = get_window(obj, c_round(px), c_round(py), rows, cols)
        esw = (probe * w).astype(C64)
        if fresnel:
            esw = fresnel_phase(esw, fresnel)
        F = fft2_u(esw)
        I = ((F.real * F.real + F.imag * F.imag).astype(F32) * F32(1.0 / (rows * cols))).astype(F32)
        if bs is not None:
            I = np.where(bs > F32(0), F32(0), I).astype(F32)
        I = (I * F32(exposure)).astype(F32)
        I = (I * F32(1.0 / exposure)).astype(F32)
        out.append(I)
    return np.stack(out)


def iterate(obj0, probe0, patterns, scanx, scany, n_iter, params: PtyParams, orders, start_iter=0):
    """ptycho::iterate (util/ptycho.cpp:429-736): per scan
    position (in the given order) the window times the probe, FFT, applyModAccurate,
    inverse FFT, the difference of exit waves and the rPIE object update
    (updateObject; from iteration 400 updateObjectAndProbeStep with the probe
    step accumulated and added after the sweep, the object clamped and the
    object/probe scales balanced first); from iteration 400 the pupil
    constraint after the sweep (back-propagate, disk of pupilSize, propagate,
    recentre the far field); mPIE momentum (FISTA-type, with the global phase
    of the covered object removed) when enabled.  After the last iteration the
    probe is back-propagated to the pupil plane and the object's global phase
    removed, as the reference leaves them.  Returns (object, pupil)."""
    rows, cols = probe0.shape
    orow, ocol = obj0.shape
    O = obj0.astype(C64).copy()
    Oprev = np.zeros_like(O)
    P = probe0.astype(C64).copy()
    Pprev = np.zeros_like(P)
    step = np.zeros_like(P)
    nscan = len(scanx)
    norm = F32(1.0 / math.sqrt(rows * cols))
    scale = F32(1.0 / params.exposure)
    probe_step_size = F32(1.0 / nscan)
    pd = int(params.pupil_size)
    res = params.resolution(rows)
    pupil_support = circle_mask(pd, pd, F32((pd + 1) / 2.0), F32((pd + 1) / 2.0), F32(pd / 2.0))
    msum = masksum(rows, cols, orow, ocol, scanx, scany, params.pupil_size)
    bs = circle_mask(rows, cols, rows >> 1, cols >> 1, params.beam_stop_size, True) if params.use_bs else None
    tk = F32(0.5 + math.sqrt(1.25))
    shifts = np.zeros((2, len(scanx)), F32)    # d_shifts (util/ptycho.cpp:110-113), zero at the start
    fres = fresnel_factor(params.lam, params.d, params.pixelsize, rows) if params.is_fresnel else None
    for it in range(start_iter, start_iter + n_iter):
        probe_max = F32(np.max((P.real * P.real + P.imag * P.imag).astype(F32)))
        obj_max = F32(0)
        if it >= UPDATE_PROBE_ITER:
            m2 = ((O.real * O.real + O.imag * O.imag).astype(F32) * msum).astype(F32)
            obj_max = F32(np.max(m2))
            thr = F32(math.sqrt(obj_max))
            om2 = (O.real * O.real + O.imag * O.imag).astype(F32)
            big = om2 > thr
            with np.errstate(divide="ignore", invalid="ignore"):
                f = np.sqrt((thr / np.where(big, om2, F32(1))).astype(F32)).astype(F32)
            O = np.where(big, ((f * O.real).astype(F32) + 1j * (f * O.imag).astype(F32)), O).astype(C64)
            sf = F32((np.float64(F32(probe_max / obj_max))) ** 0.25)
            O = (O * sf).astype(C64)
            Oprev = (Oprev * sf).astype(C64)
            P = (P * F32(1.0 / np.float64(sf))).astype(C64)
            Pprev = (Pprev * F32(1.0 / np.float64(sf))).astype(C64)     # util/ptycho.cpp:507
            obj_max = probe_max = F32(math.sqrt(np.float64(F32(obj_max * probe_max))))
        update_pos = it % 20 == 0 and it >= POSITION_UPDATE_ITER      # util/ptycho.cpp:511
        grad = np.zeros((2, nscan), F32)
        for i in orders[it - start_iter]:
            sx = c_round(F32(F32(scanx[i]) + shifts[0, i]))
            sy = c_round(F32(F32(scany[i]) + shifts[1, i]))
            w = get_window(O, sx, sy, rows, cols)
            esw = (P * w).astype(C64)
            if fres is not None:                  # util/ptycho.cpp:526-528
                esw = fresnel_phase(esw, fres)
            F = fft2_u(esw)
            pnorm = norm
            if update_pos:                        # util/ptycho.cpp:533-538: Fn * norm first
                F = (F * norm).astype(C64)
                pnorm = F32(1)
                grad[0, i], grad[1, i] = position_gradient(w, P, F, patterns[i], bs)
            if it < NOISE_PROJ_ITER:
                F = apply_mod_accurate(F, patterns[i], pnorm, scale, bs)
            else:
                F = apply_mod_noise(F, patterns[i], pnorm, scale, params.noise_level, bs)
            F = (ifft2_u(F) * norm).astype(C64)
            diff = (esw - F).astype(C64)
            if fres is not None:                  # removeFresnelPhase (util/ptycho.cpp:551)
                diff = fresnel_phase(diff, -fres)
            if it < UPDATE_PROBE_ITER:
                w = rpie(w, P, diff, probe_max, ALPHA, 1.0)
            else:
                w = rpie(w, P, diff, probe_max, ALPHA, 0.5)
                step = (step + (rpie_step(w, diff, obj_max, BETA) * probe_step_size)).astype(C64)
            update_window(O, sx, sy, w)
        if it >= UPDATE_PROBE_ITER:
            P = (P + step).astype(C64)
            step = (step * F32(0)).astype(C64)
        if update_pos:                            # util/ptycho.cpp:567-585
            with np.errstate(divide="ignore", over="ignore", invalid="ignore"):
                shifts = add_probability(shifts, grad, F32(params.position_uncertainty))
            mx = F32(F32(shifts[0].astype(np.float64).sum()) / F32(nscan))
            my = F32(F32(shifts[1].astype(np.float64).sum()) / F32(nscan))
            shifts[0] = (shifts[0] - mx).astype(F32)
            shifts[1] = (shifts[1] - my).astype(F32)
            O = shift_wave(O, -mx, -my)
            Oprev = shift_wave(Oprev, -mx, -my)
        if it >= UPDATE_PROBE_ITER:
            P = angular_spectrum(P, params.lam, params.dpupil, res, reverse=True)
            r0, c0 = (rows - pd) // 2, (cols - pd) // 2
            if it < params.zernike_iter and it % 10 == 0:    # dozernike (util/ptycho.cpp:619-621)
                crop = zernike_fit(P[r0:r0 + pd, c0:c0 + pd])
            else:
                crop = P[r0:r0 + pd, c0:c0 + pd] * (pupil_support > F32(0.5))
            P = np.zeros_like(P)
            P[r0:r0 + pd, c0:c0 + pd] = crop
            P = angular_spectrum(P, params.lam, params.dpupil, res, reverse=False)
            far = convert_fo(fft2_u(P))
            mx, my = find_middle((far.real * far.real + far.imag * far.imag).astype(F32))
            P = multiply_shift(P, F32(np.float64(F32(mx * F32(rows))) - 0.5), F32(np.float64(F32(my * F32(cols))) - 0.5))
        if it < params.zernike_iter:          # util/ptycho.cpp:665-667
            O = fista_step(O, 0.01)
        if params.mpie:
            s = (O * msum).astype(C64).astype(np.complex128).sum()
            s = complex(np.complex64(s))
            s = np.complex64(s / abs(s))
            O = (O * np.conj(s)).astype(C64)
            Oprev = (Oprev * np.conj(s)).astype(C64)
            Oprev = (O - Oprev).astype(C64)
            tkp1 = F32(0.5 + math.sqrt(0.25 + np.float64(F32(tk * tk))))
            c = F32(F32(tk - F32(1)) / tkp1)
            Oprev = (O + (Oprev * c).astype(C64)).astype(C64)
            O, Oprev = Oprev, O
            if it < params.zernike_iter and it % 10 == 0:   # dozernike: probe momentum too (682-686)
                Pprev = (P - Pprev).astype(C64)
                cz = F32(np.float64(c) * 0.8)
                Pprev = (P + (Pprev * cz).astype(C64)).astype(C64)
                P, Pprev = Pprev, P
            tk = tkp1
    pupil = angular_spectrum(P, params.lam, params.dpupil, res, reverse=True)
    s = complex(np.complex64(O.astype(np.complex128).sum()))
    s = np.complex64(s / F32(math.hypot(s.real, s.imag)))
    O = (O * np.conj(s)).astype(C64)
    return O, pupil, P


def rel_err(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))
