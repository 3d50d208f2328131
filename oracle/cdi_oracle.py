"""CPU oracle for the CDI phase-retrieval hot path.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import this
module.  It is the checker, never the product: the product path lives in
``cdixx_gb300`` and fails loudly when its CUDA library is missing.

This is a NumPy restatement of the reference's algorithm (liboyang0112/CDIxx),
each function citing the reference file:line it follows.  It runs in float64
(the error oracle) or in float32/complex64 with the reference's scalar types
(float parameters, double literals 1.9 / 1.2, float normalisation factors).

The reference's FFT is cuFFT (CUDA 13.0 toolkit, libcufft 12.0) and its
reductions are CUB (CCCL in CUDA 13.0); neither is part of the reference
sources.  cuFFT is restated as the published unnormalised 2-D DFT
(forward exp(-2 pi i), inverse exp(+2 pi i)) via ``numpy.fft``; CUB's
``DeviceReduce`` max/sum as plain reductions (float64 accumulation).
"""
from __future__ import annotations

import math
import struct
from dataclasses import dataclass, field

import numpy as np

# ---------------------------------------------------------------------------
# Algorithm enum -- include/format.hpp:22
RAAR, ER, POSER, HIO, POSHIO, FHIO, SHRINKWRAP, XCORRELATION, KKT, TV, CNT = range(11)
ALGO_NAMES = {
    "RAAR": RAAR, "HIO": HIO, "ER": ER, "POSER": POSER, "POSHIO": POSHIO,
    "FHIO": FHIO, "KKT": KKT, "shrinkWrap": SHRINKWRAP, "TV": TV,
    "XCORRELATION": XCORRELATION,
}


class AlgoParseError(ValueError):
    """The reference prints "Algorithm <x> not found" and calls exit(0)
    (src/independant/readConfig.cc:132-135)."""


def _atoi(s: str) -> int:
    # C atoi: optional leading blanks, optional sign, digits; stops at the
    # first non-digit, 0 when there are none.
    s = s.lstrip(" \t\n\r\f\v")
    m = 0
    sign = 1
    i = 0
    if i < len(s) and s[i] in "+-":
        sign = -1 if s[i] == "-" else 1
        i += 1
    while i < len(s) and s[i].isdigit():
        m = m * 10 + (ord(s[i]) - 48)
        i += 1
    return sign * m


class _Strtok:
    """strtok_r over one buffer (skips leading delimiters, cuts at the next)."""

    def __init__(self, s: str):
        self.s = s
        self.p = 0

    def next(self, delims: str):
        s, p = self.s, self.p
        while p < len(s) and s[p] in delims:
            p += 1
        if p >= len(s):
            self.p = p
            return None
        q = p
        while q < len(s) and s[q] not in delims:
            q += 1
        self.p = q + 1 if q < len(s) else q
        return s[p:q]


class AlgoParser:
    """Restatement of ``AlgoParser`` (src/independant/readConfig.cc:82-163).

    Grammar: ``n*ALGO+m*ALGO+k*(...)``.  The reference finds the first '(' and
    the first ')' (readConfig.cc:97-99) and cuts the sub-expression between
    them.  Its nested-parenthesis search (readConfig.cc:101-106) passes
    ``std::string::find`` a needle of (positione-position+1) characters that
    starts with "(" and NUL, which never occurs in the formula, so nested
    parentheses are cut at the FIRST ')' and the parse then fails with an
    unknown token such as "shrinkWrap)".  This restatement reproduces exactly
    that behaviour (raising :class:`AlgoParseError` where the reference exits).
    """

    def __init__(self, f: str):
        self.n_algo = CNT
        self.sub: list[AlgoParser] = []
        self.count: list[int] = []
        self.algo: list[int] = []
        formula = "".join(ch for ch in f if ch != " ")        # 89-95
        position = formula.find("(")                           # 97
        while position != -1:
            positione = formula.find(")")                      # 99
            if positione == -1:
                sub = formula[position + 1:]
                formula = formula[:position] + "subParser"
            else:
                sub = formula[position + 1:positione]          # 107
                formula = formula[:position] + "subParser" + formula[positione + 1:]  # 108
            self.sub.append(AlgoParser(sub))
            position = formula.find("(")                       # 110
        tok = _Strtok(formula)                                 # 112-136
        i_parser = 0
        ptr = tok.next("*")
        if ptr is None:
            raise AlgoParseError("empty algorithm string")
        while True:
            num = _atoi(ptr)
            name = tok.next("+")
            if name is None:
                raise AlgoParseError(f"Algorithm after count {ptr!r} missing")
            self.count.append(num)
            if name in ALGO_NAMES:
                self.algo.append(ALGO_NAMES[name])
            elif name == "subParser":
                self.algo.append(self.n_algo + i_parser)
                i_parser += 1
            else:
                raise AlgoParseError(f"Algorithm {name} not found")
            ptr = tok.next("*")
            if ptr is None:
                break
        self.restart()

    def restart(self):                                         # 139-145
        self.cur_algo = 0
        self.cur_count = self.count[0]
        for s in self.sub:
            s.restart()

    def next(self) -> int:                                     # 146-163
        if self.cur_count == 0:
            if self.cur_algo == len(self.algo) - 1:
                return -1
            self.cur_algo += 1
            self.cur_count = self.count[self.cur_algo]
        a = self.algo[self.cur_algo]
        if a >= self.n_algo:
            sp = self.sub[a - self.n_algo]
            ret = sp.next()
            if ret == -1:
                self.cur_count -= 1
                sp.restart()
                return self.next()
            return ret
        self.cur_count -= 1
        return a

    def expand(self, limit: int = 10_000_000) -> list[int]:
        out = []
        while True:
            a = self.next()
            if a < 0:
                return out
            out.append(a)
            if len(out) > limit:
                raise AlgoParseError("algorithm expands beyond the step limit")


# ---------------------------------------------------------------------------
# FFT restatement (cuFFT C2C, src/gpu/cudaConfig.cu:137-180)

_FFT_WORKERS = 1


def set_fft_workers(n: int):
    """Threads for the CPU FFT (scipy.fft ``workers``; 1 = NumPy's pocketfft)."""
    global _FFT_WORKERS
    _FFT_WORKERS = max(1, int(n))


def fft2_u(a):
    """Unnormalised forward 2-D DFT, exp(-2 pi i k n / N) (CUFFT_FORWARD)."""
    if _FFT_WORKERS > 1:
        import scipy.fft
        return scipy.fft.fft2(a, workers=_FFT_WORKERS)
    return np.fft.fft2(a)


def ifft2_u(a):
    """Unnormalised inverse 2-D DFT, exp(+2 pi i k n / N) (CUFFT_INVERSE)."""
    n = a.shape[-1] * a.shape[-2]
    if _FFT_WORKERS > 1:
        import scipy.fft
        return scipy.fft.ifft2(a, norm="forward", workers=_FFT_WORKERS).astype(a.dtype, copy=False)
    out = np.fft.ifft2(a)
    return (out * n).astype(a.dtype, copy=False)


# ---------------------------------------------------------------------------
# Element-wise kernels

def _real(dt):
    return np.float32 if dt == np.complex64 else np.float64


def apply_mod_abs(psi, pattern):
    """applyModAbs with state == NULL (src/gpu/cudaConfig.cu:827-841).

    psi <- sqrt(I) * psi / |psi|;  I <= 0 (or NaN) -> 0;  |psi| == 0 -> sqrt(I) + 0i.
    """
    rt = _real(psi.dtype)
    mod = np.hypot(psi.real, psi.imag).astype(rt)
    rat = np.where(pattern > 0, np.sqrt(np.where(pattern > 0, pattern, 0)), 0).astype(rt)
    zero = mod == 0
    with np.errstate(divide="ignore", invalid="ignore"):
        r2 = np.where(zero, 0, rat / np.where(zero, 1, mod)).astype(rt)
    out = np.empty_like(psi)
    out.real = np.where(zero, rat, psi.real * r2)
    out.imag = np.where(zero, 0, psi.imag * r2)
    return out


def apply_mod(psi, pattern, beamstop=None, noise_level=0, scale=1.0, rcolor=65535):
    """Noise-tolerant modulus projection, 5-argument ``applyMod`` with
    bsnorm == 1 (src/gpu/cdi.cu:438-485).  ``scale`` is ``vars.scale``
    (1/exposure, cdi.cu:16-30) and ``rcolor`` is ``vars.rcolor``."""
    rt = _real(psi.dtype)
    scale = rt(scale)
    mod2 = np.maximum(rt(0), pattern.astype(rt))
    rx, ry = psi.real.astype(rt), psi.imag.astype(rt)
    src = (rx * rx + ry * ry).astype(rt)
    maximum = scale * rt(0.95)
    mod2 = np.where(mod2 >= maximum, np.maximum(mod2, src), mod2).astype(rt)
    tol = (np.sqrt(rt(noise_level) + mod2 * rt(rcolor) / scale) * scale / rt(rcolor)).astype(rt)
    diff = mod2 - src
    val = np.where(diff > tol, mod2 - tol, np.where(diff < -tol, mod2 + tol, mod2)).astype(rt)
    zero = src == 0
    with np.errstate(divide="ignore", invalid="ignore"):
        s = np.sqrt(np.maximum(val, rt(0)) / np.where(zero, 1, src)).astype(rt)
    out = np.empty_like(psi)
    out.real = np.where(zero, val, s * rx)
    out.imag = np.where(zero, 0, s * ry)
    if beamstop is not None:
        blocked = beamstop > 0.5
        out = np.where(blocked, psi, out)
    return out


def apply_support(rho, rhop, spt, threshold, algo, beta=1.0):
    """Real-space updates, dispatched as ``applySupport`` (src/post_gpu/cdi.cc:25-36):
    RAAR cdi.cu:550-568, ER 585-600, POSER 569-584, POSHIO 601-616, HIO 518-533,
    anything else (FHIO, KKT, XCORRELATION) -> FHIO 534-549.

    ``inside = spt > threshold`` (e.g. cdi.cu:525).  The literals 1.9 and 1.2
    are double in the reference, so those products are formed in double and
    rounded once on store; ``beta`` is ``vars.beta_HIO`` (float).
    """
    rt = _real(rho.dtype)
    b = rt(beta)
    inside = spt > rt(threshold)
    xr, xi = rho.real, rho.imag
    pr, pi = rhop.real, rhop.imag

    def relax(x, p):  # x + 1.9*(p - x) in double, stored in the working type
        return (x.astype(np.float64) + 1.9 * (p - x).astype(np.float64)).astype(rt)

    if algo == HIO:
        nr = np.where(inside, pr, xr - b * pr)
        ni = np.where(inside, pi, xi - b * pi)
    elif algo == RAAR:
        c = rt(1) - rt(2) * b
        nr = np.where(inside, pr, b * xr + c * pr)
        ni = np.where(inside, pi, b * xi + c * pi)
    elif algo == ER:
        nr = np.where(inside, relax(xr, pr), 0)
        ni = np.where(inside, relax(xi, pi), 0)
    elif algo == POSER:
        ok = inside & (pr > 0)
        nr = np.where(ok, pr, 0)
        ni = np.where(ok, pi, 0)
    elif algo == POSHIO:
        ok = inside & (pr > 0)
        nr = np.where(ok, relax(xr, pr), xr - b * pr)
        ni = xi - b * pi
    else:  # FHIO and the default branch
        nr = np.where(inside, relax(xr, pr),
                      (xr.astype(np.float64) - 1.2 * pr.astype(np.float64)).astype(rt))
        ni = np.where(inside, relax(xi, pi),
                      (xi.astype(np.float64) - 1.2 * pi.astype(np.float64)).astype(rt))
    out = np.empty_like(rho)
    out.real = nr
    out.imag = ni
    return out


def rect_support(rows, cols, oversampling_spt, dtype=np.float32):
    """``createSupport`` rect (src/post_gpu/cdi.cc:240-251) filled by
    ``createMask<rect>`` (src/gpu/cudaConfig.cu:1291-1300; rect::isInside 89-92)."""
    sx = int((oversampling_spt - 1) / 2 * rows / oversampling_spt - 1)
    sy = int((oversampling_spt - 1) / 2 * cols / oversampling_spt - 1)
    ex, ey = rows - sx, cols - sy
    x = np.arange(rows)[:, None]
    y = np.arange(cols)[None, :]
    m = (x >= sx) & (x < ex) & (y >= sy) & (y < ey)
    return m.astype(dtype)


def gauss_mult_freq(psi, sigma):
    """``applyGaussMult(.., isFreq=1)`` (src/gpu/cudaConfig.cu:380-395):
    psi * exp(-(xr^2+yr^2)/(2 sigma^2)) with FFT-order coordinates."""
    rows, cols = psi.shape[-2:]
    rt = _real(psi.dtype)
    x = np.arange(rows)
    y = np.arange(cols)
    xr = np.where(x >= rows // 2, x - rows, x).astype(rt)[:, None]
    yr = np.where(y >= cols // 2, y - cols, y).astype(rt)[None, :]
    s = rt(sigma)
    f = np.exp(-(xr * xr + yr * yr) / (rt(2) * s * s)).astype(rt)
    return (psi * f).astype(psi.dtype)


def shrink_kernel_1d(n, sigma_f):
    """Spatial kernel equal to the inverse DFT of the sampled frequency
    Gaussian used by the shrinkwrap (cudaConfig.cu:380-395): periodic, length
    n, k[m] = (1/n) sum_f exp(-f^2/(2 sigma_f^2)) exp(+2 pi i f m / n), f in
    FFT order.  Returned in float64 (real part; the imaginary part is at most
    exp(-(n/2)^2/(2 sigma_f^2))/n)."""
    f = np.arange(n)
    f = np.where(f >= n // 2, f - n, f).astype(np.float64)
    g = np.exp(-(f * f) / (2.0 * sigma_f * sigma_f))
    return np.fft.ifft(g).real


# ---------------------------------------------------------------------------
# The iteration

@dataclass
class CDIState:
    psi: np.ndarray          # patternWave, FFT order
    rho: np.ndarray          # objectWave
    support: np.ndarray      # float support (raw blurred |.|^2 after a shrinkwrap)
    threshold: float = 0.5   # vars.threshold (cdi.cu:21)
    avg: float = 0.0
    gauss_sigma: float = 3.0
    iter: int = 0
    residual: float = 0.0
    history: list = field(default_factory=list)
    prtf: np.ndarray = None  # prtf.txt column when the run reached prtf_iter


def prtf_polar(img):
    """``cart2polar_kernel`` + ``edgeReduce`` (src/gpu/cudaConfig.cu:1027-1063) on
    the centred image (``cudaConvertFO`` of an FFT-order field): for radius r <
    rows/2 the float32 sum over 2*cols angles, in angle order, of the bilinear
    sample at (r cos t, r sin t) about (rows/2, cols/2)."""
    img = np.fft.fftshift(np.asarray(img, np.float32))
    rows, cols = img.shape
    nang = 2 * cols
    out = np.zeros(rows // 2, np.float32)
    a = np.arange(nang)
    ang = (a * (2.0 * np.pi / nang)).astype(np.float32)   # x * (2.0f*M_PI/cuda_row), double then float
    c, s = np.cos(ang).astype(np.float32), np.sin(ang).astype(np.float32)
    for r in range(rows // 2):
        x = np.float32(r) * c + np.float32(rows >> 1)
        y = np.float32(r) * s + np.float32(cols >> 1)
        x0, y0 = np.floor(x).astype(int), np.floor(y).astype(int)
        fx, fy = (x - x0).astype(np.float32), (y - y0).astype(np.float32)
        ok = (x0 >= 0) & (x0 + 1 < rows) & (y0 >= 0) & (y0 + 1 < cols)
        xa, ya = np.where(ok, x0, 0), np.where(ok, y0, 0)
        v = ((1 - fx) * (1 - fy) * img[xa, ya] + (1 - fx) * fy * img[xa, ya + ok] +
             fx * (1 - fy) * img[xa + ok, ya] + fx * fy * img[xa + ok, ya + ok])
        v = np.where(ok, v, np.float32(0)).astype(np.float32)
        acc = np.float32(0)
        for t in v:   # edgeReduce adds the angles one by one in float
            acc = np.float32(acc + t)
        out[r] = acc
    return out


def prepare_from_restart(psi0, dtype=np.complex128):
    """``prepareIter`` with restart (src/post_gpu/cdi.cc:201-227): rho0 =
    IFFT(psi0)/sqrt(N), followed by the extra 1/sqrt(N) of
    ``phaseRetrieve`` (cdi.cc:313)."""
    psi = np.asarray(psi0).astype(dtype)
    rows, cols = psi.shape
    rt = _real(psi.dtype)
    f = rt(1.0 / math.sqrt(rows * cols))
    rho = (ifft2_u(psi) * f).astype(dtype)
    rho = (rho * f).astype(dtype)
    return psi, rho


def shrinkwrap_step(st: CDIState, shrink_threshold: float):
    """Shrinkwrap block of ``phaseRetrieve`` (src/post_gpu/cdi.cc:326-341)."""
    rows, cols = st.psi.shape
    rt = _real(st.psi.dtype)
    sigma_f = rt(rows >> 2) / rt(st.gauss_sigma)
    tmp = gauss_mult_freq(st.psi, sigma_f)
    tmp = ifft2_u(tmp)
    spt = (tmp.real.astype(rt) ** 2 + tmp.imag.astype(rt) ** 2).astype(rt)   # getMod2 773-777
    st.support = spt
    maxs = rt(max(0.0, float(np.max(spt.astype(np.float64)))))               # findMax, init 0
    if st.avg == 0:
        s = rt(np.sum(spt.astype(np.float64)))
        st.avg = float(rt(rt(rt(s * rt(4)) / rt(rows)) / rt(cols)))
    if rt(st.avg) * rt(5) < maxs:
        maxs = rt(st.avg) * rt(5)
    st.threshold = float(rt(float(maxs) * shrink_threshold))                  # setThreshold
    if st.gauss_sigma > 2:
        st.gauss_sigma = float(rt(st.gauss_sigma * 0.99))


def phase_retrieve(psi0, pattern, algorithm, *, support=None, oversampling_spt=2.0,
                   beta=1.0, shrink_threshold=0.1, sim_ccd_bit=False, noise_level=0,
                   exposure=1.0, rcolor=65535, beamstop=None, dtype=np.complex128,
                   record=None, max_steps=None, step_noise=None, prtf_iter=-1):
    """``CDI::phaseRetrieve`` from a restart iterate (src/post_gpu/cdi.cc:297-449,
    with prepareIter cdi.cc:201-227 and initSupport 252-254).

    ``record``: optional set of step indices after which (rho, psi, support,
    threshold) are appended to ``state.history``.  The PRTF block is off
    (prtfIter beyond the run), as are plotting and video.  Returns the state;
    ``state.rho`` is scaled back by sqrt(N) (cdi.cc:406) and ``state.residual``
    is the reference's residual (cdi.cc:413-421).

    ``step_noise=(eps, seed)`` (tests only, no reference counterpart) adds
    complex Gaussian noise of relative size eps * RMS(rho) to rho after every
    projection step: a model of the per-step rounding of a float32 FFT (whose
    errors are about uniform in absolute size across pixels), used to bound how
    far two float32 implementations can drift apart along a trajectory.
    """
    noise_rng = np.random.default_rng(step_noise[1]) if step_noise else None
    rt = np.float32 if dtype == np.complex64 else np.float64
    psi, rho = prepare_from_restart(psi0, dtype)
    rows, cols = psi.shape
    pattern = np.asarray(pattern).astype(rt)
    spt = (rect_support(rows, cols, oversampling_spt, rt) if support is None
           else np.asarray(support).astype(rt))
    st = CDIState(psi=psi, rho=rho, support=spt)
    steps = AlgoParser(algorithm).expand()
    if max_steps is not None:
        steps = steps[:max_steps]
    inv_n = rt(1.0 / (rows * cols))
    prtf_map = cache = gamma0 = weights = None
    phi0 = 0.0
    for k, a in enumerate(steps):
        if a == SHRINKWRAP:
            shrinkwrap_step(st, shrink_threshold)
        elif a == TV:
            raise NotImplementedError("TV (FISTA) step is outside the phase-retrieval path")
        else:
            if sim_ccd_bit:
                st.psi = apply_mod(st.psi, pattern, beamstop, noise_level, 1.0 / exposure, rcolor)
            else:
                st.psi = apply_mod_abs(st.psi, pattern)
            rhop = (ifft2_u(st.psi) * inv_n).astype(dtype)
            st.rho = apply_support(st.rho, rhop, st.support, st.threshold, a, beta)
            if prtf_iter >= 0 and k >= prtf_iter:
                # PRTF block of phaseRetrieve (cdi.cc:355-380); cache and gamma0 start at 0
                if prtf_map is None:
                    prtf_map = np.zeros_like(st.psi)
                    cache = np.zeros_like(st.psi)
                    gamma0 = np.zeros_like(st.psi)
                mod = np.abs(st.psi)
                if k == prtf_iter:
                    gamma0 = apply_support(np.zeros_like(rhop), rhop, st.support, st.threshold, ER)
                    cache = gamma0 * gamma0
                    sm = cache.sum()
                    phi0 = float(np.float32(-np.arctan2(np.float32(sm.imag), np.float32(sm.real)) / 2))
                    theta = phi0
                    weights = prtf_polar((mod > 1e-6).astype(np.float32))
                else:
                    cache = apply_support(cache, rhop, st.support, st.threshold, ER) * np.conj(gamma0)
                    sm = cache.sum()
                    theta = float(np.float32(phi0 + np.arctan2(np.float32(sm.imag), np.float32(sm.real))))
                ph = np.where(mod > 1e-6, st.psi / np.where(mod > 1e-6, mod, 1), 0)
                prtf_map = prtf_map + ph * np.exp(1j * theta)
            if noise_rng is not None:
                z = noise_rng.standard_normal(st.rho.shape) + 1j * noise_rng.standard_normal(st.rho.shape)
                rms = np.sqrt(np.mean(np.abs(st.rho) ** 2))
                st.rho = (st.rho + step_noise[0] * rms / np.sqrt(2) * z).astype(dtype)
            st.psi = fft2_u(st.rho).astype(dtype)
        st.iter += 1
        if record is not None and k in record:
            st.history.append((st.rho.copy(), st.psi.copy(), st.support.copy(), st.threshold))
    st.rho = (st.rho * rt(math.sqrt(rows * cols))).astype(dtype)
    st.residual = residual(st.psi, pattern)
    if weights is not None:
        # |prtf_map| / (iter - prtfIter), polar sums, prtf[i]/weights[i] (cdi.cc:424-439)
        st.prtf = prtf_polar(np.abs(prtf_map) / (len(steps) - prtf_iter)) / weights
    return st


def residual(psi, pattern):
    """Final residual (src/post_gpu/cdi.cc:413-421; addRemoveOE cudaConfig.cu:907-914):
    sum over pixels of (|psi|^2 - I)^2 with pixels I >= 0.99 zeroed."""
    m2 = psi.real.astype(np.float64) ** 2 + psi.imag.astype(np.float64) ** 2
    p = pattern.astype(np.float64)
    d = np.where(p < 0.99, m2 - p, 0.0)
    return float(np.sum(d * d))


def r_factor(psi, pattern, mask=None):
    """R = sum | |psi| - sqrt(I) | / sum sqrt(I) over measured pixels (float64).
    No reference counterpart (build-only metric)."""
    a = np.abs(psi.astype(np.complex128))
    s = np.sqrt(np.maximum(pattern.astype(np.float64), 0))
    if mask is not None:
        a, s = a[mask], s[mask]
    return float(np.sum(np.abs(a - s)) / max(np.sum(s), 1e-300))


# ---------------------------------------------------------------------------
# .bin image format (src/independant/imgio.c:23-43, 223-243; include/imageFile.hpp)
_HDR = struct.Struct("<b3xiiii")   # char type; int rows, cols, nchann, typesize -> 20 bytes
FLOAT, FLOAT2 = 3, 4


def write_bin(path, arr):
    a = np.ascontiguousarray(arr)
    if np.iscomplexobj(a):
        t, data = FLOAT2, a.astype(np.complex64)
    else:
        t, data = FLOAT, a.astype(np.float32)
    with open(path, "wb") as f:
        f.write(_HDR.pack(t, a.shape[0], a.shape[1], 1, 0))
        f.write(data.tobytes())


def read_bin(path):
    with open(path, "rb") as f:
        hdr = f.read(_HDR.size)
        t, rows, cols, _, _ = _HDR.unpack(hdr)
        if t == FLOAT:
            return np.frombuffer(f.read(rows * cols * 4), np.float32).reshape(rows, cols)
        if t == FLOAT2:
            return np.frombuffer(f.read(rows * cols * 8), np.complex64).reshape(rows, cols)
        raise ValueError(f"FILETYPE unrecognized: {t}")


def find_middle(mask):
    """``findMiddle`` (src/post_gpu/misc.cc:27-42) with ``multiplyx``/``multiplyy``
    (src/gpu/cudaConfig.cu:1427-1437): the centroid of a field in units of its
    size, coordinate (x + 0.5)/rows - 0.5."""
    rows, cols = mask.shape
    m = np.asarray(mask, np.float64)
    s = m.sum()
    cx = ((np.arange(rows) + 0.5) / rows - 0.5)[:, None]
    cy = ((np.arange(cols) + 0.5) / cols - 0.5)[None, :]
    return float(np.float32((m * cx).sum() / s)), float(np.float32((m * cy).sum() / s))


def crop_about(src, out_rows, out_cols, midx, midy):
    """``crop`` (src/gpu/cudaConfig.cu:348-358) of a rows x cols field to
    out_rows x out_cols about (midx, midy), with the reference's clamping (its
    y clamp uses rows)."""
    rows, cols = src.shape
    shiftx = int(rows * np.float32(midx))
    if shiftx + out_rows // 2 > rows // 2:
        shiftx = (rows - out_rows) // 2
    elif shiftx - out_rows // 2 < -(rows // 2):
        shiftx = (out_rows - rows) // 2
    shifty = int(cols * np.float32(midy))
    if shifty + out_cols // 2 > cols // 2:
        shifty = (rows - out_cols) // 2
    elif shifty - out_cols // 2 < -(cols // 2):
        shifty = (out_cols - cols) // 2
    x = np.arange(out_rows)[:, None] + (rows - out_rows) // 2 + shiftx
    y = np.arange(out_cols)[None, :] + (cols - out_cols) // 2 + shifty
    return src.reshape(-1)[(x * cols + y)]


def sim_pattern(intensity, phase, oversampling, phase_modulation, fresnel=0.0):
    """The noise-free runSim pattern: readObjectWave (src/post_gpu/cdi.cc:62-82) places
    sqrt(I) exp(i (phaseModulation * phase - 0.5) 2 pi) at the centre of a field
    `oversampling` times larger (createWaveFront, src/gpu/cudaConfig.cu:688-708);
    prepareIter (cdi.cc:181-200) stores |FFT(object)|^2 / (rows cols) in FFT order; with
    isFresnel (fresnel = propagator's phase factor) the object takes the Fresnel phase
    first (cdi.cc:174, cudaConfig.cu:1095-1101)."""
    r, c = intensity.shape
    rows, cols = int(r * oversampling), int(c * oversampling)
    obj = np.zeros((rows, cols), np.complex128)
    ph = (np.float64(phase_modulation) * phase.astype(np.float64) - 0.5) * 2 * math.pi if phase is not None else 0.0
    x0, y0 = (rows - r) // 2, (cols - c) // 2
    obj[x0:x0 + r, y0:y0 + c] = np.sqrt(np.maximum(intensity.astype(np.float64), 0)) * np.exp(1j * ph)
    if fresnel:
        dx = (np.arange(rows) - (rows >> 1))[:, None]
        dy = (np.arange(cols) - (cols >> 1))[None, :]
        fph = (np.float32(fresnel) * (dx * dx + dy * dy).astype(np.float32)).astype(np.float32).astype(np.float64)
        obj = np.where(obj != 0, obj * np.exp(1j * fph), obj)
    F = np.fft.fft2(obj)
    return (np.abs(F) ** 2 / (rows * cols)).astype(np.float32)
