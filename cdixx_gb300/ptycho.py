"""Ptychographic reconstruction on the GPU: binding of ``include/cdx_ptycho.h``.

``Ptycho`` mirrors the reference's ``ptycho`` driver class (util/ptycho.cpp:41-736):
the same fields (``row``/``column`` probe size, ``row_O``/``column_O`` object size,
``scanposx``/``scanposy``, the optics of readConfig) and steps (``initObject``,
the noise-free ``createPattern``, ``iterate``), with the object, probe and
patterns held on the device by the library.  There is no CPU path: the calls
fail when ``_lib/libcdx.so`` is missing.
"""
from __future__ import annotations

import ctypes

import numpy as np

from .native import check, lib


class PtyParams(ctypes.Structure):
    """cdx_pty_params (include/cdx_ptycho.h)."""
    _fields_ = [("rows", ctypes.c_int), ("cols", ctypes.c_int), ("obj_rows", ctypes.c_int),
                ("obj_cols", ctypes.c_int), ("nscan", ctypes.c_int), ("lambda_", ctypes.c_double),
                ("d", ctypes.c_double), ("dpupil", ctypes.c_double), ("pixelsize", ctypes.c_double),
                ("pupil_size", ctypes.c_double), ("exposure", ctypes.c_double), ("mpie", ctypes.c_int),
                ("use_bs", ctypes.c_int), ("beam_stop_size", ctypes.c_int), ("noise_level", ctypes.c_int),
                ("position_uncertainty", ctypes.c_double), ("zernike_iter", ctypes.c_int),
                ("is_fresnel", ctypes.c_int)]


def _c64(a, shape):
    a = np.ascontiguousarray(a, dtype=np.complex64)
    if a.shape != shape:
        raise ValueError(f"expected shape {shape}, got {a.shape}")
    return a


def scan_triangle(row_O, column_O, row, column, step_size):
    """ptycho::initScan_triangle (util/ptycho.cpp:139-175): a 3 x 3 grid without
    its (2, 1) point, odd columns shifted by half a step (the middle column
    stretched), centred on the object; positions in object pixels (float)."""
    sx, sy = [], []
    maxx = maxy = 0
    minx = miny = row_O
    for i in range(3):
        for j in range(3):
            if i == 2 and j == 1:
                continue
            xstep = np.float32(i + (0 if j % 2 == 0 else 0.5))
            ystep = np.float32(j * 1)
            if j == 1:
                xstep = np.float32(xstep * 2 - 1)
            py = np.float32(xstep * np.float32(step_size))
            px = np.float32(ystep * np.float32(step_size))
            sx.append(px)
            sy.append(py)
            maxx, maxy = max(maxx, int(px)), max(maxy, int(py))   # the int bounds truncate
            minx, miny = min(minx, int(px)), min(miny, int(py))
    ox = (minx + maxx - row_O + row) >> 1
    oy = (miny + maxy - column_O + column) >> 1
    return (np.array(sx, np.float32) - np.float32(ox)).astype(np.float32), \
        (np.array(sy, np.float32) - np.float32(oy)).astype(np.float32)


def scan_orders(nscan: int, n_iter: int, seed: int) -> np.ndarray:
    """The per-sweep scan orders the reference's shuffle_array gives after srand(seed)."""
    out = np.zeros((n_iter, nscan), np.int32)
    check(lib().cdx_pty_scan_orders(nscan, n_iter, seed, out.ctypes.data_as(ctypes.c_void_p)))
    return out


class Ptycho:
    """GPU ptychography context: rows x cols probe and patterns, obj_rows x obj_cols object."""

    def __init__(self, rows, cols, obj_rows, obj_cols, scanposx, scanposy, *, lam, d, dpupil, pixelsize,
                 pupil_size=500.0, exposure=1.0, mpie=True, use_bs=False, beam_stop_size=5, noise_level=0,
                 position_uncertainty=0.0, zernike_iter=0, is_fresnel=False, stream=None):
        p = PtyParams()
        check(lib().cdx_pty_params_default(ctypes.byref(p)))
        p.rows, p.cols, p.obj_rows, p.obj_cols = rows, cols, obj_rows, obj_cols
        sx = np.ascontiguousarray(scanposx, np.float32)
        sy = np.ascontiguousarray(scanposy, np.float32)
        if sx.shape != sy.shape or sx.ndim != 1:
            raise ValueError("scanposx and scanposy must be 1-D arrays of equal length")
        p.nscan = len(sx)
        p.lambda_, p.d, p.dpupil, p.pixelsize = lam, d, dpupil, pixelsize
        p.pupil_size, p.exposure, p.mpie = pupil_size, exposure, int(bool(mpie))
        p.use_bs, p.beam_stop_size = int(bool(use_bs)), beam_stop_size
        p.noise_level, p.position_uncertainty = noise_level, position_uncertainty
        p.zernike_iter = zernike_iter
        p.is_fresnel = int(is_fresnel)
        self.params = p
        self.row, self.column, self.row_O, self.column_O, self.nscan = rows, cols, obj_rows, obj_cols, p.nscan
        self._h = ctypes.c_void_p()
        st = ctypes.c_void_p(stream) if stream is not None else None
        check(lib().cdx_pty_create(ctypes.byref(p), st, ctypes.byref(self._h)))
        self.scanposx, self.scanposy = sx, sy
        check(lib().cdx_pty_set_scan(self._h, sx.ctypes.data_as(ctypes.c_void_p), sy.ctypes.data_as(ctypes.c_void_p)))

    def close(self):
        if self._h:
            lib().cdx_pty_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # --- state ---------------------------------------------------------------
    @property
    def objectWave(self) -> np.ndarray:
        out = np.empty((self.row_O, self.column_O), np.complex64)
        check(lib().cdx_pty_get_object(self._h, out.ctypes.data_as(ctypes.c_void_p)))
        return out

    @objectWave.setter
    def objectWave(self, obj):
        a = _c64(obj, (self.row_O, self.column_O))
        check(lib().cdx_pty_set_object(self._h, a.ctypes.data_as(ctypes.c_void_p)))

    @property
    def probe(self) -> np.ndarray:
        """The probe in the sample plane (what the sweeps use)."""
        out = np.empty((self.row, self.column), np.complex64)
        check(lib().cdx_pty_get_probe(self._h, out.ctypes.data_as(ctypes.c_void_p)))
        return out

    @probe.setter
    def probe(self, p):
        a = _c64(p, (self.row, self.column))
        check(lib().cdx_pty_set_probe(self._h, a.ctypes.data_as(ctypes.c_void_p)))

    @property
    def pupil(self) -> np.ndarray:
        """The probe propagated back to the pupil plane: the reference's pupilpatternWave after iterate()."""
        out = np.empty((self.row, self.column), np.complex64)
        check(lib().cdx_pty_get_pupil(self._h, out.ctypes.data_as(ctypes.c_void_p)))
        return out

    @pupil.setter
    def pupil(self, field):
        """Set the probe to the pupil-plane field propagated by dpupil (readPupilAndObject)."""
        a = _c64(field, (self.row, self.column))
        check(lib().cdx_pty_set_pupil(self._h, a.ctypes.data_as(ctypes.c_void_p)))

    @property
    def patterns(self) -> np.ndarray:
        out = np.empty((self.nscan, self.row, self.column), np.float32)
        check(lib().cdx_pty_get_patterns(self._h, out.ctypes.data_as(ctypes.c_void_p)))
        return out

    @patterns.setter
    def patterns(self, pats):
        a = np.ascontiguousarray(pats, np.float32)
        if a.shape != (self.nscan, self.row, self.column):
            raise ValueError(f"expected shape {(self.nscan, self.row, self.column)}, got {a.shape}")
        check(lib().cdx_pty_set_patterns(self._h, a.ctypes.data_as(ctypes.c_void_p)))

    # --- the steps of the reference's ptycho program ---------------------------
    def initObject(self, seed=0):
        """Random-phase unit object and the propagated pupil disk as probe (util/ptycho.cpp:363-369)."""
        check(lib().cdx_pty_init_object(self._h, seed))

    def createPattern(self, simCCDbit=False, seed=0):
        """Diffraction patterns of the current object and probe (util/ptycho.cpp:310-359): noise
        free, or recorded by the CCD model (ccdRecord) with simCCDbit."""
        if simCCDbit:
            check(lib().cdx_pty_simulate_ccd(self._h, ctypes.c_ulonglong(seed)))
        else:
            check(lib().cdx_pty_simulate(self._h))

    def iterate(self, n_iter, first_iter=0, orders=None, seed=1):
        """ptycho::iterate: n_iter sweeps from iteration index first_iter; scan orders given
        (n_iter x nscan) or drawn like the reference's rand() shuffle after srand(seed)
        (glibc's rand() is seeded with 1 unless the program calls srand).  Returns GPU ms."""
        if orders is not None:
            o = np.ascontiguousarray(orders, np.int32)
            if o.shape != (n_iter, self.nscan):
                raise ValueError(f"orders must be {(n_iter, self.nscan)}")
            ptr = o.ctypes.data_as(ctypes.c_void_p)
        else:
            o, ptr = None, None
        check(lib().cdx_pty_iterate(self._h, first_iter, n_iter, ptr, seed))
        ms = ctypes.c_float()
        check(lib().cdx_pty_last_ms(self._h, ctypes.byref(ms)))
        return float(ms.value)
