"""ctypes binding of the C ABI in ``include/cdx.h`` (``_lib/libcdx.so``).

There is no CPU fallback: every call goes to the CUDA library, and loading
fails loudly when the library has not been built.  Arrays may be NumPy
arrays (host) or CUDA torch tensors (device); complex data are complex64 /
interleaved float pairs.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libcdx.so"

CDX_OK, CDX_ERR_ARG, CDX_ERR_SIZE, CDX_ERR_CUDA, CDX_ERR_ALGO, CDX_ERR_STATE, CDX_ERR_IO, \
    CDX_ERR_NOMEM, CDX_ERR_CONFIG, CDX_ERR_NOLIB = range(10)
CDX_HOST, CDX_DEVICE = 0, 1
CDX_FFT_ORDER, CDX_CENTERED = 0, 1
RAAR, ER, POSER, HIO, POSHIO, FHIO, SHRINKWRAP, XCORRELATION, KKT, TV = range(10)
SHRINK_FOURIER, SHRINK_SPATIAL = 0, 1
FFT_FP32, FFT_TC_BF16, FFT_TC_MMA = 0, 1, 2


class CdxError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"cdx error {code}: {msg}")
        self.code = code


class Params(ctypes.Structure):
    _fields_ = [
        ("rows", ctypes.c_int), ("cols", ctypes.c_int), ("batch", ctypes.c_int),
        ("beta", ctypes.c_float), ("shrink_threshold", ctypes.c_float),
        ("oversampling_spt", ctypes.c_float), ("exposure", ctypes.c_float),
        ("rcolor", ctypes.c_int), ("sim_ccd_bit", ctypes.c_int), ("noise_level", ctypes.c_int),
        ("shrink_mode", ctypes.c_int), ("sigma0", ctypes.c_float), ("sigma_min", ctypes.c_float),
        ("sigma_decay", ctypes.c_float), ("use_graph", ctypes.c_int), ("rf_every", ctypes.c_int),
        ("stop_rfactor", ctypes.c_float), ("fft_mode", ctypes.c_int), ("prtf_iter", ctypes.c_int),
        ("autotune", ctypes.c_int), ("plateau_iters", ctypes.c_int), ("plateau_tol", ctypes.c_float),
    ]


class Stats(ctypes.Structure):
    _fields_ = [
        ("steps", ctypes.c_int), ("iterations", ctypes.c_int), ("shrinkwraps", ctypes.c_int),
        ("residual", ctypes.c_double), ("rfactor", ctypes.c_double), ("threshold", ctypes.c_float),
        ("flags", ctypes.c_int), ("gpu_ms", ctypes.c_double), ("launches", ctypes.c_int),
        ("converged_iter", ctypes.c_int), ("rfactor_min", ctypes.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


# exported symbols and their argument types (include/cdx.h)
_P = ctypes.c_void_p
_I = ctypes.c_int
_F = ctypes.c_float
_LL = ctypes.c_longlong
_SIGS = {
    "cdx_params_default": [ctypes.POINTER(Params)],
    "cdx_create": [ctypes.POINTER(Params), _P, ctypes.POINTER(_P)],
    "cdx_destroy": [_P],
    "cdx_get_params": [_P, ctypes.POINTER(Params)],
    "cdx_device_arrays": [_P, _P, _P, _P, _P],
    "cdx_set_pattern": [_P, _I, _P, _I, _I, _F],
    "cdx_set_beamstop": [_P, _I, _P, _I, _I],
    "cdx_set_initial": [_P, _I, _P, _I],
    "cdx_random_start": [_P, ctypes.c_ulonglong],
    "cdx_set_support": [_P, _I, _P, _I],
    "cdx_set_stop_rfactor": [_P, _I, ctypes.c_double],
    "cdx_run": [_P, ctypes.c_char_p, ctypes.POINTER(Stats)],
    "cdx_run_async": [_P, ctypes.c_char_p],
    "cdx_get_stats": [_P, _I, ctypes.POINTER(Stats)],
    "cdx_group_create": [ctypes.POINTER(_P), _I, ctypes.POINTER(_P)],
    "cdx_group_run": [_P, ctypes.c_char_p, ctypes.POINTER(ctypes.c_double)],
    "cdx_group_destroy": [_P],
    "cdx_group_set_concurrent": [_P, _I],
    "cdx_get_object": [_P, _I, _P, _I],
    "cdx_get_fourier": [_P, _I, _P, _I],
    "cdx_get_support": [_P, _I, _P, _I],
    "cdx_get_prtf": [_P, _I, _P, _I],
    "cdx_get_tuning": [_P, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.c_char_p, _I],
    "cdx_tuning_save": [ctypes.c_char_p],
    "cdx_tuning_load": [ctypes.c_char_p, ctypes.POINTER(_I)],
    "cdx_phase_retrieve_host": [ctypes.POINTER(Params), ctypes.c_char_p, _P, _P, ctypes.c_ulonglong,
                                _P, _P, _P, ctypes.POINTER(Stats)],
    "cdx_release_host_cache": [],
    "cdx_fft2": [_P, _P, _I, _I, _I, _I, _P],
    "cdx_fft2_ex": [_P, _P, _I, _I, _I, _I, _I, _P],
    "cdx_ccd_noise": [_P, _LL, _F, _F, _I, ctypes.c_ulonglong, _P],
    "cdx_fresnel_factor": [ctypes.c_double, ctypes.c_double, ctypes.c_double, _I, _I],
    "cdx_fresnel_phase": [_P, _I, _I, _I, _F, _P],
    "cdx_apply_mod_abs": [_P, _P, _LL, _P],
    "cdx_apply_mod": [_P, _P, _P, _I, _F, _I, _LL, _P],
    "cdx_apply_support": [_P, _P, _P, _F, _F, _I, _LL, _P],
    "cdx_convert_fo": [_P, _P, _I, _I, _I, _I, _P],
    "cdx_iterate_noalloc": [_I, _I, _I, _F, _I, _P, _P, _F, _P, _P, _P, _P],
    "cdx_algo_expand": [ctypes.c_char_p, ctypes.POINTER(_I), _I, ctypes.POINTER(_I)],
    "cdx_read_bin": [ctypes.c_char_p, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I), _P,
                     ctypes.c_size_t],
    "cdx_write_bin": [ctypes.c_char_p, _P, _I, _I, _I],
    "cdx_size_supported": [_I],
    "cdx_last_error": [],
    "cdx_version": [],
    # include/cdx_unet.h
    "cdx_unet_config_default": [ctypes.c_void_p],
    "cdx_unet_create": [ctypes.c_void_p, _P, ctypes.POINTER(_P)],
    "cdx_unet_destroy": [_P],
    "cdx_unet_param_count": [_P],
    "cdx_unet_get_params": [_P, _P, _LL],
    "cdx_unet_set_params": [_P, _P, _LL],
    "cdx_unet_get_grads": [_P, _P, _LL],
    "cdx_unet_forward": [_P, _P, _P, _I],
    "cdx_unet_loss_backward": [_P, _P, _P, _P, _P, _I, ctypes.POINTER(ctypes.c_double)],
    "cdx_unet_adam_step": [_P, _F],
    "cdx_unet_warm_start": [_P, _P, _P, _I, _I, _P, _P],
    "cdx_gemm_bf16_tc": [_P, _P, _P, _I, _I, _I, _P, _P],
    "cdx_forward_model": [_I, _I, ctypes.c_ulonglong, _LL, ctypes.c_double, _P, _P, _P, _P, _P],
    # include/cdx_ptycho.h
    "cdx_pty_params_default": [_P],
    "cdx_pty_create": [_P, _P, ctypes.POINTER(_P)],
    "cdx_pty_destroy": [_P],
    "cdx_pty_set_scan": [_P, _P, _P],
    "cdx_pty_set_patterns": [_P, _P],
    "cdx_pty_get_patterns": [_P, _P],
    "cdx_pty_set_object": [_P, _P],
    "cdx_pty_get_object": [_P, _P],
    "cdx_pty_set_probe": [_P, _P],
    "cdx_pty_get_probe": [_P, _P],
    "cdx_pty_get_pupil": [_P, _P],
    "cdx_pty_set_pupil": [_P, _P],
    "cdx_pty_init_object": [_P, ctypes.c_ulonglong],
    "cdx_pty_simulate": [_P],
    "cdx_pty_simulate_ccd": [_P, ctypes.c_ulonglong],
    "cdx_ccd_record": [_P, _LL, _I, _F, _I, _F, ctypes.c_ulonglong, _P],
    "cdx_pty_iterate": [_P, _I, _I, _P, ctypes.c_uint],
    "cdx_pty_last_ms": [_P, ctypes.POINTER(ctypes.c_float)],
    "cdx_pty_scan_orders": [_I, _I, ctypes.c_uint, _P],
}
_RESTYPE = {"cdx_last_error": ctypes.c_char_p, "cdx_version": ctypes.c_char_p, "cdx_unet_destroy": None,
            "cdx_unet_param_count": ctypes.c_longlong, "cdx_fresnel_factor": ctypes.c_float}

_lib = None


def lib():
    """Load ``libcdx.so`` (raises when it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise CdxError(CDX_ERR_NOLIB, f"{LIB_PATH} missing: run `python -m cdixx_gb300.build` "
                                          "(the CDI path has no CPU fallback)")
        L = ctypes.CDLL(str(LIB_PATH))
        for name, args in _SIGS.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = _RESTYPE.get(name, ctypes.c_int)
        _lib = L
    return _lib


def exported_symbols():
    return list(_SIGS)


def check(code):
    if code != CDX_OK:
        raise CdxError(code, lib().cdx_last_error().decode(errors="replace"))


def default_params(rows, cols, batch=1, **kw) -> Params:
    p = Params()
    check(lib().cdx_params_default(ctypes.byref(p)))
    p.rows, p.cols, p.batch = rows, cols, batch
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p


def _buf(x, complex_ok=True):
    """(pointer, where, keepalive) of a host NumPy array or a CUDA tensor."""
    if hasattr(x, "data_ptr") and getattr(x, "is_cuda", False):
        if not x.is_contiguous():
            raise ValueError("device tensor must be contiguous")
        return ctypes.c_void_p(x.data_ptr()), CDX_DEVICE, x
    a = np.ascontiguousarray(x)
    if np.iscomplexobj(a):
        a = np.ascontiguousarray(a, dtype=np.complex64)
    else:
        a = np.ascontiguousarray(a, dtype=np.float32)
    return a.ctypes.data_as(ctypes.c_void_p), CDX_HOST, a


def algo_expand(s: str):
    n = ctypes.c_int()
    check(lib().cdx_algo_expand(s.encode(), None, 0, ctypes.byref(n)))
    out = (ctypes.c_int * max(n.value, 1))()
    check(lib().cdx_algo_expand(s.encode(), out, n.value, ctypes.byref(n)))
    return list(out[: n.value])


def read_bin(path):
    r, c, z = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    check(lib().cdx_read_bin(str(path).encode(), ctypes.byref(r), ctypes.byref(c), ctypes.byref(z), None, 0))
    out = np.empty((r.value, c.value), np.complex64 if z.value else np.float32)
    check(lib().cdx_read_bin(str(path).encode(), ctypes.byref(r), ctypes.byref(c), ctypes.byref(z),
                             out.ctypes.data_as(ctypes.c_void_p), out.size * (2 if z.value else 1)))
    return out


def write_bin(path, a):
    a = np.ascontiguousarray(a)
    z = np.iscomplexobj(a)
    a = a.astype(np.complex64 if z else np.float32)
    check(lib().cdx_write_bin(str(path).encode(), a.ctypes.data_as(ctypes.c_void_p), a.shape[0], a.shape[1],
                              int(z)))


class Context:
    """A device context holding `batch` patterns of rows x cols (cdx_create)."""

    def __init__(self, params: Params, stream=None):
        self.params = params
        self._h = ctypes.c_void_p()
        st = ctypes.c_void_p(stream) if stream is not None else None
        check(lib().cdx_create(ctypes.byref(params), st, ctypes.byref(self._h)))
        self.rows, self.cols, self.batch = params.rows, params.cols, params.batch

    def close(self):
        if self._h:
            lib().cdx_destroy(self._h)
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

    def tuning(self):
        """(pdl bits, row_chunk, report) of the launch variant in use (cdx_get_tuning): pdl bit 0 =
        the column pass is a programmatic dependent launch, bit 1 = the row pass, -1 = defaults."""
        pdl, chunk = ctypes.c_int(), ctypes.c_int()
        buf = ctypes.create_string_buffer(1024)
        check(lib().cdx_get_tuning(self._h, ctypes.byref(pdl), ctypes.byref(chunk), buf, 1024))
        return pdl.value, chunk.value, buf.value.decode()

    def set_pattern(self, idx, intensity, layout=CDX_FFT_ORDER, scale=1.0):
        p, w, _k = _buf(intensity)
        check(lib().cdx_set_pattern(self._h, idx, p, w, layout, scale))

    def set_beamstop(self, idx, bs, layout=CDX_FFT_ORDER):
        p, w, _k = _buf(bs)
        check(lib().cdx_set_beamstop(self._h, idx, p, w, layout))

    def set_initial(self, idx, psi0):
        p, w, _k = _buf(psi0)
        check(lib().cdx_set_initial(self._h, idx, p, w))

    def random_start(self, seed):
        check(lib().cdx_random_start(self._h, seed))

    def set_support(self, idx, spt):
        p, w, _k = _buf(spt)
        check(lib().cdx_set_support(self._h, idx, p, w))

    def set_stop_rfactor(self, idx, stop):
        check(lib().cdx_set_stop_rfactor(self._h, idx, float(stop)))

    def run(self, algorithm: str) -> dict:
        s = Stats()
        check(lib().cdx_run(self._h, algorithm.encode(), ctypes.byref(s)))
        return s.as_dict()

    def run_async(self, algorithm: str):
        check(lib().cdx_run_async(self._h, algorithm.encode()))

    def stats(self, idx=0) -> dict:
        s = Stats()
        check(lib().cdx_get_stats(self._h, idx, ctypes.byref(s)))
        return s.as_dict()

    def _get(self, fn, idx, cplx, out=None):
        if out is not None:
            p, w, _k = _buf(out)
            check(fn(self._h, idx, p, w))
            return out
        a = np.empty((self.rows, self.cols), np.complex64 if cplx else np.float32)
        check(fn(self._h, idx, a.ctypes.data_as(ctypes.c_void_p), CDX_HOST))
        return a

    def get_object(self, idx=0, out=None):
        return self._get(lib().cdx_get_object, idx, True, out)

    def get_fourier(self, idx=0, out=None):
        return self._get(lib().cdx_get_fourier, idx, True, out)

    def get_support(self, idx=0, out=None):
        return self._get(lib().cdx_get_support, idx, False, out)

    def get_prtf(self, idx=0):
        """PRTF of the last run: rows/2 floats (the prtf.txt column)."""
        a = np.empty(self.rows // 2, np.float32)
        check(lib().cdx_get_prtf(self._h, idx, a.ctypes.data_as(ctypes.c_void_p), CDX_HOST))
        return a

    def device_arrays(self):
        ptrs = [ctypes.c_void_p() for _ in range(4)]
        check(lib().cdx_device_arrays(self._h, *[ctypes.byref(p) for p in ptrs]))
        return [p.value for p in ptrs]


class Group:
    """Contexts of different pattern sizes run as one CUDA graph (cdx_group_*)."""

    def __init__(self, contexts, concurrent=False):
        self.contexts = list(contexts)
        arr = (ctypes.c_void_p * len(self.contexts))(*[c._h.value for c in self.contexts])
        self._h = ctypes.c_void_p()
        check(lib().cdx_group_create(arr, len(self.contexts), ctypes.byref(self._h)))
        if concurrent:
            self.set_concurrent(True)

    def set_concurrent(self, concurrent: bool):
        """Branch order of the group's graph: side by side (True) or one after another."""
        check(lib().cdx_group_set_concurrent(self._h, int(bool(concurrent))))

    def run(self, algorithm: str) -> float:
        ms = ctypes.c_double()
        check(lib().cdx_group_run(self._h, algorithm.encode(), ctypes.byref(ms)))
        return ms.value

    def close(self):
        if self._h:
            lib().cdx_group_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def phase_retrieve_host(params: Params, algorithm: str, intensity, psi0=None, seed=0, out=None):
    """One-call host-buffer path (cdx_phase_retrieve_host): returns (rho, psi, support, stats).
    `out` = (rho, psi, support) host arrays to fill (e.g. views of pinned memory), else new ones."""
    I = np.ascontiguousarray(intensity, np.float32)
    if out is not None:
        rho, psi, spt = out
        if rho.dtype != np.complex64 or psi.dtype != np.complex64 or spt.dtype != np.float32 or \
                not all(a.shape == I.shape and a.flags.c_contiguous for a in out):
            raise ValueError("out: contiguous complex64, complex64, float32 arrays of the pattern's shape")
    else:
        rho = np.empty(I.shape, np.complex64)
        psi = np.empty(I.shape, np.complex64)
        spt = np.empty(I.shape, np.float32)
    p0 = None if psi0 is None else np.ascontiguousarray(psi0, np.complex64)
    s = Stats()
    vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    check(lib().cdx_phase_retrieve_host(ctypes.byref(params), algorithm.encode(), vp(I),
                                        None if p0 is None else vp(p0), seed, vp(rho), vp(psi), vp(spt),
                                        ctypes.byref(s)))
    return rho, psi, spt, s.as_dict()


def tuning_save(path):
    """Write the autotuner's decisions of this process to a JSON file (cdx_tuning_save)."""
    check(lib().cdx_tuning_save(str(path).encode()))


def tuning_load(path) -> int:
    """Read autotuner decisions from a JSON file written by tuning_save (cdx_tuning_load);
    returns the number of entries."""
    n = ctypes.c_int()
    check(lib().cdx_tuning_load(str(path).encode(), ctypes.byref(n)))
    return n.value


def release_host_cache():
    """Free the context phase_retrieve_host keeps for its next call (cdx_release_host_cache)."""
    check(lib().cdx_release_host_cache())


def _stream_ptr(stream):
    if stream is None:
        return None
    return ctypes.c_void_p(stream)


def fft2(x, out, inverse=False, stream=None, fft_mode=0):
    """myFFT / myIFFT on device tensors (complex64, shape [..., rows, cols]).

    fft_mode 0 (FFT_FP32) is the FP32 SIMT path; 1 (FFT_TC_BF16) runs the
    radix-16 passes on tcgen05, 2 (FFT_TC_MMA) on mma.sync; both run the
    radix-16 passes on the tensor cores with a split-BF16 operand.
    """
    rows, cols = x.shape[-2], x.shape[-1]
    batch = int(np.prod(x.shape[:-2])) if x.dim() > 2 else 1
    check(lib().cdx_fft2_ex(ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(out.data_ptr()), rows, cols, batch,
                            int(inverse), int(fft_mode), _stream_ptr(stream)))
    return out


def ccd_noise(pattern, noise_level, exposure=1.0, rcolor=65535, seed=0, stream=None):
    """applyPoissonNoise_WO on a device float tensor, in place."""
    check(lib().cdx_ccd_noise(ctypes.c_void_p(pattern.data_ptr()), pattern.numel(), noise_level, exposure, rcolor,
                              ctypes.c_ulonglong(seed), _stream_ptr(stream)))
    return pattern


def fresnel_factor(lam, distance, pixelsize, rows, remove=False):
    """propagator's Fresnel phase factor pi lambda d / (pixelsize rows)^2 (float members)."""
    return float(lib().cdx_fresnel_factor(lam, distance, pixelsize, rows, int(remove)))


def fresnel_phase(field, factor, stream=None):
    """multiplyFresnelPhase_Device on a device complex64 tensor [..., rows, cols], in place."""
    rows, cols = field.shape[-2:]
    batch = int(np.prod(field.shape[:-2])) if field.dim() > 2 else 1
    check(lib().cdx_fresnel_phase(ctypes.c_void_p(field.data_ptr()), rows, cols, batch, factor, _stream_ptr(stream)))
    return field


def apply_mod_abs(psi, intensity, stream=None):
    check(lib().cdx_apply_mod_abs(ctypes.c_void_p(psi.data_ptr()), ctypes.c_void_p(intensity.data_ptr()),
                                  psi.numel(), _stream_ptr(stream)))


def apply_mod(psi, intensity, beamstop=None, noise_level=0, scale=1.0, rcolor=65535, stream=None):
    bs = None if beamstop is None else ctypes.c_void_p(beamstop.data_ptr())
    check(lib().cdx_apply_mod(ctypes.c_void_p(psi.data_ptr()), ctypes.c_void_p(intensity.data_ptr()), bs,
                              noise_level, scale, rcolor, psi.numel(), _stream_ptr(stream)))


def apply_support(rho, rho_prime, support, threshold, beta, algo, stream=None):
    check(lib().cdx_apply_support(ctypes.c_void_p(rho.data_ptr()), ctypes.c_void_p(rho_prime.data_ptr()),
                                  ctypes.c_void_p(support.data_ptr()), threshold, beta, algo, rho.numel(),
                                  _stream_ptr(stream)))


def convert_fo(x, out=None, stream=None):
    out = x if out is None else out
    rows, cols = x.shape[-2], x.shape[-1]
    batch = int(np.prod(x.shape[:-2])) if x.dim() > 2 else 1
    check(lib().cdx_convert_fo(ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(out.data_ptr()), rows, cols,
                               batch, int(x.is_complex()), _stream_ptr(stream)))
    return out
