"""Learned warm start: the CUDA U-Net of include/cdx_unet.h through ctypes.

    net = UNet(n=256, levels=4, base=32, batch=64)
    I, amp, ph, sup = forward_model(256, 64, seed, first=0)     # device tensors
    loss = net.train_step(I, amp, ph, sup, lr=1e-3)
    out = net.forward(I)                                          # [b, 4, n, n]
    psi0, support = net.warm_start(I, out)                        # for Context.set_initial / set_support

Everything runs on the GPU through the library; there is no CPU fallback.
The network's kernels run on a stream of its own; every method first makes
that stream wait for the caller's current stream (so tensors the caller just
produced, e.g. by forward_model, are complete) and afterwards makes the
caller's current stream wait for the network's (so its outputs are complete
for whatever the caller runs next).
"""
from __future__ import annotations

import ctypes

import numpy as np

from cdixx_gb300 import native


class UNetConfig(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int), ("levels", ctypes.c_int), ("base", ctypes.c_int), ("batch", ctypes.c_int),
                ("groups", ctypes.c_int), ("slope", ctypes.c_float), ("support_weight", ctypes.c_float),
                ("seed", ctypes.c_ulonglong), ("umma", ctypes.c_int)]


def _ptr(t):
    if not (hasattr(t, "is_cuda") and t.is_cuda and t.is_contiguous()):
        raise ValueError("expected a contiguous CUDA tensor")
    return ctypes.c_void_p(t.data_ptr())


def default_config(**kw) -> UNetConfig:
    c = UNetConfig()
    native.check(native.lib().cdx_unet_config_default(ctypes.byref(c)))
    for k, v in kw.items():
        if not hasattr(c, k):
            raise KeyError(k)
        setattr(c, k, v)
    return c


class UNet:
    def __init__(self, stream=None, **cfg):
        import torch
        self.cfg = default_config(**cfg)
        self._h = ctypes.c_void_p()
        self.stream = torch.cuda.Stream() if stream is None else torch.cuda.ExternalStream(stream)
        native.check(native.lib().cdx_unet_create(ctypes.byref(self.cfg), ctypes.c_void_p(self.stream.cuda_stream),
                                                  ctypes.byref(self._h)))
        self.n_params = int(native.lib().cdx_unet_param_count(self._h))

    def _enter(self):
        import torch
        self.stream.wait_stream(torch.cuda.current_stream())

    def _leave(self):
        import torch
        torch.cuda.current_stream().wait_stream(self.stream)

    def close(self):
        if self._h:
            native.lib().cdx_unet_destroy(self._h)
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

    def params(self) -> np.ndarray:
        out = np.empty(self.n_params, np.float32)
        native.check(native.lib().cdx_unet_get_params(self._h, out.ctypes.data_as(ctypes.c_void_p), self.n_params))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        if p.size != self.n_params:
            raise ValueError("parameter count mismatch")
        native.check(native.lib().cdx_unet_set_params(self._h, p.ctypes.data_as(ctypes.c_void_p), self.n_params))

    def grads(self) -> np.ndarray:
        out = np.empty(self.n_params, np.float32)
        native.check(native.lib().cdx_unet_get_grads(self._h, out.ctypes.data_as(ctypes.c_void_p), self.n_params))
        return out

    def forward(self, intensity, out=None):
        import torch
        b = intensity.shape[0]
        n = self.cfg.n
        if out is None:
            out = torch.empty((b, 4, n, n), dtype=torch.float32, device=intensity.device)
        self._enter()
        native.check(native.lib().cdx_unet_forward(self._h, _ptr(intensity), _ptr(out), b))
        self._leave()
        return out

    def loss_backward(self, intensity, amp_t, phase_t, support_t) -> float:
        loss = ctypes.c_double()
        self._enter()
        native.check(native.lib().cdx_unet_loss_backward(self._h, _ptr(intensity), _ptr(amp_t), _ptr(phase_t),
                                                         _ptr(support_t), intensity.shape[0], ctypes.byref(loss)))
        self._leave()
        return loss.value

    def adam_step(self, lr=1e-3):
        self._enter()
        native.check(native.lib().cdx_unet_adam_step(self._h, ctypes.c_float(lr)))
        self._leave()

    def train_step(self, intensity, amp_t, phase_t, support_t, lr=1e-3) -> float:
        loss = self.loss_backward(intensity, amp_t, phase_t, support_t)
        self.adam_step(lr)
        return loss

    def warm_start(self, intensity, out, dilate=3):
        """(psi0 complex64 [b, n, n] pattern FFT order, support float [b, n, n] object frame) on the device."""
        import torch
        b, n = intensity.shape[0], self.cfg.n
        psi0 = torch.empty((b, n, n), dtype=torch.complex64, device=intensity.device)
        sup = torch.empty((b, n, n), dtype=torch.float32, device=intensity.device)
        self._enter()
        native.check(native.lib().cdx_unet_warm_start(self._h, _ptr(intensity), _ptr(out), b, int(dilate), _ptr(psi0),
                                                      _ptr(sup)))
        self._leave()
        return psi0, sup


def forward_model(n, count, seed, first=0, photons=1e6, device="cuda", stream=None):
    """Seeded synthetic pairs on the GPU: (intensity FFT order, amplitude, phase, support; centred).
    Queued on `stream` (default: the current torch stream) without waiting for it."""
    import torch
    I = torch.empty((count, n, n), dtype=torch.float32, device=device)
    a = torch.empty_like(I)
    p = torch.empty_like(I)
    s = torch.empty_like(I)
    st = ctypes.c_void_p(stream if stream is not None else torch.cuda.current_stream().cuda_stream)
    native.check(native.lib().cdx_forward_model(n, count, ctypes.c_ulonglong(seed), first, ctypes.c_double(photons),
                                                _ptr(I), _ptr(a), _ptr(p), _ptr(s), st))
    return I, a, p, s


def train(net: UNet, steps, seed, photons=1e6, lr=1e-3, first=0, log_every=0):
    """Adam on fresh forward-model batches: batch k uses patterns first + k*batch .. (k+1)*batch - 1."""
    b, n = net.cfg.batch, net.cfg.n
    losses = []
    for k in range(steps):
        I, a, p, s = forward_model(n, b, seed, first + k * b, photons)
        losses.append(net.train_step(I, a, p, s, lr))
        if log_every and (k % log_every == 0 or k == steps - 1):
            print(f"step {k}: loss {losses[-1]:.5f}", flush=True)
    return losses
