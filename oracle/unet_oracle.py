"""FP64 NumPy restatement of the warm-start U-Net (test infrastructure only).

The oracle for the CUDA network in cdixx_gb300/csrc/cdx_unet*.cu: the same
layer list, flat parameter order, GroupNorm + LeakyReLU, twin-invariant loss
and analytic backward, in float64.  Used by the tests to check the GPU
gradients (and checked itself against central finite differences).  The
reference's own U-Nets (python/UNet.py:45-85; Conv3x3-BN-LeakyReLU blocks,
stride-2 conv down, ConvTranspose up, concatenated skips) are PyTorch and
cannot run here; this is the build's network, not a restatement of theirs.
"""
from __future__ import annotations

import numpy as np


# ----------------------------------------------------------------- layers
def build(n, levels, base):
    """Layer list: dicts with kind ('conv'|'convt'|'head'), in0, in1, cin, cout, k, s, p, in_h, out_h,
    and parameter offsets (w, g, b, bias) in the flat vector; returns (layers, n_params)."""
    L = []
    npar = 0

    def add(kind, in0, in1, cin, cout, k, s, p, in_h):
        nonlocal npar
        d = dict(kind=kind, in0=in0, in1=in1, cin=cin, cout=cout, k=k, s=s, p=p, in_h=in_h)
        d["out_h"] = in_h * 2 if kind == "convt" else (in_h + 2 * p - k) // s + 1
        if kind == "convt":
            d["wshape"] = (cin, k, k, cout)
        else:
            d["wshape"] = (cout, k, k, 1 if in0 < 0 else cin)
        d["w"] = npar
        npar += int(np.prod(d["wshape"]))
        if kind != "head":
            d["g"] = npar
            npar += cout
            d["b"] = npar
            npar += cout
        else:
            d["bias"] = npar
            npar += 4
        L.append(d)
        return len(L) - 1

    skip = [0] * levels
    h, ch = n, base
    cur = add("conv", -1, -1, 1, ch, 3, 1, 1, h)
    cur = add("conv", cur, -1, ch, ch, 3, 1, 1, h)
    skip[0] = cur
    for lv in range(1, levels):
        cur = add("conv", cur, -1, ch, ch * 2, 3, 2, 1, h)
        h //= 2
        ch *= 2
        cur = add("conv", cur, -1, ch, ch, 3, 1, 1, h)
        skip[lv] = cur
    for lv in range(levels - 2, -1, -1):
        up = add("convt", cur, -1, ch, ch // 2, 2, 2, 0, h)
        h *= 2
        ch //= 2
        cur = add("conv", up, skip[lv], 2 * ch, ch, 3, 1, 1, h)
    add("head", cur, -1, ch, 4, 1, 1, 0, h)
    return L, npar


def _cols(x, k, s, p, Ho, Wo):
    N, H, W, C = x.shape
    xp = np.pad(x, ((0, 0), (p, p), (p, p), (0, 0)))
    cols = np.empty((N, Ho, Wo, k, k, C))
    for ky in range(k):
        for kx in range(k):
            cols[:, :, :, ky, kx, :] = xp[:, ky:ky + s * (Ho - 1) + 1:s, kx:kx + s * (Wo - 1) + 1:s, :]
    return cols


def conv_fwd(x, w, s, p):
    Co, k = w.shape[0], w.shape[1]
    N, H, W, C = x.shape
    Ho, Wo = (H + 2 * p - k) // s + 1, (W + 2 * p - k) // s + 1
    cols = _cols(x, k, s, p, Ho, Wo)
    y = cols.reshape(-1, k * k * C) @ w.reshape(Co, -1).T
    return y.reshape(N, Ho, Wo, Co)


def conv_dgrad(dy, w, s, p, in_shape):
    N, H, W, C = in_shape
    Co, k = w.shape[0], w.shape[1]
    Ho, Wo = dy.shape[1], dy.shape[2]
    dcols = (dy.reshape(-1, Co) @ w.reshape(Co, -1)).reshape(N, Ho, Wo, k, k, C)
    dxp = np.zeros((N, H + 2 * p, W + 2 * p, C))
    for ky in range(k):
        for kx in range(k):
            dxp[:, ky:ky + s * (Ho - 1) + 1:s, kx:kx + s * (Wo - 1) + 1:s, :] += dcols[:, :, :, ky, kx, :]
    return dxp[:, p:p + H, p:p + W, :]


def conv_wgrad(x, dy, k, s, p):
    Co = dy.shape[3]
    cols = _cols(x, k, s, p, dy.shape[1], dy.shape[2])
    return (dy.reshape(-1, Co).T @ cols.reshape(dy.shape[0] * dy.shape[1] * dy.shape[2], -1)).reshape(
        Co, k, k, x.shape[3])


def gn_fwd(x, gamma, beta, G, slope, eps=1e-5):
    N, H, W, C = x.shape
    xg = x.reshape(N, H * W, G, C // G)
    mean = xg.mean(axis=(1, 3), keepdims=True)
    var = xg.var(axis=(1, 3), keepdims=True)
    rstd = 1.0 / np.sqrt(var + eps)
    xh = ((xg - mean) * rstd).reshape(N, H, W, C)
    z = xh * gamma + beta
    a = np.where(z > 0, z, slope * z)
    return a, (xh, rstd, z)


def gn_bwd(da, cache, gamma, G, slope):
    xh, rstd, z = cache
    N, H, W, C = da.shape
    dz = da * np.where(z > 0, 1.0, slope)
    dgamma = (dz * xh).sum(axis=(0, 1, 2))
    dbeta = dz.sum(axis=(0, 1, 2))
    dxh = (dz * gamma).reshape(N, H * W, G, C // G)
    xhg = xh.reshape(N, H * W, G, C // G)
    M = H * W * (C // G)
    s1 = dxh.sum(axis=(1, 3), keepdims=True)
    s2 = (dxh * xhg).sum(axis=(1, 3), keepdims=True)
    dx = rstd * (dxh - s1 / M - xhg * s2 / M)
    return dx.reshape(N, H, W, C), dgamma, dbeta


def bf16(x):
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    b = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def prep_input(I):
    """log(1 + I) / max, centred (fftshift), [N, n, n, 1]."""
    x = np.log1p(np.maximum(I.astype(np.float64), 0))
    mx = x.reshape(x.shape[0], -1).max(axis=1)
    x = x / np.where(mx > 0, mx, 1.0)[:, None, None]
    return np.fft.fftshift(x, axes=(1, 2))[..., None]


def _twin(a):
    n = a.shape[-1]
    idx = (-np.arange(n)) % n
    return a[..., idx, :][..., idx]


def loss_terms(o, at, pt, st, ws):
    c, s = np.cos(pt), np.sin(pt)
    z = o[..., 3]
    bce = np.maximum(z, 0) - z * st + np.log1p(np.exp(-np.abs(z)))
    return (o[..., 0] - at) ** 2 + at * ((o[..., 1] - c) ** 2 + (o[..., 2] - s) ** 2) + ws * bce


def forward_backward(params, I, amp_t, ph_t, sup_t, n, levels, base, groups=8, slope=0.01, ws=0.1, backward=True,
                     round_bf16=False):
    """(loss, grads, head output [N, n, n, 4]) of the network on intensity I [N, n, n] (FFT order).

    round_bf16 rounds to BF16 where the CUDA network does (weights, the input,
    every activation, and the conv-output gradients fed to the products);
    everything else stays float64."""
    L, npar = build(n, levels, base)
    P = params.astype(np.float64)
    rnd = bf16 if round_bf16 else (lambda a: a)
    acts, caches, ins = [], [], []
    x0 = rnd(prep_input(I))

    def act(i):
        return x0 if i < 0 else acts[i]

    for d in L:
        w = rnd(P[d["w"]:d["w"] + int(np.prod(d["wshape"]))].reshape(d["wshape"]))
        if d["kind"] == "convt":
            xin = act(d["in0"])
            N = xin.shape[0]
            y = conv_dgrad(xin, w, d["s"], d["p"], (N, d["out_h"], d["out_h"], d["cout"]))
        else:
            xin = act(d["in0"]) if d["in1"] < 0 else np.concatenate([act(d["in0"]), act(d["in1"])], axis=3)
            y = conv_fwd(xin, w, d["s"], d["p"])
        ins.append(xin)
        if d["kind"] == "head":
            y = y + P[d["bias"]:d["bias"] + 4]
            acts.append(y)
            caches.append(None)
        else:
            a, cache = gn_fwd(y, P[d["g"]:d["g"] + d["cout"]], P[d["b"]:d["b"] + d["cout"]], groups, slope)
            acts.append(rnd(a))
            caches.append(cache)
    out = acts[-1]
    N = out.shape[0]
    l_id = loss_terms(out, amp_t, ph_t, sup_t, ws).reshape(N, -1).mean(axis=1)
    l_tw = loss_terms(out, _twin(amp_t), -_twin(ph_t), _twin(sup_t), ws).reshape(N, -1).mean(axis=1)
    twin = l_tw < l_id
    loss = float(np.where(twin, l_tw, l_id).mean())
    if not backward:
        return loss, None, out
    at = np.where(twin[:, None, None], _twin(amp_t), amp_t)
    pt = np.where(twin[:, None, None], -_twin(ph_t), ph_t)
    st = np.where(twin[:, None, None], _twin(sup_t), sup_t)
    sc = 1.0 / (n * n * N)
    dout = np.zeros_like(out)
    dout[..., 0] = 2 * (out[..., 0] - at) * sc
    dout[..., 1] = 2 * at * (out[..., 1] - np.cos(pt)) * sc
    dout[..., 2] = 2 * at * (out[..., 2] - np.sin(pt)) * sc
    dout[..., 3] = ws * (1 / (1 + np.exp(-out[..., 3])) - st) * sc
    grads = np.zeros(npar)
    dacts = [np.zeros_like(a) for a in acts]
    dacts[-1] = dout
    for li in range(len(L) - 1, -1, -1):
        d = L[li]
        w = rnd(P[d["w"]:d["w"] + int(np.prod(d["wshape"]))].reshape(d["wshape"]))
        if d["kind"] == "head":
            dy = dacts[li]
            grads[d["bias"]:d["bias"] + 4] = dy.sum(axis=(0, 1, 2))
            dy = rnd(dy)
        else:
            dy, dg, db = gn_bwd(dacts[li], caches[li], P[d["g"]:d["g"] + d["cout"]], groups, slope)
            dy = rnd(dy)
            grads[d["g"]:d["g"] + d["cout"]] = dg
            grads[d["b"]:d["b"] + d["cout"]] = db
        xin = ins[li]
        if d["kind"] == "convt":
            gw = conv_wgrad(dy, xin, d["k"], d["s"], d["p"])
            dx = conv_fwd(dy, w, d["s"], d["p"])
        else:
            gw = conv_wgrad(xin, dy, d["k"], d["s"], d["p"])
            dx = conv_dgrad(dy, w, d["s"], d["p"], xin.shape)
        grads[d["w"]:d["w"] + gw.size] = gw.ravel()
        if d["in0"] >= 0:
            if d["in1"] < 0:
                dacts[d["in0"]] += dx
            else:
                c0 = dacts[d["in0"]].shape[3]
                dacts[d["in0"]] += dx[..., :c0]
                dacts[d["in1"]] += dx[..., c0:]
    return loss, grads, out


def init_params(n, levels, base, seed=1):
    """He-normal weights (any seeded draw; the GPU network's own init is not reproduced)."""
    L, npar = build(n, levels, base)
    g = np.random.default_rng(seed)
    p = np.zeros(npar)
    for d in L:
        cnt = int(np.prod(d["wshape"]))
        fan = d["cin"] if d["kind"] == "convt" else d["k"] * d["k"] * d["wshape"][3]
        sd = np.sqrt((1.0 if d["kind"] == "head" else 2.0) / fan)
        p[d["w"]:d["w"] + cnt] = g.normal(0, sd, cnt)
        if d["kind"] != "head":
            p[d["g"]:d["g"] + d["cout"]] = 1.0 + 0.1 * g.standard_normal(d["cout"])
            p[d["b"]:d["b"] + d["cout"]] = 0.1 * g.standard_normal(d["cout"])
        else:
            p[d["bias"]:d["bias"] + 4] = 0.1 * g.standard_normal(4)
    return p
