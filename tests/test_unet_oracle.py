"""CPU checks of the FP64 U-Net oracle: its analytic backward against central
finite differences (the oracle the GPU gradients are then held to)."""
import numpy as np

from cdixx_gb300 import synth
from oracle import unet_oracle as U


def small_case(n=16, batch=2, seed=3):
    I, amp, ph, sup = [], [], [], []
    for b in range(batch):
        obj, disk = synth.blob_object(n, seed, b, disk_frac=0.5, sig=(1.0, 2.0))
        I.append(synth.pattern_from_object(obj, 1e5, seed, b))
        a = np.abs(obj)
        amp.append(a)
        ph.append(np.angle(obj) + 0.3 * disk)
        sup.append((a > 0.02).astype(float))
    return np.array(I), np.array(amp), np.array(ph), np.array(sup)


def test_layer_list_and_parameter_count():
    L, npar = U.build(256, 4, 32)
    assert [d["kind"] for d in L].count("convt") == 3 and L[-1]["kind"] == "head"
    assert L[-2]["out_h"] == 256 and L[7]["out_h"] == 32
    assert 1_500_000 < npar < 2_500_000


def test_backward_matches_finite_differences():
    n, levels, base = 16, 2, 8
    I, amp, ph, sup = small_case(n)
    p = U.init_params(n, levels, base, seed=5)
    loss, g, _ = U.forward_backward(p, I, amp, ph, sup, n, levels, base)
    rng = np.random.default_rng(0)
    L, npar = U.build(n, levels, base)
    idx = rng.choice(npar, 40, replace=False)
    h = 1e-6
    for i in idx:
        q = p.copy()
        q[i] += h
        lp = U.forward_backward(q, I, amp, ph, sup, n, levels, base, backward=False)[0]
        q[i] -= 2 * h
        lm = U.forward_backward(q, I, amp, ph, sup, n, levels, base, backward=False)[0]
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(fd), (i, fd, g[i])
