"""GPU tests of the warm-start U-Net and the GPU forward model.

Tolerances.  The network computes with BF16 operands and FP32 accumulation.
Against the oracle run with the same BF16 roundings (oracle/unet_oracle.py,
round_bf16=True): output within relative L2 5e-3, loss within 2e-3, whole
gradient within relative L2 3e-2 and each layer's weight gradient within
0.1 -- differences left are accumulation order and BF16 ties flipped by it
(largest on the tiny one-channel-per-group network).
Against the plain FP64 oracle (the precision the BF16 path gives): whole
gradient within relative L2 0.1, cosine >= 0.995.
"""
import numpy as np
import pytest

from cdixx_gb300 import synth
from oracle import fwdmodel_oracle as FM
from oracle import unet_oracle as U

pytestmark = pytest.mark.gpu


def small_case(n, batch, seed=3):
    I, amp, ph, sup = [], [], [], []
    for b in range(batch):
        obj, disk = synth.blob_object(n, seed, b, disk_frac=0.5, sig=(1.0, 2.0 + n / 16))
        I.append(synth.pattern_from_object(obj, 1e5, seed, b))
        a = np.abs(obj)
        amp.append(a)
        ph.append(0.4 * disk * np.cos(np.arange(n) / 3.0)[None, :])
        sup.append((a > 0.02).astype(float))
    return [np.array(x, np.float32) for x in (I, amp, ph, sup)]


@pytest.mark.parametrize("n,levels,base", [(16, 2, 8), (32, 3, 16), (64, 4, 16)])
def test_gradients_match_fp64_oracle(cdx, torch_cuda, n, levels, base):
    torch = torch_cuda
    from cdixx_gb300 import unet
    batch = 2
    I, amp, ph, sup = small_case(n, batch)
    p = U.init_params(n, levels, base, seed=7)
    loss_64, g_64, out_64 = U.forward_backward(p, I, amp, ph, sup, n, levels, base)
    loss_ref, g_ref, out_ref = U.forward_backward(p, I, amp, ph, sup, n, levels, base, round_bf16=True)
    with unet.UNet(n=n, levels=levels, base=base, batch=batch, groups=8) as net:
        assert net.n_params == p.size
        net.set_params(p)
        dev = [torch.from_numpy(x).cuda() for x in (I, amp, ph, sup)]
        out = net.forward(dev[0]).cpu().numpy().transpose(0, 2, 3, 1)
        loss = net.loss_backward(*dev)
        g = net.grads().astype(np.float64)

    def rel(a, b):
        return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)

    cos = g @ g_64 / (np.linalg.norm(g) * np.linalg.norm(g_64))
    print(f"n={n} levels={levels}: vs BF16-rounded oracle: output {rel(out, out_ref):.2e}, "
          f"loss {abs(loss - loss_ref) / loss_ref:.2e}, grad {rel(g, g_ref):.3e}; "
          f"vs FP64: grad {rel(g, g_64):.3e}, cosine {cos:.5f}; BF16 oracle vs FP64 grad {rel(g_ref, g_64):.3e}")
    assert rel(out, out_ref) < 5e-3
    assert abs(loss - loss_ref) <= 2e-3 * abs(loss_ref)
    assert rel(g, g_ref) < 3e-2
    assert rel(g, g_64) < 0.1 and cos > 0.995
    L, _ = U.build(n, levels, base)
    for d in L:
        sl = slice(d["w"], d["w"] + int(np.prod(d["wshape"])))
        assert rel(g[sl], g_ref[sl]) < 0.1, (d["kind"], d["wshape"], rel(g[sl], g_ref[sl]))


def test_forward_model_matches_restatement(cdx, torch_cuda):
    from cdixx_gb300 import unet
    n, count, seed, first = 64, 3, 11, 5
    I, a, p, s = unet.forward_model(n, count, seed, first, photons=1e7)
    a, s, I = a.cpu().numpy(), s.cpu().numpy(), I.cpu().numpy().astype(np.float64)
    for b in range(count):
        v, sup = FM.render(n, seed, first + b)
        assert np.max(np.abs(a[b] - v)) <= 1e-6 * max(v.max(), 1.0)
        assert np.mean(s[b] != sup) < 1e-3
        lam = FM.expected_intensity(n, seed, first + b, 1e7)
        # Poisson: counts are integers; total and per-pixel deviations as the distribution says
        assert np.all(I[b] == np.round(I[b])) and I[b].min() >= 0
        assert abs(I[b].sum() - 1e7) < 5 * np.sqrt(1e7)
        z = (I[b] - lam) / np.sqrt(np.maximum(lam, 1e-12))
        big = lam > 20
        assert abs(z[big].mean()) < 0.1 and 0.85 < z[big].std() < 1.15
    # the same pattern index gives the same pattern in another batch
    I2, a2, _, _ = unet.forward_model(n, 1, seed, first + 1, photons=1e7)
    assert np.array_equal(I2.cpu().numpy()[0], I[1].astype(np.float32))


def test_training_reduces_loss(cdx, torch_cuda):
    from cdixx_gb300 import unet
    with unet.UNet(n=64, levels=3, base=16, batch=16, seed=3) as net:
        losses = unet.train(net, 80, seed=99, photons=1e6, lr=2e-3)
    first, last = np.mean(losses[:5]), np.mean(losses[-5:])
    print(f"loss {first:.4f} -> {last:.4f}")
    assert np.isfinite(losses).all() and last < 0.6 * first


def test_unet_errors(cdx, torch_cuda):
    from cdixx_gb300 import unet
    with pytest.raises(cdx.CdxError):
        unet.UNet(n=100, levels=4, base=32, batch=2)
    with pytest.raises(cdx.CdxError):
        unet.UNet(n=64, levels=3, base=12, batch=2)
    with unet.UNet(n=32, levels=2, base=8, batch=2) as net:
        torch = torch_cuda
        x = torch.zeros((3, 32, 32), device="cuda")
        with pytest.raises(cdx.CdxError):
            net.forward(x)


def _reach(cdx, I, truth, n, count, psi, sup, alg, target):
    from cdixx_gb300 import metrics
    prm = cdx.default_params(n, n, batch=count, beta=0.9, shrink_threshold=0.1, oversampling_spt=2.0, rf_every=10,
                             stop_rfactor=target)
    with cdx.Context(prm) as ctx:
        for i in range(count):
            ctx.set_pattern(i, I[i])
        if psi is None:
            ctx.random_start(12345)
        else:
            for i in range(count):
                ctx.set_initial(i, psi[i])
                ctx.set_support(i, sup[i])
        ctx.run(alg)
        conv = np.array([ctx.stats(i)["converged_iter"] for i in range(count)])
        err = np.array([metrics.error_vs_truth(ctx.get_object(i), truth[i]) for i in range(count)])
    return (conv >= 0).mean(), np.median(err)


def test_warm_start_from_truth_is_a_fixed_point_of_er(cdx, torch_cuda):
    """The warm-start plumbing: the true object given as network output gives
    Psi0 = FFT(rho_true) scaled to sqrt(I) and the true support, from which ER
    stays at the truth (noise-free pattern)."""
    torch = torch_cuda
    from cdixx_gb300 import unet
    n, count = 128, 4
    I, a, p, s = unet.forward_model(n, count, 31, 0, -1e6)
    o = torch.zeros((count, 4, n, n), device="cuda")
    o[:, 0] = a
    o[:, 1] = 1.0
    o[:, 3] = torch.where(s > 0, 10.0, -10.0)
    with unet.UNet(n=n, levels=3, base=8, batch=count) as net:
        psi, sup = net.warm_start(I, o, 0)
    assert torch.equal(sup, s)
    frac, err = _reach(cdx, I, a.cpu().numpy(), n, count, psi, sup, "20*ER", 2e-3)
    print(f"truth start: reached {frac:.2f}, error {err:.2e}")
    assert frac == 1.0 and err < 2e-3


def test_warm_start_gain_over_random_phase_hio(cdx, torch_cuda):
    """A U-Net trained here on forward-model pairs (128^2, noise-free held-out
    patterns): HIO/ER from its warm start (Psi0 and support, support fixed)
    reaches R <= 0.02 on more patterns, and a lower error against the true
    object, than the reference's path (random phase, rect support, shrinkwrap
    every 20) in the same 1000 iterations."""
    from cdixx_gb300 import unet
    n, count = 128, 32
    with unet.UNet(n=n, levels=3, base=16, batch=32, seed=2) as net:
        losses = unet.train(net, 600, seed=4242, photons=1e6, lr=2e-3)
        I, a, p, s = unet.forward_model(n, count, 777, 0, -1e6)
        out = net.forward(I)
        psi_w, sup_w = net.warm_start(I, out, 3)
    truth = a.cpu().numpy()
    sw = "+".join(["20*HIO+1*shrinkWrap"] * 9) + "+20*ER+1*shrinkWrap"
    f0, e0 = _reach(cdx, I, truth, n, count, None, None, f"5*({sw})", 2e-2)
    f1, e1 = _reach(cdx, I, truth, n, count, psi_w, sup_w, "5*(180*HIO+20*ER)", 2e-2)
    print(f"loss {losses[0]:.4f} -> {np.mean(losses[-10:]):.4f}; reached R<=0.02: random {f0:.2f} (error {e0:.3f}), "
          f"warm {f1:.2f} (error {e1:.3f})")
    assert f1 >= f0 + 0.25 and e1 < e0


def test_tcgen05_and_mma_sync_convolutions_agree(cdx, torch_cuda):
    """The forward and data-gradient convolutions on tcgen05/TMEM and on
    mma.sync (default) give the same network output and gradients (measured:
    the same bits -- both add exact BF16 products in 16-term chunks in the
    same K order; the bound allows FP32 accumulation-order differences)."""
    torch = torch_cuda
    from cdixx_gb300 import unet
    n, levels, base, batch = 64, 3, 16, 2
    I, amp, ph, sup = small_case(n, batch)
    p = U.init_params(n, levels, base, seed=9)
    dev = [torch.from_numpy(x).cuda() for x in (I, amp, ph, sup)]
    res = []
    for mode in (1, 0):
        with unet.UNet(n=n, levels=levels, base=base, batch=batch, groups=8, umma=mode) as net:
            net.set_params(p)
            out = net.forward(dev[0]).cpu().numpy()
            loss = net.loss_backward(*dev)
            res.append((out, loss, net.grads().astype(np.float64)))
    (o1, l1, g1), (o0, l0, g0) = res
    ro = np.linalg.norm(o1 - o0) / np.linalg.norm(o0)
    rg = np.linalg.norm(g1 - g0) / np.linalg.norm(g0)
    print(f"tcgen05 vs mma.sync: output {ro:.2e}, loss {abs(l1 - l0) / l0:.2e}, gradient {rg:.2e}")
    assert ro < 5e-3 and abs(l1 - l0) <= 2e-3 * l0 and rg < 3e-2


def test_training_needs_no_host_synchronisation(cdx, torch_cuda):
    """The forward model queues its batch on the caller's stream and returns;
    the network's own stream waits for it.  Training with no host sync must
    give the same losses, bit for bit, as training with a device sync after
    every generated batch (every kernel here is deterministic)."""
    torch = torch_cuda
    from cdixx_gb300 import unet
    runs = []
    for sync in (False, True):
        with unet.UNet(n=64, levels=3, base=16, batch=16, seed=9) as net:
            losses = []
            for k in range(25):
                I, a, p, s = unet.forward_model(64, 16, 4321, k * 16, 1e6)
                if sync:
                    torch.cuda.synchronize()
                losses.append(net.train_step(I, a, p, s, 2e-3))
            runs.append(losses)
    assert np.all(np.isfinite(runs[0]))
    assert runs[0] == runs[1]
