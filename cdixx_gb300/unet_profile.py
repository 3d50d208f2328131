"""Small self-checking U-Net training workload for kernel captures, e.g.

    python -m cdixx_gb300.unet_profile --n 256 --batch 16 --steps 3

Trains the warm-start network for a few Adam steps on forward-model batches
and exits non-zero when the loss is not finite.  Prints the mean time of a
training step (forward, loss, backward, Adam) measured with CUDA events.
"""
from __future__ import annotations

import argparse
import sys

import numpy as np


def main(argv=None):
    import torch
    from cdixx_gb300 import unet
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--levels", type=int, default=4)
    ap.add_argument("--base", type=int, default=32)
    ap.add_argument("--umma", type=int, default=0, help="1: tcgen05 convolutions, 0: mma.sync")
    a = ap.parse_args(argv)
    net = unet.UNet(n=a.n, levels=a.levels, base=a.base, batch=a.batch, seed=1, umma=a.umma)
    I, amp, ph, sup = unet.forward_model(a.n, a.batch, 7, 0, 1e6)
    net.train_step(I, amp, ph, sup)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    losses = [net.train_step(I, amp, ph, sup) for _ in range(a.steps)]
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / a.steps
    ok = bool(np.isfinite(losses).all())
    print(f"n={a.n} batch={a.batch} levels={a.levels} base={a.base} umma={a.umma}: {ms:.2f} ms/step, "
          f"loss {losses[-1]:.5f}, "
          f"finite={ok}")
    net.close()
    return 0 if ok else 1


if __name__ == "__main__":
    sys.exit(main())
