"""Small, self-checking workload for kernel captures (ncu -k / -c).

Runs a few fused iterations of one synthetic pattern through the C ABI and
exits non-zero when the result is not finite, e.g.

    python -m cdixx_gb300.profile_case --n 2048 --iters 3 --algo RAAR

Graph capture is off so every kernel is a plain stream launch: after the
set-up launches, each iteration is one column pass and one row pass
(col_pass_kernel, row_pass_kernel), plus the final FFT, norm and
reductions of the run.
"""
from __future__ import annotations

import argparse
import sys

import numpy as np

from cdixx_gb300 import native as cdx


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=2048)
    ap.add_argument("--batch", type=int, default=1)
    ap.add_argument("--iters", type=int, default=3)
    ap.add_argument("--algo", default="RAAR")
    ap.add_argument("--fft-mode", type=int, default=cdx.FFT_FP32)
    ap.add_argument("--repeat", type=int, default=2)
    a = ap.parse_args(argv)
    rng = np.random.default_rng(0)
    I = (rng.random((a.n, a.n)) * 100).astype(np.float32)
    psi0 = (np.sqrt(I) * np.where(rng.random((a.n, a.n)) > 0.5, -1, 1)).astype(np.complex64)
    p = cdx.default_params(a.n, a.n, batch=a.batch, oversampling_spt=4.0, beta=0.9, use_graph=0,
                           fft_mode=a.fft_mode)
    with cdx.Context(p) as ctx:
        for b in range(a.batch):
            ctx.set_pattern(b, I)
            ctx.set_initial(b, psi0)
        for _ in range(a.repeat):
            s = ctx.run(f"{a.iters}*{a.algo}")
        rho = ctx.get_object(0)
    ok = bool(np.isfinite(rho).all()) and np.isfinite(s["residual"])
    print(f"n={a.n} batch={a.batch} {a.iters}*{a.algo}: {s['gpu_ms'] / a.iters * 1000:.1f} us/iter, "
          f"launches {s['launches']}, finite={ok}")
    return 0 if ok else 1


if __name__ == "__main__":
    sys.exit(main())
