"""Self-checking dense GEMM workload for the tcgen05 kernel (cdx_gemm_bf16_tc), e.g.

    python -m cdixx_gb300.gemm_profile --m 16384 --n 128 --k 4096

Times D = A B^T with CUDA events and checks it against an FP32 product.
"""
from __future__ import annotations

import argparse
import ctypes
import sys


def main(argv=None):
    import torch
    from cdixx_gb300 import native as cdx
    ap = argparse.ArgumentParser()
    ap.add_argument("--m", type=int, default=16384)
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--k", type=int, default=4096)
    ap.add_argument("--reps", type=int, default=10)
    a = ap.parse_args(argv)
    g = torch.Generator(device="cuda").manual_seed(1)
    A = torch.randn(a.m, a.k, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(a.n, a.k, device="cuda", generator=g).to(torch.bfloat16)
    D = torch.empty(a.m, a.n, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    args = [ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(B.data_ptr()), ctypes.c_void_p(D.data_ptr()),
            a.m, a.n, a.k, ctypes.c_void_p(err.data_ptr()), None]
    cdx.check(cdx.lib().cdx_gemm_bf16_tc(*args))
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(a.reps):
        cdx.lib().cdx_gemm_bf16_tc(*args)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / a.reps
    ref = A.float() @ B.float().T
    rel = (torch.linalg.vector_norm(D - ref) / torch.linalg.vector_norm(ref)).item()
    tf = 2.0 * a.m * a.n * a.k / (ms / 1000) / 1e12
    ok = rel < 1e-5 and int(err.item()) == 0
    print(f"gemm {a.m}x{a.n}x{a.k}: {ms * 1000:.1f} us, {tf:.1f} TFLOP/s, rel L2 {rel:.2e}, ok={ok}")
    return 0 if ok else 1


if __name__ == "__main__":
    sys.exit(main())
