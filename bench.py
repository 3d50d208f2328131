"""Benchmark of the CDI phase-retrieval path on one GB300.

Workload (the large single-pattern configuration): one 2048x2048 complex64
pattern of a phase object (amplitude U[0.5,1], phase in [0,pi] from smoothed
noise, 512-px support with a random smooth boundary), Poisson noise at 1e9
photons; RAAR beta = 0.9 with a shrinkwrap every 50 iterations.  One bench
step = one shrinkwrap period (50 RAAR iterations + 1 shrinkwrap) of that
pattern; the full job (2000 iterations) is 40 steps.

  value    iterations/s with the pattern already resident in HBM (cdx_run_async
           on device buffers; L2 flushed between steps, each step timed with
           CUDA events on the context's stream)
  e2e      iterations/s of the whole 2000-iteration job through the host-buffer
           C-ABI call cdx_phase_retrieve_host (H2D of I and Psi0, D2H of rho, Psi
           and the support inside the timed region)
  roofline algorithmic bytes of one fused iteration (21 B/px: read rho 8 + I 4 +
           support 1, write rho 8) / the measured duration of one iteration (its
           column + row pass), against the measured HBM copy bandwidth.

  warm_start  the learned warm start: a U-Net trained here (one pass over 50k
           forward-model seeds, batch 64) against the plain random-phase path on
           1024 held-out 256^2 patterns, patterns/s reaching R <= 0.02
  batched  512 patterns of uneven sizes {128..512}^2, HIO/ER 500 each, one
           CUDA graph: patterns/s

`--impl reference` times the CPU restatement of the reference path (the
oracle, float32, multi-threaded scipy FFT) on a bounded sample of the same
workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N = 2048
PHOTONS = 1e9
SEED = 20260101
BETA = 0.9
SW_EVERY = 50
STEP_ALGO = f"{SW_EVERY}*RAAR+1*shrinkWrap"
JOB_ALGO = f"40*({SW_EVERY}*RAAR+1*shrinkWrap)"
JOB_ITERS = 40 * SW_EVERY
ALG_BYTES_PER_PX_ITER = 21.0
METRIC = "iter/s"
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one 2048^2 iteration,
# col_pass_rk<2048> + row_pass_rk<2048>, from one `ncu --set full` capture of
# `python bench.py case pass --n 2048 --iters 3` (-k regex:pass_rk -s 3 -c 2):
# 50.41 + 0.05 + 67.68 + 11.77 MB, cold caches
PASS_TRAFFIC_2048 = 129_913_000
WORKLOAD = "2048x2048 complex64 phase object, 1e9 photons, RAAR beta=0.9, shrinkwrap every 50"


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu=0):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_inputs():
    from cdixx_gb300 import synth
    obj, sup, I = synth.config1_case(seed=SEED, n=N, photons=PHOTONS)
    psi0 = synth.random_phase_start(I, SEED)
    return I, psi0


def cpu_sample(I, psi0, iters, threads):
    """Oracle (float32 CPU restatement) on `iters` RAAR iterations: iterations/s."""
    from oracle import cdi_oracle as O
    O.set_fft_workers(threads)
    t0 = time.perf_counter()
    O.phase_retrieve(psi0, I, f"{iters}*RAAR", oversampling_spt=4.0, beta=BETA, shrink_threshold=0.1,
                     dtype=np.complex64)
    dt = time.perf_counter() - t0
    return iters / dt, dt


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    I, psi0 = make_inputs()
    threads = os.cpu_count() or 1
    iters = 2
    cpu_sample(I, psi0, 1, threads)   # warm the FFT plans
    vals = []
    t_all = 0.0
    for _ in range(args.warmup):
        cpu_sample(I, psi0, iters, threads)
    for _ in range(args.steps):
        v, dt = cpu_sample(I, psi0, iters, threads)
        vals.append(v)
        t_all += dt
    v = float(np.median(vals))
    line = {
        "metric": METRIC, "value": v, "unit": "iter/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000 * t_all / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "impl": "reference",
        "config": {"workload": WORKLOAD, "sample": f"{iters} RAAR iterations per step"},
        "cpu_baseline": {"value": v, "unit": "iter/s", "cores": threads, "kind": "port",
                         "sample": f"{iters} RAAR iterations of the 2048^2 pattern per step, float32 oracle, "
                                   f"scipy.fft with {threads} workers"},
        "e2e": {"value": v, "unit": "iter/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------------------
# Learned warm start (configs 3 and 4).  Both arms run the same schedule -- the
# plain CDI configuration's HIO beta 0.9 x180 then ER x20 with a shrinkwrap
# every 20 iterations, to 2000 iterations -- and differ only in the start: the
# plain arm from a binary random phase and the rect support, the learned arm
# from the network's Psi0 and support (refreshed by the same shrinkwraps).  The
# in-loop R-factor is checked every RF_EVERY iterations; a pattern stops by
#   literal  R <= 1e-3 (the stated target; below the Poisson floor of these
#            photon counts, so it measures the full 2000-iteration cost),
#   floor    R <= 1.01 x its Poisson floor (the R-factor of the true object
#            against the noisy pattern, from the forward model's noise-free
#            intensity),
#   plateau  its lowest R-factor has not fallen by 1 % for 400 iterations.
# patterns/s = patterns that stopped / GPU seconds of the arm (network forward
# and warm start included); the error against the true object is reported for
# every arm and criterion as the equal-error evidence.
WARM_N, WARM_BATCH, WARM_TRAIN_SEEDS, WARM_EVAL = 256, 64, 50_000, 1024
WARM_PHOTONS = 1e6
NET_512_BATCH, NET_512_SEEDS = 16, 12_800
EVAL_ALGO = "10*(" + "+".join(["20*HIO+1*shrinkWrap"] * 9) + "+20*ER+1*shrinkWrap)"
EVAL_ITERS = 2000
RF_EVERY = 10
WARM_DILATE = 3
CRITERIA = {
    "literal": dict(stop_rfactor=1e-3),
    "floor": dict(floor_factor=1.01),
    "plateau": dict(plateau_iters=400, plateau_tol=0.01),
}
COMBINED_SIZES = (256, 512)
COMBINED_PATTERNS = 4096


def train_network(n, batch, seeds, photons, seed):
    """A U-Net of 4 levels and 32 base channels trained by the library's own
    kernels on fresh forward-model pairs (Adam 1e-3): (network, summary)."""
    import torch
    from cdixx_gb300 import unet
    net = unet.UNet(n=n, levels=4, base=32, batch=batch, seed=seed)
    steps = seeds // batch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    losses = unet.train(net, steps, seed=seed, photons=photons, lr=1e-3)
    torch.cuda.synchronize()
    return net, {"n": n, "seeds": steps * batch, "batch": batch, "photons": photons, "lr": 1e-3,
                 "seconds": time.perf_counter() - t0, "loss_first": losses[0],
                 "loss_last": float(np.mean(losses[-20:]))}


def eval_set(n, photons, seed, first=0):
    """Held-out patterns of side n, one photon count each: intensity [b, n, n]
    (FFT order), the true object [b, n, n] (centred, complex) and each
    pattern's Poisson floor R = sum|sqrt(lambda) - sqrt(I)| / sum sqrt(I)."""
    import torch
    from cdixx_gb300 import unet
    b = len(photons)
    I = torch.empty((b, n, n), dtype=torch.float32, device="cuda")
    lam = torch.empty_like(I)
    truth = torch.empty((b, n, n), dtype=torch.complex64, device="cuda")
    for i, ph in enumerate(photons):
        Ii, a, p, _ = unet.forward_model(n, 1, seed, first + i, float(ph))
        Li, _, _, _ = unet.forward_model(n, 1, seed, first + i, -float(ph))
        I[i], lam[i] = Ii[0], Li[0]
        truth[i] = torch.polar(a[0], p[0])
    sI, sL = torch.sqrt(torch.clamp(I, min=0)), torch.sqrt(torch.clamp(lam, min=0))
    floor = ((sI - sL).abs().sum(dim=(1, 2)) / sI.sum(dim=(1, 2))).double().cpu().numpy()
    return I, truth, floor


def warm_starts(net, I, truth=None):
    """Network forward + warm start in chunks of the network's batch: (Psi0,
    support, GPU seconds by CUDA events[, median error against the truth of the
    network's own object a e^{i atan2(s, c)} on sigmoid(logit) > 0.5])."""
    import torch
    from cdixx_gb300 import metrics
    b, n = I.shape[0], I.shape[1]
    psi = torch.empty((b, n, n), dtype=torch.complex64, device="cuda")
    sup = torch.empty((b, n, n), dtype=torch.float32, device="cuda")
    obj = torch.empty((b, n, n), dtype=torch.complex64, device="cuda")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    B = net.cfg.batch
    outs = []
    e0.record()
    for s in range(0, b, B):
        out = net.forward(I[s:s + B])
        p, q = net.warm_start(I[s:s + B], out, WARM_DILATE)
        psi[s:s + B], sup[s:s + B] = p, q
        outs.append(out)
    e1.record()
    torch.cuda.synchronize()
    secs = e0.elapsed_time(e1) / 1000.0
    if truth is None:
        return psi, sup, secs
    for k, out in enumerate(outs):
        a, c, si, lg = out[:, 0], out[:, 1], out[:, 2], out[:, 3]
        obj[k * B:k * B + out.shape[0]] = torch.polar(a, torch.atan2(si, c)) * (lg > 0)
    return psi, sup, secs, float(np.median(metrics.error_vs_truth_batch(obj, truth)))


def run_arm(sets, starts, crit, fft_mode, seed):
    """One arm under one stop criterion over every size in `sets` ({n: (I,
    truth, floor)}), all sizes one CUDA graph (cdx_group).  `starts`: {n: (Psi0,
    support, net seconds)} for the learned arm, None for the plain arm."""
    import torch
    from cdixx_gb300 import metrics
    from cdixx_gb300 import native as cdx
    c = CRITERIA[crit]
    ctxs = []
    for n, (I, truth, floor) in sets.items():
        prm = cdx.default_params(n, n, batch=I.shape[0], beta=0.9, shrink_threshold=0.1, oversampling_spt=4.0,
                                 rf_every=RF_EVERY, fft_mode=fft_mode, stop_rfactor=c.get("stop_rfactor", 0.0),
                                 plateau_iters=c.get("plateau_iters", 0), plateau_tol=c.get("plateau_tol", 0.01))
        ctx = cdx.Context(prm)
        for i in range(I.shape[0]):
            ctx.set_pattern(i, I[i])
        if starts is None:
            ctx.random_start(seed + n)
        else:
            psi, sup, _ = starts[n]
            for i in range(I.shape[0]):
                ctx.set_initial(i, psi[i])
                ctx.set_support(i, sup[i])
        if "floor_factor" in c:
            for i in range(I.shape[0]):
                ctx.set_stop_rfactor(i, c["floor_factor"] * floor[i])
        ctxs.append(ctx)
    g = cdx.Group(ctxs)
    ms = g.run(EVAL_ALGO)
    conv, err, ratio = [], [], []
    for ctx, (n, (I, truth, floor)) in zip(ctxs, sets.items()):
        rho = torch.empty((I.shape[0], n, n), dtype=torch.complex64, device="cuda")
        for i in range(I.shape[0]):
            st = ctx.stats(i)
            conv.append(st["converged_iter"])
            ratio.append(st["rfactor_min"] / floor[i])
            ctx.get_object(i, out=rho[i])
        err.append(metrics.error_vs_truth_batch(rho, truth))
    g.close()
    for ctx in ctxs:
        ctx.close()
    conv, err, ratio = np.array(conv), np.concatenate(err), np.array(ratio)
    net_s = sum(v[2] for v in starts.values()) if starts else 0.0
    secs = ms / 1000.0 + net_s
    done = conv >= 0
    return {"patterns_per_s": float(done.sum() / secs), "reached": float(done.mean()),
            "median_iterations": float(np.median(conv[done])) if done.any() else None,
            "gpu_s": secs, "net_s": net_s,
            "median_error_vs_truth": float(np.median(err)),
            "median_error_vs_truth_reached": float(np.median(err[done])) if done.any() else None,
            "median_rmin_over_floor": float(np.median(ratio))}


def compare(arms, base="plain", learned="learned"):
    out = {}
    for crit in CRITERIA:
        pp = arms[base][crit]["patterns_per_s"]
        lp = arms[learned][crit]["patterns_per_s"]
        out[crit] = {"speedup": lp / pp if pp > 0 else None,
                     "median_error_vs_truth": {k: arms[k][crit]["median_error_vs_truth"] for k in arms}}
    return out


def warm_start_section(net):
    """Config 3: the 256^2 network (trained at 1e6 photons) against random-phase
    HIO on 1024 held-out seeds at 1e6 photons, FP32 iteration in both arms."""
    from cdixx_gb300 import native as cdx
    I, truth, floor = eval_set(WARM_N, [WARM_PHOTONS] * WARM_EVAL, SEED + 1)
    sets = {WARM_N: (I, truth, floor)}
    psi, sup, net_s, net_err = warm_starts(net, I, truth)
    arms = {"plain": {}, "learned": {}}
    for crit in CRITERIA:
        arms["plain"][crit] = run_arm(sets, None, crit, cdx.FFT_FP32, SEED)
        arms["learned"][crit] = run_arm(sets, {WARM_N: (psi, sup, net_s)}, crit, cdx.FFT_FP32, SEED)
    return {"metric": "patterns/s to the stop criterion (learned warm start vs random-phase HIO)",
            "patterns": WARM_EVAL, "n": WARM_N, "photons": WARM_PHOTONS,
            "data": "held-out forward-model seeds (8 blobs in a 64-px disk), Poisson noise",
            "algorithm": EVAL_ALGO, "rf_every": RF_EVERY, "criteria": CRITERIA,
            "median_poisson_floor": float(np.median(floor)), "network_alone_median_error_vs_truth": net_err,
            "arms": arms, "compare": compare(arms)}


def combined_section(nets):
    """Config 4: 4096 patterns, 256^2 and 512^2 mixed 3:1, photons log-uniform
    1e5..1e8; learned warm start + tensor-core FFT against the plain fused FP32
    path (and learned + FP32), every size one CUDA graph per run."""
    from cdixx_gb300 import native as cdx
    rng = np.random.default_rng(SEED + 4)
    counts = {256: COMBINED_PATTERNS * 3 // 4, 512: COMBINED_PATTERNS // 4}
    sets, starts, net_err = {}, {}, {}
    for k, n in enumerate(COMBINED_SIZES):
        photons = 10 ** rng.uniform(5, 8, counts[n])
        sets[n] = eval_set(n, photons, SEED + 40 + k)
        *starts[n], net_err[str(n)] = warm_starts(nets[n], sets[n][0], sets[n][1])
    arms = {"plain": {}, "learned_tc": {}, "learned": {}}
    for crit in CRITERIA:
        arms["plain"][crit] = run_arm(sets, None, crit, cdx.FFT_FP32, SEED)
        arms["learned_tc"][crit] = run_arm(sets, starts, crit, cdx.FFT_TC_BF16, SEED)
        arms["learned"][crit] = run_arm(sets, starts, crit, cdx.FFT_FP32, SEED)
    floors = np.concatenate([v[2] for v in sets.values()])
    return {"metric": "patterns/s to the stop criterion (learned + TC-FFT vs plain FP32 HIO)",
            "patterns": COMBINED_PATTERNS, "sizes": {str(n): counts[n] for n in COMBINED_SIZES},
            "photons": "log-uniform 1e5..1e8", "algorithm": EVAL_ALGO, "rf_every": RF_EVERY, "criteria": CRITERIA,
            "median_poisson_floor": float(np.median(floors)), "network_alone_median_error_vs_truth": net_err,
            "arms": arms,
            "compare": compare(arms, learned="learned_tc"), "compare_fp32": compare(arms, learned="learned"),
            "launch": "one CUDA graph per run (cdx_group), one branch per size"}


def northstar_sections():
    """Train the 256^2 and 512^2 networks, then configs 3 and 4."""
    net256, tr256 = train_network(WARM_N, WARM_BATCH, WARM_TRAIN_SEEDS, WARM_PHOTONS, SEED)
    net512, tr512 = train_network(512, NET_512_BATCH, NET_512_SEEDS, WARM_PHOTONS, SEED + 512)
    warm = warm_start_section(net256)
    warm["train"] = tr256
    comb = combined_section({256: net256, 512: net512})
    comb["train"] = {"256": tr256, "512": tr512}
    net256.close()
    net512.close()
    return warm, comb


BATCH_SIZES = (128, 192, 256, 384, 512)
BATCH_PATTERNS = 512
BATCH_ALGO = "500*HIO+500*ER"


def batched_section():
    """512 patterns of uneven sizes (uniform over BATCH_SIZES squared, photons
    log-uniform 1e5..1e8, blob objects in a support of 1/4 linear size), HIO and
    ER 500 iterations each, every size one context, all run as one CUDA graph.
    Each context first tunes its launch variant (autotune) and is timed alone,
    so the line shows the tuner's choice per size; the group's graph runs its
    branches one after another (the default) and, timed separately from the same
    start, side by side."""
    import torch
    from cdixx_gb300 import native as cdx
    from cdixx_gb300 import unet
    rng = np.random.default_rng(SEED)
    sizes = rng.choice(BATCH_SIZES, BATCH_PATTERNS)
    photons = 10 ** rng.uniform(5, 8, BATCH_PATTERNS)
    ctxs = []
    per_size = {}
    px = 0
    for n in BATCH_SIZES:
        idx = np.nonzero(sizes == n)[0]
        if len(idx) == 0:
            continue
        ctx = cdx.Context(cdx.default_params(int(n), int(n), batch=len(idx), beta=0.9, oversampling_spt=2.0,
                                             autotune=1))
        for j, p in enumerate(idx):
            I, _, _, _ = unet.forward_model(int(n), 1, SEED + 2, int(p), float(photons[p]))
            ctx.set_pattern(j, I[0])
        ctx.random_start(SEED + int(n))
        ctx.run("2*HIO")                  # tunes the launch variant on this context's data
        ctx.random_start(SEED + int(n))
        alone = ctx.run(BATCH_ALGO)["gpu_ms"]
        pdl, chunk, _ = ctx.tuning()
        per_size[str(n)] = {"patterns": int(len(idx)), "alone_ms": alone,
                            "tuned": {"pdl_col": int(pdl > 0 and pdl & 1), "pdl_row": int(pdl > 0 and pdl >> 1 & 1),
                                      "row_chunk_bits": chunk}}
        ctxs.append(ctx)
        px += len(idx) * int(n) * int(n)
    g = cdx.Group(ctxs)
    g.run("2*HIO")   # warm-up; the timed algorithm's graph is built inside the timed call,
    # but gpu_ms covers only its launch (events on the group's stream)
    for c in ctxs:
        c.random_start(SEED)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ms = g.run(BATCH_ALGO)
    wall = time.perf_counter() - t0
    # the same run with the branches side by side, from the same start
    g.set_concurrent(True)
    g.run("2*HIO")
    for c in ctxs:
        c.random_start(SEED)
    ms_side = g.run(BATCH_ALGO)
    g.close()
    for c in ctxs:
        c.close()
    iters = 1000
    sum_alone = float(sum(v["alone_ms"] for v in per_size.values()))
    return {"metric": "patterns/s", "patterns": BATCH_PATTERNS, "sizes": list(BATCH_SIZES),
            "algorithm": BATCH_ALGO, "patterns_per_s": BATCH_PATTERNS / (ms / 1000.0),
            "pixel_iterations_per_s": px * iters / (ms / 1000.0), "gpu_ms": ms, "wall_ms_incl_graph_build": wall * 1000,
            "contexts": len(ctxs), "per_size": per_size, "sizes_one_by_one_ms": sum_alone,
            "graph_gain_over_one_by_one": sum_alone / ms,
            "gpu_ms_branches_side_by_side": ms_side,
            "launch": "one CUDA graph (cdx_group) with one branch per size, one after another"}


# ---------------------------------------------------------------------------
# GPU comparator (bench only, not the product and not `--impl reference`): the
# reference's iteration structure on the same GPU -- cuFFT C2C and one
# element-wise kernel per operation (applyModAbs, IFFT, applyNorm,
# ApplyHIOSupport, FFT; cdi.cc:349-381) from _lib/libcdx_cufft_cmp.so --
# against the fused two-kernel HIO iteration, same pattern, same start.
CMP_ITERS = 50


def comparator_section():
    import ctypes
    import torch
    from cdixx_gb300 import native as cdx
    from cdixx_gb300 import synth
    lib = ctypes.CDLL(str(ROOT / "cdixx_gb300" / "_lib" / "libcdx_cufft_cmp.so"))
    lib.cmp_iterate.argtypes = [ctypes.c_int] * 4 + [ctypes.c_void_p] * 5 + [ctypes.c_float, ctypes.c_float,
                                                                              ctypes.c_void_p]
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    out = {"structure": "cuFFT C2C + applyModAbs + applyNorm + ApplyHIOSupport kernels (5 launches/iteration) vs "
                        "col_pass_rk + row_pass_rk (2 launches/iteration)", "algorithm": "HIO beta 0.9"}
    cases = [("2048x2048 x1", 2048, 1, lambda: make_inputs()),
             ("256x256 x64", 256, 64, None)]
    stream = torch.cuda.Stream()
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    for name, n, b, mk in cases:
        if mk is not None:
            I_np, psi_np = mk()
            I_np, psi_np = I_np[None], psi_np[None]
        else:
            I_np = np.stack([synth.config0_case(seed=SEED + i, n=n, photons=1e6)[2] for i in range(b)])
            psi_np = np.stack([synth.random_phase_start(I_np[i], SEED + i) for i in range(b)])
        prm = cdx.default_params(n, n, batch=b, oversampling_spt=4.0, beta=0.9)
        ctx = cdx.Context(prm, stream=stream.cuda_stream)
        for i in range(b):
            ctx.set_pattern(i, I_np[i])
            ctx.set_initial(i, psi_np[i])
        spt = torch.from_numpy(np.stack([ctx.get_support(i) for i in range(b)])).cuda()
        I = torch.from_numpy(I_np).cuda()
        psi = torch.from_numpy(psi_np).cuda()
        rho = torch.fft.ifft2(psi)                    # rho0 = IFFT(Psi0)/N
        rhop = torch.empty_like(rho)
        torch.cuda.synchronize()
        # agreement: 5 iterations from the same start
        rc = lib.cmp_iterate(n, n, b, 5, P(psi), P(rho), P(rhop), P(I), P(spt), 0.5, 0.9, stream.cuda_stream)
        if rc:
            raise RuntimeError(f"comparator failed: {rc}")
        ctx.run("5*HIO")
        torch.cuda.synchronize()
        a = rho[0].cpu().numpy() * np.float32(n)      # phaseRetrieve leaves rho scaled by sqrt(N)
        g = ctx.get_object(0)
        agree = float(np.linalg.norm(a - g) / np.linalg.norm(g))

        def timed(fn):
            vals = []
            for _ in range(5):
                with torch.cuda.stream(stream):
                    flush.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                fn()
                e1.record(stream)
                torch.cuda.synchronize()
                vals.append(e0.elapsed_time(e1) * 1000.0 / CMP_ITERS)
            return float(np.median(vals))

        us_cmp = timed(lambda: lib.cmp_iterate(n, n, b, CMP_ITERS, P(psi), P(rho), P(rhop), P(I), P(spt), 0.5, 0.9,
                                               stream.cuda_stream))
        us_fused = timed(lambda: ctx.run_async(f"{CMP_ITERS}*HIO"))
        ctx.close()
        out[name] = {"us_per_iteration_cufft_structure": us_cmp, "us_per_iteration_fused": us_fused,
                     "fused_speedup": us_cmp / us_fused, "rel_l2_after_5_iterations": agree,
                     "l2": "flushed (512 MB write) before each block of 50"}
    return out


def tc_section():
    """The large single-pattern configuration's two FFT paths, on the same pattern:
    the plain fused FP32 iteration (fft_mode 0) against the split-BF16 tensor-core
    FFT on tcgen05 (fft_mode 1) and on mma.sync (fft_mode 2).  Per mode: us per RAAR
    iteration (events, L2 flushed before each block of 50), the error of one 2-D
    FFT against the float64 DFT (numpy), and the error of one RAAR iteration from
    the same start against the FP32 path (longer runs diverge: RAAR amplifies any
    rounding difference)."""
    import torch
    from cdixx_gb300 import native as cdx
    I, psi0 = make_inputs()
    stream = torch.cuda.Stream()
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    rng = np.random.default_rng(SEED)
    x = (rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))).astype(np.complex64)
    ref = np.fft.fft2(x.astype(np.complex128))
    xt = torch.from_numpy(x).cuda()
    out = {"workload": WORKLOAD, "algorithm": f"{SW_EVERY}*RAAR per timed block", "modes": {}}
    rho_fp32 = None
    for mode, name in ((0, "fp32"), (1, "tc_bf16_tcgen05"), (2, "tc_bf16_mma_sync")):
        y = torch.empty_like(xt)
        cdx.fft2(xt, y, fft_mode=mode)
        torch.cuda.synchronize()
        fft_err = float(np.linalg.norm(y.cpu().numpy() - ref) / np.linalg.norm(ref))
        p = cdx.default_params(N, N, oversampling_spt=4.0, beta=BETA, fft_mode=mode)
        ctx = cdx.Context(p, stream=stream.cuda_stream)
        ctx.set_pattern(0, I)
        ctx.set_initial(0, psi0)
        ctx.run("1*RAAR")
        rho = ctx.get_object(0)
        if mode == 0:
            rho_fp32 = rho
        vals = []
        for _ in range(5):
            with torch.cuda.stream(stream):
                flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            ctx.run_async(f"{SW_EVERY}*RAAR")
            e1.record(stream)
            torch.cuda.synchronize()
            vals.append(e0.elapsed_time(e1) * 1000.0 / SW_EVERY)
        ctx.close()
        out["modes"][name] = {"us_per_iteration": float(np.median(vals)), "fft2_rel_l2_vs_fp64": fft_err,
                              "rho_rel_l2_vs_fp32_one_iteration": float(np.linalg.norm(rho - rho_fp32) /
                                                                   np.linalg.norm(rho_fp32))}
    f = out["modes"]["fp32"]["us_per_iteration"]
    for k in ("tc_bf16_tcgen05", "tc_bf16_mma_sync"):
        out["modes"][k]["time_vs_fp32"] = out["modes"][k]["us_per_iteration"] / f
    return out


# Ptychography: the reference's own configuration (html/default/ptycho.cfg optics,
# 512^2 probe, row_O = column_O = 1280, initScan_triangle with stepSize 250).
PTY_R, PTY_RO, PTY_STEP = 512, 1280, 250.0
PTY_OPTICS = dict(lam=0.6328, d=125e3, dpupil=6.8e3, pixelsize=13.0, pupil_size=335.0083, exposure=0.01,
                  zernike_iter=1200)
PTY_SWEEPS = 100


def ptycho_section(cpu=True):
    """rPIE + mPIE sweeps (ptycho::iterate, object phase with the FISTA object step of
    zernikeIter 1200) on the reference's configuration with noise-free simulated
    patterns of a smooth synthetic object: sweeps/s from CUDA events around
    cdx_pty_iterate, probe-phase sweep times (with and without the Zernike pupil
    fit), the roofline of a sweep and the oracle on one sweep as the CPU baseline."""
    from cdixx_gb300 import ptycho as PT
    sx, sy = PT.scan_triangle(PTY_RO, PTY_RO, PTY_R, PTY_R, PTY_STEP)
    t = PT.Ptycho(PTY_R, PTY_R, PTY_RO, PTY_RO, sx, sy, **PTY_OPTICS)
    x = np.linspace(-1, 1, PTY_RO, dtype=np.float32)[:, None]
    y = np.linspace(-1, 1, PTY_RO, dtype=np.float32)[None, :]
    truth = ((0.6 + 0.4 * np.cos(9 * x) * np.sin(7 * y)) * np.exp(1.2j * np.sin(5 * x + 3 * y))).astype(np.complex64)
    t.initObject(seed=SEED)
    obj0, probe0 = t.objectWave, t.probe
    t.objectWave = truth
    t.createPattern()
    t.objectWave = obj0
    t.iterate(3, seed=1)                      # warm-up (graph capture)
    t.objectWave = obj0
    t.probe = probe0
    ms = t.iterate(PTY_SWEEPS, seed=1)
    sweeps_s = PTY_SWEEPS / (ms / 1000.0)
    t.probe = probe0
    ms_probe = t.iterate(20, first_iter=400, seed=2)      # two of them with the Zernike pupil fit
    t.probe = probe0
    ms_zk = t.iterate(1, first_iter=400, seed=3)
    t.probe = probe0
    ms_nozk = t.iterate(1, first_iter=401, seed=3)
    n, on, ns = PTY_R * PTY_R, PTY_RO * PTY_RO, len(sx)
    # algorithmic bytes of a sweep: per position the object window read and written,
    # the probe and the pattern read (8 + 8 + 8 + 4 B/px); the FISTA step reads and
    # writes the object (16 B/px); the momentum step reads the object, its history and
    # the overlap mask and writes both (36 B/px of the object)
    alg = ns * 28 * n + (16 + 36) * on
    achieved = alg / (ms / PTY_SWEEPS / 1000.0) / 1e9
    peak, peak_kind = peaks()
    out = {"metric": "ptycho sweeps/s", "value": sweeps_s, "positions_per_s": sweeps_s * ns,
           "config": {"probe": PTY_R, "object": PTY_RO, "positions": ns, "scan": "initScan_triangle, stepSize 250",
                      "optics": PTY_OPTICS, "sweeps": PTY_SWEEPS, "mPIE": True,
                      "data": "noise-free patterns of a synthetic smooth object (createPattern)"},
           "ms_per_sweep": ms / PTY_SWEEPS, "ms_per_probe_phase_sweep": ms_probe / 20,
           "ms_zernike_sweep": ms_zk, "ms_probe_sweep_without_zernike": ms_nozk,
           "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                        "alg_bytes_per_sweep": alg, "peak_kind": peak_kind},
           "gpu_launches_per_sweep": 3 * ns + 5 + 0.1}   # + the probe momentum every tenth sweep
    if cpu:
        from oracle import ptycho_oracle as PO
        prm = PO.PtyParams(lam=PTY_OPTICS["lam"], d=PTY_OPTICS["d"], dpupil=PTY_OPTICS["dpupil"],
                           pixelsize=PTY_OPTICS["pixelsize"], pupil_size=PTY_OPTICS["pupil_size"],
                           exposure=PTY_OPTICS["exposure"], mpie=True, zernike_iter=PTY_OPTICS["zernike_iter"])
        pats = t.patterns
        orders = PO.scan_orders(ns, 1, 1)
        t0 = time.perf_counter()
        PO.iterate(obj0, probe0, pats, sx, sy, 1, prm, orders)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": 1.0 / dt, "unit": "sweeps/s", "cores": 1, "kind": "port",
                               "sample": f"1 sweep of the same case, NumPy oracle ({dt:.2f} s)"}
    t.close()
    return out


def replica_throughput(local_ms, local_units, dist=None, device=None):
    """Whole-job throughput of independent replicas: every rank times its own
    units between two barriers; the job time is the slowest rank's (MAX), the
    work the sum over ranks, so value = sum(units) / max(ms).  No data-path
    collective: the two reductions run once, outside the timed region."""
    if dist is None:
        return local_units / (local_ms / 1000.0), local_ms
    import torch
    t = torch.tensor([float(local_ms), float(local_units)], dtype=torch.float64, device=device)
    ms = t[:1].clone()
    units = t[1:].clone()
    dist.all_reduce(ms, op=dist.ReduceOp.MAX)
    dist.all_reduce(units, op=dist.ReduceOp.SUM)
    return float(units.item()) / (float(ms.item()) / 1000.0), float(ms.item())


def run_gpu(args):
    import torch
    from cdixx_gb300 import native as cdx

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    I, psi0 = make_inputs()
    # autotune: the context times its launch variants (PDL x row-pass chunk width) on its own
    # state before the first run (untimed warm-up) and keeps the fastest
    p = cdx.default_params(N, N, oversampling_spt=4.0, beta=BETA, shrink_threshold=0.1, autotune=1)
    stream = torch.cuda.Stream()
    ctx = cdx.Context(p, stream=stream.cuda_stream)
    ctx.set_pattern(0, I)
    ctx.set_initial(0, psi0)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def step():
        ctx.run_async(STEP_ALGO)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    launches_per_step = ctx.stats()["launches"]

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    for i in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
            ev[i][0].record(stream)
        step()
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = float(sum(step_ms))
    clk = clocks.stop()
    iters = SW_EVERY * args.steps
    value, total_ms = replica_throughput(total_ms, iters, dist, device="cuda")

    # roofline: pure iterations, events around each block of 50, L2 flushed before each
    it_ms = []
    for _ in range(5):
        with torch.cuda.stream(stream):
            flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        ctx.run_async(f"{SW_EVERY}*RAAR")
        b.record(stream)
        torch.cuda.synchronize()
        it_ms.append(a.elapsed_time(b) / SW_EVERY)
    t_iter = float(np.median(it_ms)) / 1000.0
    peak, peak_kind = peaks()
    achieved = ALG_BYTES_PER_PX_ITER * N * N / t_iter / 1e9
    traffic = PASS_TRAFFIC_2048
    # e2e: the whole job through the host-buffer C-ABI call
    e2e_vals = []
    h2d = I.nbytes + psi0.nbytes
    d2h = 2 * psi0.nbytes + I.nbytes
    # the call keeps its context and the job's CUDA graph for the next call with the same parameters
    pe = cdx.default_params(N, N, oversampling_spt=4.0, beta=BETA, shrink_threshold=0.1, autotune=1)
    # the job's host buffers in pinned memory (inputs and the results the call writes)
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    I_h, psi0_h = pin(I), pin(psi0)
    outs = (torch.empty(psi0.shape, dtype=torch.complex64, pin_memory=True).numpy(),
            torch.empty(psi0.shape, dtype=torch.complex64, pin_memory=True).numpy(),
            torch.empty(I.shape, dtype=torch.float32, pin_memory=True).numpy())
    for k in range(4):   # the first job warms the host allocator, the page cache and the kept graph; median of three
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        cdx.phase_retrieve_host(pe, JOB_ALGO, I_h, psi0_h, out=outs)
        dt = time.perf_counter() - t0
        if k > 0:
            e2e_vals.append(JOB_ITERS / dt)
    e2e = float(np.median(e2e_vals))

    cpu = None
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        cpu_sample(I, psi0, 1, threads)
        v, dt = cpu_sample(I, psi0, 2, threads)
        cpu = {"value": v, "unit": "iter/s", "cores": threads, "kind": "port",
               "sample": "2 RAAR iterations of the 2048^2 pattern, float32 oracle, "
                         f"scipy.fft with {threads} workers ({dt:.2f} s)"}
    warm = comb = batched = pty = cmpr = tcs = None
    if rank == 0 and not args.no_comparator:
        cmpr = comparator_section()
    if rank == 0 and not args.no_tc:
        tcs = tc_section()
    if rank == 0 and not args.no_ptycho:
        pty = ptycho_section(cpu=not args.no_cpu)
    if rank == 0 and not args.no_warm:
        warm, comb = northstar_sections()
    if rank == 0 and not args.no_batched:
        batched = batched_section()
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "iter/s", "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "step": STEP_ALGO, "patterns": 1, "rows": N, "cols": N,
                       "l2": "flushed (512 MB write) before every step", "parallelism": "replicas",
                       "patterns_per_s": value / JOB_ITERS, "path": "fused FP32 (column pass + row pass)",
                       "launch_variant": ctx.tuning()[2]},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                         "kernel": "one fused iteration (col_pass_rk<2048> + row_pass_rk<2048>)",
                         "t_iter_us": t_iter * 1e6},
            "e2e": {"value": e2e, "unit": "iter/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "step": "whole 2000-iteration job via cdx_phase_retrieve_host", "host_buffers": "pinned"},
            "cpu_baseline": cpu,
            "clocks": clk,
            "gpu_launches": launches_per_step * args.steps,
            "gpu_comparator": cmpr,
            "tc_fft": tcs,
            "warm_start": warm,
            "combined": comb,
            "batched": batched,
            "ptycho": pty,
        }
        print(json.dumps(line))
    ctx.close()
    if dist:
        dist.destroy_process_group()
    return 0


# ---------------------------------------------------------------------------
# Small self-checking workloads for kernel captures (ncu -k / -c):
#   python bench.py case pass --n 2048 --iters 3 [--fft-mode 1] [--batch B]
#   python bench.py case gemm --m 16384 --n 128 --k 4096
#   python bench.py case unet [--n 256 --batch 16 --steps 3 --umma 0]
#   python bench.py case ptycho [--probe 512 --object 1280 --sweeps 10 --first 400 --zernike-iter 1200]
# Each exits non-zero when its result is not finite (or, for the GEMM, not the
# FP32 product), so a capture is only taken of a run that worked.

def case_pass(a):
    """A few fused iterations of one synthetic pattern through the C ABI, graph
    capture off: after the set-up launches each iteration is one column pass and
    one row pass, then the final FFT, norm and reductions of the run.  At 2048^2
    the pattern is the large single-pattern configuration's; other sizes take
    uniform random intensities."""
    from cdixx_gb300 import native as cdx
    if a.n == N:   # the large single-pattern configuration's own pattern (Poisson, 60 % zeros)
        I, psi0 = make_inputs()
    else:
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


def case_gemm(a):
    """D = A B^T on the tcgen05 GEMM (cdx_gemm_bf16_tc), timed with CUDA events
    and checked against an FP32 product."""
    import ctypes
    import torch
    from cdixx_gb300 import native as cdx
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


def case_unet(a):
    """A few Adam steps of the warm-start network on one forward-model batch:
    mean training-step time (forward, loss, backward, Adam) by CUDA events."""
    import torch
    from cdixx_gb300 import unet
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
          f"loss {losses[-1]:.5f}, finite={ok}")
    net.close()
    return 0 if ok else 1


def case_ptycho(a):
    """rPIE + mPIE sweeps on the triangle scan of the reference's ptychography
    driver (its default optics) from noise-free patterns of a smooth object;
    fails when the object is not finite or the far-field error did not fall."""
    from cdixx_gb300 import ptycho as PT
    R, RO = a.probe, a.object
    sx, sy = PT.scan_triangle(RO, RO, R, R, a.step)
    t = PT.Ptycho(R, R, RO, RO, sx, sy, lam=0.6328, d=125e3, dpupil=6.8e3, pixelsize=13.0,
                  pupil_size=min(335.0083, R * 0.65), exposure=0.01, zernike_iter=a.zernike_iter)
    x = np.linspace(-1, 1, RO, dtype=np.float32)[:, None]
    y = np.linspace(-1, 1, RO, dtype=np.float32)[None, :]
    truth = ((0.6 + 0.4 * np.cos(9 * x) * np.sin(7 * y)) * np.exp(1.2j * np.sin(5 * x + 3 * y))).astype(np.complex64)
    t.initObject(seed=1)
    obj0 = t.objectWave
    t.objectWave = truth
    t.createPattern()
    pats = t.patterns
    t.objectWave = obj0
    t.iterate(1, first_iter=a.first, seed=3)
    t.objectWave = obj0
    ms = t.iterate(a.sweeps, first_iter=a.first, seed=5)
    obj = t.objectWave
    ok = bool(np.isfinite(obj).all())
    t.objectWave = obj
    t.createPattern()
    sim = t.patterns
    err = float(np.abs(np.sqrt(np.maximum(sim, 0)) - np.sqrt(pats)).sum() / np.sqrt(pats).sum())
    print(f"probe {R} object {RO} positions {len(sx)}: {ms / a.sweeps:.3f} ms/sweep, far-field error {err:.4f}, "
          f"finite={ok}")
    t.close()
    return 0 if ok and err < 1.0 else 1


def run_case(argv):
    ap = argparse.ArgumentParser(prog="bench.py case")
    sub = ap.add_subparsers(dest="case", required=True)
    c = sub.add_parser("pass")
    c.add_argument("--n", type=int, default=2048)
    c.add_argument("--batch", type=int, default=1)
    c.add_argument("--iters", type=int, default=3)
    c.add_argument("--algo", default="RAAR")
    c.add_argument("--fft-mode", type=int, default=0)
    c.add_argument("--repeat", type=int, default=2)
    c = sub.add_parser("gemm")
    c.add_argument("--m", type=int, default=16384)
    c.add_argument("--n", type=int, default=128)
    c.add_argument("--k", type=int, default=4096)
    c.add_argument("--reps", type=int, default=10)
    c = sub.add_parser("unet")
    c.add_argument("--n", type=int, default=256)
    c.add_argument("--batch", type=int, default=16)
    c.add_argument("--steps", type=int, default=3)
    c.add_argument("--levels", type=int, default=4)
    c.add_argument("--base", type=int, default=32)
    c.add_argument("--umma", type=int, default=0, help="1: tcgen05 convolutions, 0: mma.sync")
    c = sub.add_parser("ptycho")
    c.add_argument("--probe", type=int, default=512)
    c.add_argument("--object", type=int, default=1280)
    c.add_argument("--sweeps", type=int, default=10)
    c.add_argument("--step", type=float, default=250.0)
    c.add_argument("--first", type=int, default=0, help="iteration index of the first sweep (400+: probe phase)")
    c.add_argument("--zernike-iter", type=int, default=0,
                   help="zernikeIter (the reference's ptycho.cfg: 1200): FISTA step, probe momentum, Zernike fit")
    a = ap.parse_args(argv)
    return {"pass": case_pass, "gemm": case_gemm, "unet": case_unet, "ptycho": case_ptycho}[a.case](a)


def main():
    if len(sys.argv) > 1 and sys.argv[1] == "case":
        return run_case(sys.argv[2:])
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-warm", action="store_true", help="skip the learned warm-start section")
    ap.add_argument("--no-batched", action="store_true", help="skip the uneven-size batch section")
    ap.add_argument("--no-ptycho", action="store_true", help="skip the ptychography section")
    ap.add_argument("--no-comparator", action="store_true", help="skip the cuFFT-structure comparator section")
    ap.add_argument("--no-tc", action="store_true", help="skip the tensor-core FFT leg of the 2048^2 configuration")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
