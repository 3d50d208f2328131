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
# col_pass_rk<2048> + row_pass_rk<2048>, from one ncu capture of
# `python bench.py case pass --n 2048 --iters 3` (profiles/pass_kernels_2048.md)
PASS_TRAFFIC_2048 = 131_400_000
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


WARM_N, WARM_BATCH, WARM_TRAIN_SEEDS, WARM_EVAL = 256, 64, 50_000, 1024
WARM_TARGET = 0.02
# the reference's path for this object family: HIO beta 0.9 x180 then ER x20 with a
# shrinkwrap every 20 iterations, from a random-phase start and the rect support
PLAIN_ALGO = "10*(" + "+".join(["20*HIO+1*shrinkWrap"] * 9) + "+20*ER+1*shrinkWrap)"
# from the network's warm start: the same HIO/ER schedule on its (fixed) support
WARM_ALGO = "10*(180*HIO+20*ER)"


def warm_start_section():
    """Learned warm start (U-Net trained here by the library's own kernels) vs the
    plain random-phase path on held-out noise-free 256^2 blob patterns: patterns/s
    that reach R <= WARM_TARGET within 2000 iterations (per-pattern stop)."""
    import torch
    from cdixx_gb300 import metrics, unet
    from cdixx_gb300 import native as cdx
    n, B = WARM_N, WARM_BATCH
    net = unet.UNet(n=n, levels=4, base=32, batch=B, seed=SEED)
    steps = WARM_TRAIN_SEEDS // B
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    losses = unet.train(net, steps, seed=SEED, photons=1e6, lr=1e-3)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    res = {"plain": [0, 0.0, [], []], "learned": [0, 0.0, [], []]}   # reached, seconds, iters, errors
    ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
    for k in range(WARM_EVAL // B):
        I, a, _, _ = unet.forward_model(n, B, SEED + 1, k * B, -1e6)
        truth = a.cpu().numpy() if k < 2 else None
        ev[0].record()
        out = net.forward(I)
        psi_w, sup_w = net.warm_start(I, out, 3)
        ev[1].record()
        torch.cuda.synchronize()
        net_s = ev[0].elapsed_time(ev[1]) / 1000.0
        for mode in ("plain", "learned"):
            prm = cdx.default_params(n, n, batch=B, beta=0.9, shrink_threshold=0.1, oversampling_spt=2.0,
                                     rf_every=10, stop_rfactor=WARM_TARGET)
            with cdx.Context(prm) as ctx:
                for i in range(B):
                    ctx.set_pattern(i, I[i])
                if mode == "plain":
                    ctx.random_start(SEED + k)
                else:
                    for i in range(B):
                        ctx.set_initial(i, psi_w[i])
                        ctx.set_support(i, sup_w[i])
                st = ctx.run(PLAIN_ALGO if mode == "plain" else WARM_ALGO)
                conv = [ctx.stats(i)["converged_iter"] for i in range(B)]
                r = res[mode]
                r[0] += sum(c >= 0 for c in conv)
                r[1] += st["gpu_ms"] / 1000.0 + (net_s if mode == "learned" else 0.0)
                r[2] += [c for c in conv if c >= 0]
                if truth is not None:
                    r[3] += [metrics.error_vs_truth(ctx.get_object(i), truth[i]) for i in range(B)]
    out = {"metric": f"patterns/s reaching R<={WARM_TARGET} within 2000 iterations",
           "patterns": WARM_EVAL, "n": n, "data": "noise-free synthetic blob objects (held-out seeds)",
           "train": {"seeds": steps * B, "batch": B, "lr": 1e-3, "seconds": train_s,
                     "loss_first": losses[0], "loss_last": float(np.mean(losses[-20:]))}}
    for mode, (reached, secs, its, errs) in res.items():
        out[mode] = {"patterns_per_s": reached / secs, "reached": reached / WARM_EVAL,
                     "median_iterations": float(np.median(its)) if its else None,
                     "gpu_s": secs, "median_error_vs_truth": float(np.median(errs)) if errs else None,
                     "algorithm": PLAIN_ALGO if mode == "plain" else WARM_ALGO + " (+ U-Net forward)"}
    pp = out["plain"]["patterns_per_s"]
    out["speedup"] = out["learned"]["patterns_per_s"] / pp if pp > 0 else None
    net.close()
    return out


BATCH_SIZES = (128, 192, 256, 384, 512)
BATCH_PATTERNS = 512
BATCH_ALGO = "500*HIO+500*ER"


def batched_section():
    """512 patterns of uneven sizes (uniform over BATCH_SIZES squared, photons
    log-uniform 1e5..1e8, blob objects in a support of 1/4 linear size), HIO and
    ER 500 iterations each, every size one context, all run as one CUDA graph."""
    import torch
    from cdixx_gb300 import native as cdx
    from cdixx_gb300 import unet
    rng = np.random.default_rng(SEED)
    sizes = rng.choice(BATCH_SIZES, BATCH_PATTERNS)
    photons = 10 ** rng.uniform(5, 8, BATCH_PATTERNS)
    ctxs = []
    px = 0
    for n in BATCH_SIZES:
        idx = np.nonzero(sizes == n)[0]
        if len(idx) == 0:
            continue
        ctx = cdx.Context(cdx.default_params(int(n), int(n), batch=len(idx), beta=0.9, oversampling_spt=2.0))
        for j, p in enumerate(idx):
            I, _, _, _ = unet.forward_model(int(n), 1, SEED + 2, int(p), float(photons[p]))
            ctx.set_pattern(j, I[0])
        ctx.random_start(SEED + int(n))
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
    g.close()
    for c in ctxs:
        c.close()
    iters = 1000
    return {"metric": "patterns/s", "patterns": BATCH_PATTERNS, "sizes": list(BATCH_SIZES),
            "algorithm": BATCH_ALGO, "patterns_per_s": BATCH_PATTERNS / (ms / 1000.0),
            "pixel_iterations_per_s": px * iters / (ms / 1000.0), "gpu_ms": ms, "wall_ms_incl_graph_build": wall * 1000,
            "contexts": len(ctxs), "launch": "one CUDA graph (cdx_group) with one branch per size"}


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
    pe = cdx.default_params(N, N, oversampling_spt=4.0, beta=BETA, shrink_threshold=0.1, use_graph=0, autotune=1)
    # the job's host buffers in pinned memory (inputs and the results the call writes)
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    I_h, psi0_h = pin(I), pin(psi0)
    outs = (torch.empty(psi0.shape, dtype=torch.complex64, pin_memory=True).numpy(),
            torch.empty(psi0.shape, dtype=torch.complex64, pin_memory=True).numpy(),
            torch.empty(I.shape, dtype=torch.float32, pin_memory=True).numpy())
    for k in range(4):   # the first job warms the host allocator and the page cache; median of three
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
    warm = batched = pty = None
    if rank == 0 and not args.no_ptycho:
        pty = ptycho_section(cpu=not args.no_cpu)
    if rank == 0 and not args.no_warm:
        warm = warm_start_section()
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
            "warm_start": warm,
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
    one row pass, then the final FFT, norm and reductions of the run."""
    from cdixx_gb300 import native as cdx
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
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
