"""Benchmark: converged pixels/s of the batched plain-method inversion.

Workload (one "step"): the whole synthetic 4096 x 4096 single scene of the
plain method -- 4 OLI-like bands (443/482/561/655 nm), sun 35 deg, nadir,
truth H~U(0.5,25) m, P~logU(0.005,0.1), G~logU(0.005,0.2),
X~logU(0.001,0.05), B~U(0.05,0.5) on sand, N(0, 2e-4) noise, 15 % of pixels
masked -- inverted with the cold-start Nelder-Mead at reqmin 1e-10,
kcount 2000 on one GPU.  The scene is generated on the device with the
seeded generator (synthetic data: the reference ships no dataset).

metric: converged pixels per second whose depth is within 1 cm of the FP64
oracle.  The full-scene FP64 reference is the FP64 kernel (its parity with
the CPU oracle is what tests/test_gpu_invert.py asserts); a random sample
of pixels is also re-fitted by the CPU oracle in the same run and the
within-1-cm fraction of that sample is reported and applied.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl photic|reference]
                  [--npix P] [--precision fp64|df64|fp32]

Under torchrun each rank inverts its own scene shard of the same size
(pixels are independent: weak scaling, no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SEED = 20260101
METRIC = "converged pixels/s at |dH|<=1cm vs FP64 (plain cold-start Nelder-Mead, 1 GB300)"
UNIT = "px/s"


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons while timing."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm = [float(r[1]) for r in self.rows if len(r) > 8 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 8 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            if len(r) > 8:
                for k, n in enumerate(names):
                    if r[5 + k].lower().startswith("active"):
                        reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(self.rows)}


def cpu_oracle_rate(npix: int, seed: int):
    """The CPU oracle (C restatement of the reference path, OpenMP over
    pixels) on a bounded sample of the same workload."""
    from oracle import oracle as O
    rrs, _ = O.generate_single(seed, npix, pix0=7_000_000)
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    out = O.invert_batch(rrs, nthreads=threads)
    dt = time.perf_counter() - t0
    conv = int(np.sum((out[:, 9] == 0) & (out[:, 8] == 1)))
    return conv / dt, threads, dt, npix, out


def run_reference(args, ws, rank):
    """--impl reference: the reference path on the host cores (the oracle
    port of it; the reference's own build needs sources absent here)."""
    if rank != 0:
        return
    from oracle import oracle as O
    kind = "reference" if O.reference_available() else "port"
    threads = os.cpu_count() or 1
    n = args.ref_sample
    rrs, _ = O.generate_single(SEED, n, pix0=7_000_000)
    which = "reference" if kind == "reference" else "port"
    for _ in range(args.warmup):
        O.invert_batch(rrs[: max(1, n // 16)], which=which, nthreads=threads)
    times, convs = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        out = O.invert_batch(rrs, which=which, nthreads=threads)
        times.append(time.perf_counter() - t0)
        convs.append(int(np.sum((out[:, 9] == 0) & (out[:, 8] == 1))))
    t = float(np.mean(times))
    value = float(np.mean(convs)) / t
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded generator, plain-method prior)",
            "config": {"workload": "plain method, 4096x4096 single scene, 4 bands, "
                                   "reqmin 1e-10 kcount 2000 (bounded sample per step)",
                       "sample_pixels": n, "host_threads": threads},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind,
                             "sample": f"{n} pixels of the same generator per step"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="photic", choices=["photic", "reference"])
    ap.add_argument("--npix", type=int, default=4096 * 4096)
    ap.add_argument("--precision", default="fp64", choices=["fp64", "df64", "fp32", "guarded"])
    ap.add_argument("--warmup-npix", type=int, default=1 << 20)
    ap.add_argument("--sample", type=int, default=2048, help="pixels re-fitted by the CPU oracle")
    ap.add_argument("--cpu-sample", type=int, default=1 << 16)
    ap.add_argument("--ref-sample", type=int, default=1 << 16)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--warm-npix", type=int, default=1 << 22,
                    help="pixels of the 8192x8192 scene for the warm-start comparison (0: skip)")
    ap.add_argument("--train-forward", type=int, default=1 << 23)
    ap.add_argument("--train-inverted", type=int, default=1 << 20)
    ap.add_argument("--train-epochs", type=int, default=4)
    ap.add_argument("--polish-iters", type=int, default=25,
                    help="Levenberg-Marquardt steps on each surrogate seed (0: raw prediction)")
    ap.add_argument("--seed-step-scale", type=float, default=0.1,
                    help="initial simplex of a seeded fit, relative to the cold-start steps")
    ap.add_argument("--joint-npix", type=int, default=1 << 18,
                    help="pixels of the 4096x4096 temporal grid for the joint-fit leg (0: skip)")
    ap.add_argument("--region-side", type=int, default=96,
                    help="side of the square grid for the spatial-region leg (0: skip)")
    ap.add_argument("--nc-side", type=int, default=4096,
                    help="side of the scene written to and read from netCDF band files (0: off)")
    ap.add_argument("--serve-requests", type=int, default=12,
                    help="tile requests of the serving leg (0: skip)")
    ap.add_argument("--serve-rate", type=float, default=50.0)
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")

    ws, rank, local = _dist()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return

    import torch
    import photic_gb300 as pg
    from photic_gb300 import _lib as L

    from photic_gb300 import replicas
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    pg_ = replicas.init("nccl", dev)
    stream = torch.cuda.current_stream()
    cfg = pg.Config(precision=args.precision)
    npix = args.npix
    pix0 = replicas.shard_start(rank, npix)
    rrs, truth = pg.generate_scene(npix, seed=SEED, config=cfg, pix0=pix0, device=dev)
    out = pg.alloc_outputs(npix, dev, ("depth", "depth_f64", "P", "G", "X", "bottom_albedo",
                                       "model_error", "evals", "status"))

    counter = torch.zeros(1, dtype=torch.int64, device=dev)
    L.check(L.lib().photic_set_counter(counter.data_ptr()))
    # warm-up on a slice of the scene (W launches)
    for _ in range(args.warmup):
        pg.invert(rrs[: min(npix, args.warmup_npix)], cfg)
    pg.sync()

    def barrier():
        if pg_ is not None:
            pg_.barrier()

    clocks = Clocks(local)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        pg.invert(rrs, cfg, out=out)
    ev1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    barrier()
    pg.sync()
    ms_step = ev0.elapsed_time(ev1) / args.steps
    L.check(L.lib().photic_set_counter(None))
    ms_step = replicas.max_over_ranks(ms_step, pg_, dev)

    status = out["status"].cpu().numpy()
    fitted = (status & 0xFF) == 0
    conv = fitted & ((status >> 8) & 1).astype(bool)
    evals = out["evals"].cpu().numpy().astype(np.int64)
    h = out["depth_f64"].cpu().numpy()

    # FP64 reference of the full scene: the FP64 kernel itself, or a run of it.
    if args.precision == "fp64":
        h64 = h
    else:
        ref = pg.invert(rrs, pg.Config(precision="fp64"),
                        fields=("depth_f64", "status"))
        pg.sync()
        h64 = ref["depth_f64"].cpu().numpy()
    within = conv & (np.abs(h - h64) <= 0.01)

    # CPU-oracle sample: same pixels, FP64 C restatement of the reference.
    sample_frac, sample_stats = 1.0, None
    if rank == 0 and args.sample > 0:
        from oracle import oracle as O
        rng = np.random.default_rng(1)
        idx = np.sort(rng.choice(npix, size=min(args.sample, npix), replace=False))
        r_np = rrs[torch.tensor(idx, device=dev)].cpu().numpy()
        o = O.invert_batch(r_np, nthreads=os.cpu_count() or 1)
        m = (o[:, 9] == 0) & conv[idx]
        d = np.abs(h[idx][m] - o[m, 0])
        sample_frac = float(np.mean(d <= 0.01)) if m.any() else 1.0
        sample_stats = {"pixels": int(m.sum()), "median_abs_dH_m": float(np.median(d)),
                        "p99_abs_dH_m": float(np.quantile(d, 0.99)),
                        "frac_within_1cm": sample_frac}
    good = float(np.sum(within)) * sample_frac
    good = replicas.sum_over_ranks(good, pg_, dev)
    value = good / (ms_step * 1e-3)

    # Roofline of the inversion kernel: FP64 pipe.
    p64 = np.zeros(1)
    p32 = np.zeros(1)
    pmu = np.zeros(1)
    import ctypes as C
    L.check(L.lib().photic_measure_peaks(p64.ctypes.data_as(C.POINTER(C.c_double)),
                                         p32.ctypes.data_as(C.POINTER(C.c_double)),
                                         pmu.ctypes.data_as(C.POINTER(C.c_double))))
    total_evals = float(evals.sum())
    flops_per_eval = FLOPS_PER_EVAL_F64
    achieved = total_evals * flops_per_eval / (ms_step * 1e-3) / 1e12
    roof = {"bound": "fp64-pipe", "achieved": achieved, "peak": float(p64[0]),
            "unit": "TFLOP/s", "frac": achieved / float(p64[0]),
            "traffic": TRAFFIC_BYTES_PER_PIXEL * npix,
            "traffic_note": "DRAM bytes per launch, scaled by pixels from an ncu capture of "
                            "a 65536-pixel launch of this kernel taken before its simplex "
                            "vectors moved from local memory to registers (most of those "
                            "bytes were the local-memory stack frame); not yet recaptured",
            "peak_source": "measured by photic_measure_peaks (DFMA chains) in this run",
            "evals_per_s": total_evals / (ms_step * 1e-3),
            "flops_per_eval": flops_per_eval}

    # End to end through the public API with host buffers.
    e2e = None
    if rank == 0:
        host_in = rrs.cpu().pin_memory()
        host_depth = torch.empty(npix, dtype=torch.float32).pin_memory()
        host_status = torch.empty(npix, dtype=torch.int32).pin_memory()
        dev_in = torch.empty_like(rrs)
        o2 = pg.alloc_outputs(npix, dev, ("depth", "status"))
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        t0.record(stream)
        dev_in.copy_(host_in, non_blocking=True)
        pg.invert(dev_in, cfg, out=o2)
        host_depth.copy_(o2["depth"], non_blocking=True)
        host_status.copy_(o2["status"], non_blocking=True)
        t1.record(stream)
        torch.cuda.synchronize()
        e2e_ms = t0.elapsed_time(t1)
        st2 = host_status.numpy()
        conv2 = ((st2 & 0xFF) == 0) & ((st2 >> 8) & 1).astype(bool)
        within2 = conv2 & (np.abs(host_depth.numpy().astype(np.float64) - h64) <= 0.01)
        e2e = {"value": float(np.sum(within2)) * sample_frac / (e2e_ms * 1e-3), "unit": UNIT,
               "h2d_bytes_per_step": int(host_in.numel() * 4),
               "d2h_bytes_per_step": int(npix * 8), "ms_per_step": e2e_ms}

    cpu = None
    if rank == 0 and not args.no_cpu and args.cpu_sample > 0:
        rate, threads, dt, n, _ = cpu_oracle_rate(args.cpu_sample, SEED)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{n} pixels of the same generator, {dt:.1f} s on {threads} threads"}

    temporal = None
    if rank == 0 and args.joint_npix > 0:
        temporal = temporal_leg(args, dev)
    regions = None
    if rank == 0 and args.region_side > 0:
        regions = region_leg(args, dev)
    warm, net, serving = None, None, None
    if rank == 0 and args.warm_npix > 0:
        net, warm = warm_start_leg(args, dev)
    if rank == 0 and args.serve_requests > 0:
        serving = serving_leg(args, net)
    ncgrid = None
    if rank == 0 and args.nc_side > 0:
        try:
            ncgrid = ncgrid_leg(args, dev, rrs)
        except Exception as e:  # the format leg must not cost the headline line
            ncgrid = {"error": f"{type(e).__name__}: {e}"}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": {"fp64": "f64", "df64": "df64 (2 x f32)", "fp32": "f32",
                          "guarded": "f64 decisions (df64 screening)"}[args.precision],
                "data": "synthetic (seeded on-device generator, plain-method prior)",
                "config": {"workload": "plain method, 4096x4096 single scene, 4 bands, "
                                       "cold start, reqmin 1e-10, kcount 2000",
                           "pixels_per_gpu": npix, "precision": args.precision,
                           "l2": "inputs 268 MB > L2; compute-bound kernel"},
                "gpu_launches": args.steps,
                "exact_evals_per_step": int(counter.item()) // max(1, args.steps + args.warmup),
                "pixels": {"fitted": int(fitted.sum()), "converged": int(conv.sum()),
                           "within_1cm_of_fp64": int(within.sum()),
                           "mean_evals": float(evals[fitted].mean()) if fitted.any() else 0.0},
                "oracle_sample": sample_stats, "roofline": roof, "cpu_baseline": cpu,
                "warm_start": warm, "serving": serving, "temporal": temporal,
                "regions": regions, "ncgrid": ncgrid,
                "e2e": e2e, "clocks": clk}
        print(json.dumps(line))
    if pg_ is not None:
        pg_.destroy_process_group()


def warm_start_leg(args, dev):
    """Surrogate-warm vs plain cold-start Nelder-Mead on a sample of the
    8192 x 8192 scene: train the network on photic's own forward-model
    samples and converged inversions, seed the fit (cold fallback where the
    seed's spectral residual exceeds 3 sigma of the noise), and compare
    converged pixels/s; parity of the seeded fits is checked against the
    CPU oracle started from the same seeds."""
    import torch
    import photic_gb300 as pg
    from photic_gb300 import surrogate as S
    from oracle import oracle as O

    t0 = time.perf_counter()
    net = S.Surrogate(seed=1)
    x, t = S.training_data(args.train_forward, args.train_inverted, seed=31, device=dev)
    t_data = time.perf_counter() - t0
    hist = S.train(net, x, t, epochs=args.train_epochs, batch=8192, lr=2e-3)
    del x, t
    n = args.warm_npix
    # pixels of the 8192^2 scene (seeded generator; row-major pixel ids)
    rrs, _ = pg.generate_scene(n, seed=SEED + 2, pix0=8192 * 4096, device=dev)
    cfg = pg.Config()
    fields = ("depth_f64", "status", "evals")

    def timed(fn):
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev0.record()
        r = fn()
        ev1.record()
        torch.cuda.synchronize()
        return r, ev0.elapsed_time(ev1) * 1e-3

    wcfg = pg.Config(seed_step_scale=args.seed_step_scale)
    # warm the kernels (and the lazily loaded library code of each step)
    pg.invert(rrs[:4096], cfg, fields=fields)
    s_w, _ = net.seeds(rrs[:4096], cfg, polish_iters=args.polish_iters)
    pg.invert(rrs[:4096], wcfg, seeds=s_w, order=pg.fallbacks_first(s_w), fields=fields)
    torch.cuda.synchronize()
    cold, t_cold = timed(lambda: pg.invert(rrs, cfg, fields=fields))
    # the raw network prediction as seed, for comparison
    (seeds0, _), t_seed0 = timed(lambda: net.seeds(rrs, cfg))
    warm0, t_warm0 = timed(lambda: pg.invert(rrs, wcfg, seeds=seeds0, fields=fields))
    (seeds, res, order), t_seed = timed(
        lambda: (*net.seeds(rrs, cfg, polish_iters=args.polish_iters), None))
    order, t_order = timed(lambda: pg.fallbacks_first(seeds))
    t_seed += t_order
    warm, t_warm = timed(lambda: pg.invert(rrs, wcfg, seeds=seeds, order=order, fields=fields))
    pg.sync()

    def conv(o):
        st = o["status"]
        return (((st & 0xFF) == 0) & ((st >> 8) & 1).bool())
    cc, cw = conv(cold), conv(warm)
    seeded = ~torch.isnan(seeds[:, 0]) & ((cold["status"] & 0xFF) == 0)
    # parity of the warm path: the oracle started from the same seeds
    idx = torch.arange(0, n, max(1, n // 1024), device=dev)
    sd_np = seeds[idx].cpu().numpy()
    ref = O.invert_batch(rrs[idx].cpu().numpy(), seeds=sd_np, seed_step_scale=args.seed_step_scale,
                         nthreads=os.cpu_count() or 1)
    m = (ref[:, 9] == 0) & cw[idx].cpu().numpy()
    d = np.abs(warm["depth_f64"][idx].cpu().numpy()[m] - ref[m, 0])
    within = float(np.mean(d <= 0.01)) if m.any() else 1.0
    v_cold = float(cc.sum().item()) / t_cold
    v_warm = float(cw.sum().item()) * within / (t_warm + t_seed)
    v_warm0 = float(conv(warm0).sum().item()) / (t_warm0 + t_seed0)
    seeded0 = ~torch.isnan(seeds0[:, 0]) & ((cold["status"] & 0xFF) == 0)
    return net, {"workload": f"{n} pixels of the 8192x8192 plain-method scene",
            "cold_px_s": v_cold, "warm_px_s": v_warm, "speedup": v_warm / v_cold,
            "seed": f"network prediction + {args.polish_iters} Levenberg-Marquardt steps, "
                    f"simplex scale {args.seed_step_scale}; cold-start fallbacks queued first",
            "unpolished": {"warm_px_s": v_warm0, "speedup": v_warm0 / v_cold,
                           "seeded_share": float(seeded0.float().mean().item())},
            "seeded_share": float(seeded.float().mean().item()),
            "evals_per_pixel_cold": float(cold["evals"].float()[cc].mean().item()),
            "evals_per_pixel_warm": float(warm["evals"].float()[cw].mean().item()),
            "seed_ms": t_seed * 1e3, "fallback": "seed spectral RMS > 3 x 2e-4",
            "train": {"samples": hist["samples"], "epochs": args.train_epochs,
                      "seconds": hist["seconds"], "data_seconds": t_data,
                      "final_loss": hist["loss"][-1]},
            "parity_vs_seeded_oracle": {"pixels": int(m.sum()),
                                        "median_abs_dH_m": float(np.median(d)) if m.any() else 0.0,
                                        "p99_abs_dH_m": float(np.quantile(d, 0.99)) if m.any() else 0.0,
                                        "frac_within_1cm": within}}


def temporal_leg(args, dev):
    """Temporal joint fit on a sample of the 4096 x 4096 grid (k ~ U{2..8}
    scenes per pixel, shared depth, per-scene sun zenith U(25, 50) deg), all
    ragged pixels in one CUDA-graph replay, in the reference's parameter
    layout (n = 3 + 3k) and the per-scene-albedo layout (n = 1 + 4k).
    Parity against the FP64 oracle on a sub-sample; the oracle's own rate on
    the host cores beside it."""
    import torch
    import photic_gb300 as pg
    from oracle import oracle as O
    n = args.joint_npix
    offs, th, rrs, _ = pg.generate_joint(n, seed=20260202, device=dev)
    n_obs = rrs.shape[0]
    offs_h, th_h, rrs_h = offs.cpu().numpy(), th.cpu().numpy(), rrs.cpu().numpy()
    rng = np.random.default_rng(5)
    sub = np.sort(rng.choice(n, size=min(n, 192), replace=False))
    counts = offs_h[1:] - offs_h[:-1]
    so = np.zeros(len(sub) + 1, dtype=np.int32)
    so[1:] = np.cumsum(counts[sub])
    obs = np.concatenate([np.arange(offs_h[p], offs_h[p + 1]) for p in sub])
    res = {"workload": f"{n} pixels of the 4096x4096 temporal grid, k ~ U{{2..8}}",
           "observations": int(n_obs), "mean_scenes": float(n_obs / n)}
    for layout in ("reference", "scene_b"):
        cfg = pg.Config(layout=layout)
        g = pg.JointGraph(n, n_obs, cfg, fields=("depth_f64", "status", "evals"))
        g.run(offs, th, rrs)
        pg.sync()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev0.record()
        out = g.run()
        ev1.record()
        torch.cuda.synchronize()
        pg.sync()
        t = ev0.elapsed_time(ev1) * 1e-3
        st = out["status"]
        conv = ((st & 0xFF) == 0) & ((st >> 8) & 1).bool()
        ref = O.joint_invert_batch(so, th_h[obs], rrs_h[obs],
                                   layout=0 if layout == "reference" else 1,
                                   nthreads=os.cpu_count() or 1)
        m = (ref[:, 9] == 0) & conv[torch.tensor(sub, device=dev)].cpu().numpy()
        d = np.abs(out["depth_f64"][torch.tensor(sub, device=dev)].cpu().numpy()[m] - ref[m, 0])
        within = float(np.mean(d <= 0.01)) if m.any() else 1.0
        t0 = time.perf_counter()
        O.joint_invert_batch(so, th_h[obs], rrs_h[obs], layout=0 if layout == "reference" else 1,
                             nthreads=os.cpu_count() or 1)
        t_cpu = time.perf_counter() - t0
        res[layout] = {
            "n_params": "3 + 3k" if layout == "reference" else "1 + 4k",
            "converged_px_s_within_1cm": float(conv.sum().item()) * within / t,
            "seconds": t, "converged_share": float(conv.float().mean().item()),
            "mean_evals": float(out["evals"].float().mean().item()),
            "graph": "one replay: binning + 8 per-k kernels on parallel branches",
            "oracle_sample": {"pixels": int(m.sum()),
                              "median_abs_dH_m": float(np.median(d)) if m.any() else 0.0,
                              "p99_abs_dH_m": float(np.quantile(d, 0.99)) if m.any() else 0.0,
                              "frac_within_1cm": within},
            "cpu_oracle_px_s": len(sub) / t_cpu, "cpu_threads": os.cpu_count() or 1}
        del g, out
    torch.cuda.empty_cache()
    return res


def region_leg(args, dev):
    """Spatial-region fit (3 x 3 neighbourhoods) of a square grid of the
    plain-method generator: converged pixels/s, parity against the FP64
    oracle on a corner block, and the oracle's own rate beside it."""
    import torch
    import photic_gb300 as pg
    from oracle import oracle as O
    n = args.region_side
    rrs, _ = pg.generate_scene(n * n, seed=SEED + 5, device=dev)
    grid = rrs.reshape(n, n, 4).contiguous()
    cfg = pg.Config()
    pg.region_invert(grid[:8, :8].contiguous(), cfg, fields=("depth_f64", "status"))
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record()
    out = pg.region_invert(grid, cfg, fields=("depth_f64", "status", "evals"))
    ev1.record()
    torch.cuda.synchronize()
    pg.sync()
    t = ev0.elapsed_time(ev1) * 1e-3
    st = out["status"]
    conv = ((st & 0xFF) == 0) & ((st >> 8) & 1).bool()
    # parity on a 16 x 16 corner block fitted on its own (its edge pixels
    # see a clamped neighbourhood, as on the GPU for the same block)
    k = min(16, n)
    blk = grid[:k, :k].contiguous()
    g_blk = pg.region_invert(blk, cfg, fields=("depth_f64", "status"))
    pg.sync()
    t0 = time.perf_counter()
    ref = O.region_invert_batch(blk.cpu().numpy(), nthreads=os.cpu_count() or 1)
    t_cpu = time.perf_counter() - t0
    fit = (g_blk["status"].cpu().numpy() & 0xFF) == 0
    d = np.abs(g_blk["depth_f64"].cpu().numpy()[fit] - ref[fit, 0])
    within = float(np.mean(d <= 0.01)) if fit.any() else 1.0
    return {"workload": f"{n}x{n} grid, 3x3 regions per pixel (n = 3R + 3 <= 30 unknowns)",
            "converged_px_s_within_1cm": float(conv.sum().item()) * within / t, "seconds": t,
            "converged_share": float(conv.float().mean().item()),
            "mean_evals": float(out["evals"].float().mean().item()),
            "oracle_sample": {"pixels": int(fit.sum()), "frac_within_1cm": within,
                              "median_abs_dH_m": float(np.median(d)) if fit.any() else 0.0},
            "cpu_oracle_px_s": k * k / t_cpu, "cpu_threads": os.cpu_count() or 1}


def ncgrid_leg(args, dev, rrs):
    """The scene's bands through the reference's netCDF grid files
    (model/nc.c): each band written from the device (GPU packing, host
    container), the four files read back into the inversion's layout (host
    container, GPU unpacking), and the two kernels timed alone against the
    measured HBM copy rate.  Algorithmic bytes: unpacking reads 2 B and
    writes 4 B per cell and band; packing reads 4 B and writes 2 B per cell
    (its three passes read the grid three times).  Parity: the unpacked
    bands and the packed grid against the CPU oracle on a sample."""
    import tempfile
    import torch
    from photic_gb300 import ncgrid as N
    from oracle import oracle as O
    import math
    n = min(args.nc_side, math.isqrt(rrs.shape[0]))
    npix = n * n
    nodata = -9999.0
    lons = np.linspace(150.0, 151.0, n).astype(np.float32)
    lats = np.linspace(-24.0, -23.0, n).astype(np.float32)
    bands = [rrs[:npix, b].reshape(n, n).contiguous() for b in range(4)]
    tmp = tempfile.mkdtemp(prefix="photic_nc_")
    paths = [os.path.join(tmp, f"band{b}.nc") for b in range(4)]
    try:
        N.write_grid(paths[0], bands[0], lons, lats, nodata)  # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for b in range(4):
            N.write_grid(paths[b], bands[b], lons, lats, nodata)
        t_write = time.perf_counter() - t0
        N.read_bands(paths)  # warm-up (and page cache)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out, info, _, _ = N.read_bands(paths)
        torch.cuda.synchronize()
        t_read = time.perf_counter() - t0
        packed, infos = [], []
        for b in range(4):
            pk, inf = N.pack(bands[b], nodata)
            inf.update(ncols=n, nrows=n)
            packed.append(pk)
            infos.append(inf)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        reps = 5
        N.unpack_bands(packed, infos, npix)
        torch.cuda.synchronize()
        ev[0].record()
        for _ in range(reps):
            N.unpack_bands(packed, infos, npix)
        ev[1].record()
        for _ in range(reps):
            N.pack(bands[0], nodata)
        ev[2].record()
        torch.cuda.synchronize()
        t_un = ev[0].elapsed_time(ev[1]) / reps * 1e-3
        t_pk = ev[1].elapsed_time(ev[2]) / reps * 1e-3
        peak = None
        try:
            with open(os.path.join(os.path.dirname(os.path.abspath(__file__)),
                                   "MEASURED_PEAKS.json")) as f:
                peak = float(json.load(f)["hbm_gbs"])
        except (OSError, KeyError, ValueError):
            pass
        un_gbs = npix * 4 * 6 / t_un / 1e9
        pk_gbs = npix * 6 / t_pk / 1e9
        # parity on a sample of cells
        k = min(npix, 1 << 20)
        g0 = bands[0].reshape(-1)[:k].cpu().numpy().reshape(1, -1)
        want, off, sc, mv = O.nc_compress(g0, nodata)
        got_pk, inf0 = N.pack(bands[0].reshape(-1)[:k].contiguous(), nodata)
        got = np.frombuffer(got_pk.cpu().numpy().tobytes(), dtype=">i2").astype(np.int16)
        pack_ok = bool(np.array_equal(got, want.reshape(-1)) and
                       np.float32(inf0["scale_factor"]) == np.float32(sc))
        p_full = np.frombuffer(packed[0].cpu().numpy().tobytes(), dtype=">i2").astype(np.int16)
        dec, _ = O.nc_decompress(p_full[:k], infos[0]["add_offset"], infos[0]["scale_factor"],
                                 infos[0]["missing_value"], nodata)
        unpack_ok = dec.tobytes() == out[:k, 0].contiguous().cpu().numpy().tobytes()
        return {"workload": f"{n}x{n} scene, 4 band files (short-packed, {2 * npix >> 20} MiB each)",
                "write_grid_px_s": 4 * npix / t_write, "read_bands_px_s": npix / t_read,
                "unpack": {"ms": t_un * 1e3, "algorithmic_bytes_per_px": 24,
                           "achieved_gbs": un_gbs,
                           "frac_of_measured_hbm": un_gbs / peak if peak else None},
                "pack": {"ms": t_pk * 1e3, "algorithmic_bytes_per_cell": 6,
                         "achieved_gbs": pk_gbs,
                         "frac_of_measured_hbm": pk_gbs / peak if peak else None,
                         "note": "three passes read the grid three times (14 B/cell moved)"},
                "oracle_sample": {"cells": k, "pack_identical": pack_ok,
                                  "unpack_identical": bool(unpack_ok)}}
    finally:
        for p in paths:
            if os.path.exists(p):
                os.remove(p)
        os.rmdir(tmp)


def serving_leg(args, net):
    """Tile requests (square, side logU(256, 4096), Poisson arrivals)
    through the serving loop, plain cold start and, when a trained network
    is at hand, warm start; same schedule for both."""
    import torch
    from photic_gb300 import serve as S
    sched = lambda: S.poisson_schedule(args.serve_requests, rate=args.serve_rate)
    out = {"schedule": {"requests": args.serve_requests, "rate_per_s": args.serve_rate,
                        "side": "logU(256, 4096)", "seed": 20260404,
                        "pixels": sum(r.npix for r in sched())}}
    # the kernels and allocator are warm from the legs before
    out["cold"] = S.serve(sched())
    if net is not None:
        out["warm"] = S.serve(sched(), surrogate=net)
        out["warm_vs_cold_px_s"] = out["warm"]["px_s"] / out["cold"]["px_s"]
    torch.cuda.empty_cache()
    return out


# Algorithmic double-precision operations of one cost evaluation at 4 bands
# (adds, multiplies, divides, square roots; exp/log counted as one each):
# 43 per band (photic_fp64.cuh cost_f64) + 9 in the tail.
FLOPS_PER_EVAL_F64 = 4 * 43 + 9

# dram__bytes_read.sum + dram__bytes_write.sum of the FP64 inversion kernel
# over a 65 536-pixel launch (26.730240 MB + 19.621888 MB), per pixel: 16 B
# of spectra and the outputs, the rest the threads' local-memory stack frames
# leaving L2.  Under 1 GB/s at the kernel's rate.
TRAFFIC_BYTES_PER_PIXEL = (26.730240e6 + 19.621888e6) / 65536

if __name__ == "__main__":
    main()
