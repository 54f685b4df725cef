"""Benchmark: converged pixels/s of the surrogate-warm batched inversion
against the plain cold-start Nelder-Mead, on one GB300.

Workload of the headline (one "step"): one tile of the synthetic 8192 x 8192
single scene of the plain method -- 4 OLI-like bands (443/482/561/655 nm),
sun 35 deg, nadir, truth H~U(0.5,25) m, P~logU(0.005,0.1),
G~logU(0.005,0.2), X~logU(0.001,0.05), B~U(0.05,0.5) on sand, N(0, 2e-4)
noise, 15 % of pixels masked.  The scene (67 108 864 pixels) is processed
as 4 tiles of 2048 x 8192 pixels; a step seeds one tile from the learned
warm start (network prediction + Levenberg-Marquardt polish, cold
multi-start where the seed's spectral residual exceeds 3 sigma of the
noise) and fits it with the batched Nelder-Mead at reqmin 1e-10, kcount
2000, FP64.  Steps cycle through the tiles.  The network is trained first
(untimed) on photic's own forward-model samples and converged inversions.
The scene is generated on the device by the seeded generator (synthetic
data: the reference ships no dataset).

metric: converged pixels per second whose depth is within 1 cm of the FP64
oracle started from the same seeds (a random sample of the timed pixels is
re-fitted by the CPU oracle in the same run; its within-1-cm fraction is
applied).  Beside it: the plain cold-start method over the same full scene
(plain_value, warm_over_plain), what the network adds over the same polish
started from the reference's cold-start guess, the 4096 x 4096 plain scene,
the temporal joint fit, 3 x 3 regions, netCDF band files and the serving
loop.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl photic|reference]

Under torchrun each rank fits its own 8192 x 8192 scene shard (pixels are
independent: weak scaling, no collective on the data path).
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
SCENE_SEED = SEED + 2  # the 8192 x 8192 scene
METRIC = ("converged pixels/s at |dH|<=1cm vs FP64 (surrogate-warm Nelder-Mead, "
          "8192x8192 scene, 1 GB300)")
UNIT = "px/s"
WORKLOAD = ("learned warm start, 8192x8192 single scene (4 tiles of 2048x8192 px), 4 bands, "
            "reqmin 1e-10, kcount 2000, FP64; network + 25 Levenberg-Marquardt steps, cold "
            "fallback above 3 sigma")


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


def _nvtx(push: bool):
    """An NVTX range named "timed" around the timed steps, so that a profiler
    can restrict its launch list to them (ncu --nvtx --nvtx-include timed/)."""
    import torch
    try:
        if push:
            torch.cuda.nvtx.range_push("timed")
        else:
            torch.cuda.nvtx.range_pop()
    except (RuntimeError, AttributeError):
        pass


def _rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.abs(a - b) / np.maximum(np.abs(b), 1e-30)


def oracle_stats(h_gpu, ref, mask, gpu_pgxb=None):
    """|dH| against the oracle record `ref` (oracle/oracle.py columns) over
    `mask`, with the relative P/G/X/bottom-albedo errors when given."""
    d = np.abs(np.asarray(h_gpu)[mask] - ref[mask, 0])
    if d.size == 0:
        return {"pixels": 0, "frac_within_1cm": 1.0}
    s = {"pixels": int(d.size), "median_abs_dH_m": float(np.median(d)),
         "p99_abs_dH_m": float(np.quantile(d, 0.99)), "frac_within_1cm": float(np.mean(d <= 0.01)),
         "identical_depth": float(np.mean(d == 0))}
    if gpu_pgxb is not None:
        for k, col in (("P", 11), ("G", 19), ("X", 27), ("B", 1)):
            if k in gpu_pgxb:
                e = _rel(np.asarray(gpu_pgxb[k])[mask], ref[mask, col])
                s[f"rel_err_{k}"] = {"median": float(np.median(e)),
                                     "p99": float(np.quantile(e, 0.99))}
    return s


def cpu_oracle_rate(npix: int, seed: int, pix0: int):
    """The CPU oracle (C restatement of the reference path, OpenMP over
    pixels) on a bounded sample of the same workload, cold start."""
    from oracle import oracle as O
    rrs, _ = O.generate_single(seed, npix, pix0=pix0)
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    out = O.invert_batch(rrs, nthreads=threads)
    dt = time.perf_counter() - t0
    conv = int(np.sum((out[:, 9] == 0) & (out[:, 8] == 1)))
    return conv / dt, threads, dt, npix, out


def run_reference(args, ws, rank):
    """--impl reference: the reference path on the host cores (the oracle
    port of it, pinned bit for bit to the reference; the reference's own
    build needs sources absent on the GPU host), cold start -- the method
    the reference runs -- on pixels of the same 8192 x 8192 scene."""
    if rank != 0:
        return
    from oracle import oracle as O
    kind = "reference" if O.reference_available() else "port"
    threads = os.cpu_count() or 1
    n = args.ref_sample
    rrs, _ = O.generate_single(SCENE_SEED, n, pix0=8192 * 4096)
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
            "config": {"workload": "the reference's cold-start method on the 8192x8192 "
                                   "single scene, 4 bands, reqmin 1e-10 kcount 2000 (bounded "
                                   "sample per step)",
                       "sample_pixels": n, "host_threads": threads},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind,
                             "sample": f"{n} pixels of the same generator per step"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def train_network(args, dev):
    """The learned warm start's network, trained on the device by photic's
    own kernels on forward-model samples and converged inversions."""
    from photic_gb300 import surrogate as S
    t0 = time.perf_counter()
    net = S.Surrogate(seed=1)
    x, t = S.training_data(args.train_forward, args.train_inverted, seed=31, device=dev)
    t_data = time.perf_counter() - t0
    hist = S.train(net, x, t, epochs=args.train_epochs, batch=8192, lr=2e-3)
    return net, {"samples": hist["samples"], "epochs": args.train_epochs,
                 "seconds": hist["seconds"], "data_seconds": t_data,
                 "final_loss": hist["loss"][-1]}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="photic", choices=["photic", "reference"])
    ap.add_argument("--side", type=int, default=8192, help="side of the headline scene")
    ap.add_argument("--tiles", type=int, default=4, help="tiles (steps) per scene pass")
    ap.add_argument("--sample", type=int, default=2048, help="pixels re-fitted by the CPU oracle")
    ap.add_argument("--cpu-sample", type=int, default=1 << 20)
    ap.add_argument("--ref-sample", type=int, default=1 << 16)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain pass over the scene")
    ap.add_argument("--gain", type=int, default=1, help="network-gain leg on one tile (0: skip)")
    ap.add_argument("--train-forward", type=int, default=1 << 23)
    ap.add_argument("--train-inverted", type=int, default=1 << 20)
    ap.add_argument("--train-epochs", type=int, default=4)
    ap.add_argument("--polish-iters", type=int, default=25,
                    help="Levenberg-Marquardt steps on each surrogate seed (0: raw prediction)")
    ap.add_argument("--seed-step-scale", type=float, default=0.1,
                    help="initial simplex of a seeded fit, relative to the cold-start steps")
    ap.add_argument("--plain-side", type=int, default=4096,
                    help="side of the plain-method scene leg (0: skip)")
    ap.add_argument("--precision-npix", type=int, default=1 << 20,
                    help="pixels of the precision-policy leg (0: skip)")
    ap.add_argument("--joint-npix", type=int, default=1 << 18,
                    help="pixels of the 4096x4096 temporal grid for the joint-fit leg (0: skip)")
    ap.add_argument("--region-side", type=int, default=96,
                    help="side of the square grid for the spatial-region leg (0: skip)")
    ap.add_argument("--lut-side", type=int, default=4096,
                    help="side of the coherent scene of the lookup-table leg (0: skip)")
    ap.add_argument("--lut-oracle-chains", type=int, default=8,
                    help="chains of the lookup-table leg re-run by the oracle")
    ap.add_argument("--lut-cpu-side", type=int, default=128,
                    help="side of the crop the lookup-table loop runs on one CPU thread")
    ap.add_argument("--glut-side", type=int, default=96,
                    help="side of the coherent scene of the general lookup-table leg (0: skip)")
    ap.add_argument("--glut-cpu-side", type=int, default=20,
                    help="side of the crop the general loop runs on one CPU thread")
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
    from photic_gb300 import surrogate as S

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    pg_ = replicas.init("nccl", dev)
    stream = torch.cuda.current_stream()
    cfg = pg.Config()
    wcfg = pg.Config(seed_step_scale=args.seed_step_scale)
    npix = args.side * args.side
    tiles = args.tiles
    if npix % tiles:
        ap.error("--tiles must divide the scene")
    tile = npix // tiles
    pix0 = replicas.shard_start(rank, npix)
    scene, truth = pg.generate_scene(npix, seed=SCENE_SEED, config=cfg, pix0=pix0, device=dev)
    truth_h = truth[:, 0].cpu().numpy()
    del truth
    fields = ("depth_f64", "status", "evals")
    out = pg.alloc_outputs(npix, dev, fields)
    seeds_all = torch.empty(npix, 6, dtype=torch.float64, device=dev)

    net, train = train_network(args, dev)

    def tile_of(k):
        k %= tiles
        return k, slice(k * tile, (k + 1) * tile)

    inv_ms = []

    def step(i, time_inv=False):
        k, sl = tile_of(i)
        t = scene[sl]
        seeds, _ = net.seeds(t, cfg, polish_iters=args.polish_iters)
        order = pg.fallbacks_first(seeds)
        o = {f: out[f][sl] for f in fields}
        if time_inv:
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        pg.invert(t, wcfg, seeds=seeds, order=order, out=o)
        if time_inv:
            e1.record(stream)
            inv_ms.append((e0, e1))
        seeds_all[sl].copy_(seeds)

    for i in range(args.warmup):
        step(i)
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
    _nvtx(True)
    for i in range(args.steps):
        step(args.warmup + i, time_inv=True)
    _nvtx(False)
    ev1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    barrier()
    pg.sync()
    ms_step = ev0.elapsed_time(ev1) / args.steps
    ms_inv = sum(a.elapsed_time(b) for a, b in inv_ms) / args.steps
    ms_step = replicas.max_over_ranks(ms_step, pg_, dev)

    status = out["status"].cpu().numpy()
    fitted = (status & 0xFF) == 0
    conv = fitted & ((status >> 8) & 1).astype(bool)
    evals = out["evals"].cpu().numpy().astype(np.int64)
    h = out["depth_f64"].cpu().numpy()
    seeds_np = seeds_all.cpu().numpy()
    timed_tiles = [tile_of(args.warmup + i)[0] for i in range(args.steps)]
    conv_per_tile = [int(conv[k * tile:(k + 1) * tile].sum()) for k in range(tiles)]
    evals_per_tile = [float(evals[k * tile:(k + 1) * tile].sum()) for k in range(tiles)]
    timed_pix = sorted(set(timed_tiles))

    # CPU oracle started from the same seeds on a sample of the timed pixels
    sample_frac, warm_stats = 1.0, None
    from oracle import oracle as O
    nthreads = os.cpu_count() or 1
    rng = np.random.default_rng(1)
    pool = np.concatenate([np.arange(k * tile, (k + 1) * tile) for k in timed_pix])
    if rank == 0 and args.sample > 0:
        idx = np.sort(rng.choice(pool, size=min(args.sample, pool.size), replace=False))
        r_np = scene[torch.tensor(idx, device=dev)].cpu().numpy()
        o = O.invert_batch(r_np, seeds=seeds_np[idx], seed_step_scale=args.seed_step_scale,
                           nthreads=nthreads)
        m = (o[:, 9] == 0) & conv[idx]
        warm_stats = oracle_stats(h[idx], o, m)
        warm_stats["seeded_share"] = float(np.mean(~np.isnan(seeds_np[idx, 0])))
        sample_frac = warm_stats["frac_within_1cm"]
    good = float(sum(conv_per_tile[k] for k in timed_tiles)) * sample_frac
    good = replicas.sum_over_ranks(good, pg_, dev)
    value = good / (ms_step * 1e-3 * args.steps)

    # Roofline of the dominant kernel (the inversion, FP64 pipe)
    import ctypes as C
    p64, p32, pmu = np.zeros(1), np.zeros(1), np.zeros(1)
    L.check(L.lib().photic_measure_peaks(p64.ctypes.data_as(C.POINTER(C.c_double)),
                                         p32.ctypes.data_as(C.POINTER(C.c_double)),
                                         pmu.ctypes.data_as(C.POINTER(C.c_double))))
    ev_step = sum(evals_per_tile[k] for k in timed_tiles) / args.steps
    achieved = ev_step * FLOPS_PER_EVAL_F64 / (ms_inv * 1e-3) / 1e12
    roof = {"bound": "fp64-pipe", "achieved": achieved, "peak": float(p64[0]),
            "unit": "TFLOP/s", "frac": achieved / float(p64[0]),
            "traffic": TRAFFIC_BYTES_PER_PIXEL * tile,
            "traffic_note": TRAFFIC_NOTE,
            "kernel": "invert_kernel<PrecF64, 4, 256>",
            "kernel_ms_per_launch": ms_inv, "kernel_share_of_step": ms_inv / ms_step,
            "peak_source": "FP64 FMA rate measured by photic_measure_peaks in this run "
                           "(MEASURED_PEAKS.json holds only the HBM copy and bf16 GEMM peaks)",
            "evals_per_s": ev_step / (ms_inv * 1e-3), "flops_per_eval": FLOPS_PER_EVAL_F64,
            "fp64_instructions_per_eval": FP64_INST_PER_EVAL}

    # Plain cold-start method over the same full scene
    plain = None
    plain_h = None
    if not args.no_plain:
        pout = pg.alloc_outputs(npix, dev, fields)
        pg.invert(scene[:65536], cfg, fields=fields)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for k in range(tiles):
            sl = slice(k * tile, (k + 1) * tile)
            pg.invert(scene[sl], cfg, out={f: pout[f][sl] for f in fields})
        e1.record(stream)
        torch.cuda.synchronize()
        pg.sync()
        t_plain = e0.elapsed_time(e1) * 1e-3
        pst = pout["status"].cpu().numpy()
        pconv = ((pst & 0xFF) == 0) & ((pst >> 8) & 1).astype(bool)
        plain_h = pout["depth_f64"].cpu().numpy()
        pev = pout["evals"].cpu().numpy()
        cold_stats, cold_frac = None, 1.0
        if rank == 0 and args.sample > 0:
            idx = np.sort(rng.choice(npix, size=min(args.sample, npix), replace=False))
            o = O.invert_batch(scene[torch.tensor(idx, device=dev)].cpu().numpy(),
                               nthreads=nthreads)
            m = (o[:, 9] == 0) & pconv[idx]
            cold_stats = oracle_stats(plain_h[idx], o, m)
            cold_frac = cold_stats["frac_within_1cm"]
        pgood = replicas.sum_over_ranks(float(pconv.sum()) * cold_frac, pg_, dev)
        t_plain_max = replicas.max_over_ranks(t_plain, pg_, dev)
        both = conv & pconv
        dwc = np.abs(h[both] - plain_h[both])
        vs_truth = {"pixels": int(both.sum()),
                    "warm_median_abs_m": float(np.median(np.abs(h[both] - truth_h[both]))),
                    "cold_median_abs_m": float(np.median(np.abs(plain_h[both] - truth_h[both]))),
                    "warm_p90_abs_m": float(np.quantile(np.abs(h[both] - truth_h[both]), 0.9)),
                    "cold_p90_abs_m": float(np.quantile(np.abs(plain_h[both] - truth_h[both]),
                                                        0.9))}
        plain = {"value": pgood / t_plain_max, "unit": UNIT, "seconds": t_plain,
                 "pixels": npix, "converged_share": float(pconv.mean()),
                 "evals_per_pixel": float(pev[pconv].mean()),
                 "oracle_sample": cold_stats,
                 "warm_vs_cold_depth": {
                     "pixels": int(both.sum()),
                     "median_abs_m": float(np.median(dwc)),
                     "p90_abs_m": float(np.quantile(dwc, 0.9)),
                     "frac_within_1cm": float(np.mean(dwc <= 0.01)),
                     "note": "warm and cold fits land on different points of the "
                             "underdetermined solution set; each is checked against the "
                             "oracle started from its own start"},
                 "depth_vs_generator_truth": vs_truth}
        del pout
        torch.cuda.empty_cache()

    warm_evals = float(evals[conv].mean()) if conv.any() else 0.0
    gain = None
    if rank == 0 and args.gain:
        gain = gain_leg(args, dev, net, scene[:tile], conv[:tile], evals[:tile], ms_step)

    # End to end through the public API with host buffers, one full scene pass
    e2e = None
    if rank == 0:
        e2e = e2e_leg(args, dev, net, scene, tile, tiles, sample_frac)

    cpu = None
    if rank == 0 and not args.no_cpu and args.cpu_sample > 0:
        rate, threads, dt, n, _ = cpu_oracle_rate(args.cpu_sample, SCENE_SEED, 8192 * 4096)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{n} pixels of the 8192x8192 scene, cold start (the reference's "
                         f"method), {dt:.1f} s on {threads} threads"}

    plain4096 = None
    if rank == 0 and args.plain_side > 0:
        plain4096 = plain_scene_leg(args, dev)
    precision = None
    if rank == 0 and args.precision_npix > 0:
        precision = precision_leg(args, dev)
    temporal = None
    if rank == 0 and args.joint_npix > 0:
        temporal = temporal_leg(args, dev)
    regions = None
    if rank == 0 and args.region_side > 0:
        regions = region_leg(args, dev)
    serving = None
    if rank == 0 and args.serve_requests > 0:
        serving = serving_leg(args, net)
    lutr = None
    if rank == 0 and args.lut_side > 0:
        lutr = lut_leg(args, dev)
    glut = None
    if rank == 0 and args.glut_side > 0:
        glut = glut_leg(args, dev)
    ncgrid = None
    if rank == 0 and args.nc_side > 0:
        try:
            ncgrid = ncgrid_leg(args, dev, scene)
        except Exception as e:  # the format leg must not cost the headline line
            ncgrid = {"error": f"{type(e).__name__}: {e}"}

    if rank == 0:
        # kernels of this library per step: the surrogate's feature kernel,
        # per 2^20-row chunk its standardisation + 4 GEMMs + de-normalisation,
        # the seed polish and the inversion
        launches = args.steps * (1 + 6 * ((tile + (1 << 20) - 1) >> 20) + 1 + 1)
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64",
                "data": "synthetic (seeded on-device generator, plain-method prior)",
                "config": {"workload": WORKLOAD, "pixels_per_gpu": npix,
                           "pixels_per_step": tile, "precision": "fp64",
                           "l2": "inputs 268 MB per step > L2; compute-bound kernel"},
                "plain_value": plain["value"] if plain else None,
                "warm_over_plain": value / plain["value"] if plain else None,
                "gpu_launches": launches,
                "pixels": {"fitted_share": float(fitted.mean()),
                           "converged_share": float(conv.mean()),
                           "seeded_share": float(np.mean(~np.isnan(seeds_np[fitted, 0]))),
                           "evals_per_pixel_warm": warm_evals},
                "oracle_sample": warm_stats, "roofline": roof, "cpu_baseline": cpu,
                "plain": plain, "network_gain": gain, "train": train,
                "seed_polish_ms_per_step": ms_step - ms_inv,
                "plain_4096x4096": plain4096, "precision": precision,
                "serving": serving, "temporal": temporal,
                "regions": regions, "lut": lutr, "general_lut": glut, "ncgrid": ncgrid, "e2e": e2e,
                "clocks": clk}
        print(json.dumps(line))
    if pg_ is not None:
        pg_.destroy_process_group()


def gain_leg(args, dev, net, rrs, conv_net, evals_net, ms_net):
    """What the trained network earns on one tile: seeds from the raw
    network prediction, and the same Levenberg-Marquardt polish and residual
    test started without the network from the reference's cold-start guess
    (model/samodel.c:2266-2273, 2342-2351, depth 10 m, also 4 m and 25 m);
    each against the network + polish of the timed steps."""
    import torch
    import photic_gb300 as pg
    from photic_gb300 import surrogate as S
    cfg = pg.Config()
    wcfg = pg.Config(seed_step_scale=args.seed_step_scale)
    fields = ("depth_f64", "status", "evals")

    def run(make_seeds):
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        seeds, _ = make_seeds()
        o = pg.invert(rrs, wcfg, seeds=seeds, order=pg.fallbacks_first(seeds), fields=fields)
        e1.record()
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) * 1e-3
        st = o["status"].cpu().numpy()
        c = ((st & 0xFF) == 0) & ((st >> 8) & 1).astype(bool)
        fit = (st & 0xFF) == 0
        sd = seeds.cpu().numpy()
        return {"px_s": float(c.sum()) / t, "seconds": t,
                "seeded_share": float(np.mean(~np.isnan(sd[fit, 0]))),
                "evals_per_pixel": float(o["evals"].cpu().numpy()[c].mean())}

    raw = run(lambda: net.seeds(rrs, cfg, polish_iters=0))
    heur = run(lambda: S.heuristic_seeds(rrs, cfg, polish_iters=args.polish_iters, h_guess=10.0))
    net_polish = {"px_s": float(conv_net.sum()) / (ms_net * 1e-3),
                  "evals_per_pixel": float(evals_net[conv_net].mean())}
    return {"tile_pixels": int(rrs.shape[0]),
            "network_polished": net_polish, "network_raw": raw,
            "heuristic_polished": heur,
            "network_over_heuristic_px_s": net_polish["px_s"] / heur["px_s"],
            "note": "px/s here without the oracle-sample factor; the same polish, residual "
                    "test and simplex scale in both polished rows"}


def e2e_leg(args, dev, net, scene, tile, tiles, sample_frac):
    """The headline through the public API with host buffers: per tile the
    pinned host spectra go to the device, are seeded and fitted, and depth
    and status come back; one full pass over the scene."""
    import torch
    import photic_gb300 as pg
    cfg = pg.Config()
    wcfg = pg.Config(seed_step_scale=args.seed_step_scale)
    host_in = scene.cpu().pin_memory()
    host_depth = torch.empty(scene.shape[0], dtype=torch.float32).pin_memory()
    host_status = torch.empty(scene.shape[0], dtype=torch.int32).pin_memory()
    dev_in = torch.empty(tile, scene.shape[1], dtype=torch.float32, device=dev)
    o = pg.alloc_outputs(tile, dev, ("depth", "status"))
    stream = torch.cuda.current_stream()
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for k in range(tiles):
        sl = slice(k * tile, (k + 1) * tile)
        dev_in.copy_(host_in[sl], non_blocking=True)
        seeds, _ = net.seeds(dev_in, cfg, polish_iters=args.polish_iters)
        pg.invert(dev_in, wcfg, seeds=seeds, order=pg.fallbacks_first(seeds), out=o)
        host_depth[sl].copy_(o["depth"], non_blocking=True)
        host_status[sl].copy_(o["status"], non_blocking=True)
    t1.record(stream)
    torch.cuda.synchronize()
    ms = t0.elapsed_time(t1)
    st = host_status.numpy()
    conv = ((st & 0xFF) == 0) & ((st >> 8) & 1).astype(bool)
    return {"value": float(conv.sum()) * sample_frac / (ms * 1e-3), "unit": UNIT,
            "h2d_bytes_per_step": int(tile * scene.shape[1] * 4),
            "d2h_bytes_per_step": int(tile * 8), "ms_per_step": ms / tiles,
            "note": "one pass over the scene's tiles; per tile H2D of the spectra, seeding, "
                    "the ordered inversion and D2H of depth and status"}


def precision_leg(args, dev):
    """The precision policies on the same 2^20 pixels of the 4096 x 4096
    scene: FP64 (the headline), the FP32 forward model with the
    special-function unit, double-float, and guarded (double-float screening,
    FP64 decisions), each against the FP64 oracle on a sample, with the
    guarded kernel's tally of how its decisions were taken."""
    import torch
    import photic_gb300 as pg
    from photic_gb300 import _lib as L
    from oracle import oracle as O
    n = args.precision_npix
    rrs, _ = pg.generate_scene(n, seed=SEED, pix0=4096 * 1024, device=dev, with_truth=False)
    rng = np.random.default_rng(3)
    idx = np.sort(rng.choice(n, size=min(args.sample, n), replace=False))
    ref = O.invert_batch(rrs[torch.tensor(idx, device=dev)].cpu().numpy(),
                         nthreads=os.cpu_count() or 1)
    stats = torch.zeros(5, dtype=torch.int64, device=dev)
    res = {"workload": f"{n} pixels of the 4096x4096 plain-method scene, cold start"}
    fields = ("depth_f64", "status", "evals")
    for prec in ("fp64", "fp32", "df64", "guarded"):
        cfg = pg.Config(precision=prec)
        pg.invert(rrs[:8192], cfg, fields=fields)
        torch.cuda.synchronize()
        stats.zero_()
        L.check(L.lib().photic_set_guard_stats(stats.data_ptr()))
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        out = pg.invert(rrs, cfg, fields=fields)
        e1.record()
        torch.cuda.synchronize()
        L.check(L.lib().photic_set_guard_stats(None))
        pg.sync()
        t = e0.elapsed_time(e1) * 1e-3
        st = out["status"].cpu().numpy()
        conv = ((st & 0xFF) == 0) & ((st >> 8) & 1).astype(bool)
        h = out["depth_f64"].cpu().numpy()
        m = (ref[:, 9] == 0) & conv[idx]
        s = oracle_stats(h[idx], ref, m)
        ev = out["evals"].cpu().numpy()
        r = {"converged_px_s": float(conv.sum()) / t, "seconds": t,
             "evals_per_s": float(ev.sum()) / t, "oracle_sample": s,
             "converged_px_s_within_1cm": float(conv.sum()) * s["frac_within_1cm"] / t}
        if prec == "guarded":
            g = stats.cpu().numpy().astype(float)
            dec = g[0] + g[1] + g[2]
            r["decisions"] = {"exact_known": g[0] / dec, "screened": g[1] / dec,
                              "deferred_to_fp64": g[2] / dec,
                              "lane_trips_waiting": g[3] / max(g[4], 1.0)}
        res[prec] = r
    del rrs
    torch.cuda.empty_cache()
    return res


def plain_scene_leg(args, dev):
    """The plain cold-start method on the 4096 x 4096 scene (one pass), with
    its CPU-oracle sample."""
    import torch
    import photic_gb300 as pg
    from oracle import oracle as O
    n = args.plain_side * args.plain_side
    rrs, _ = pg.generate_scene(n, seed=SEED, device=dev, with_truth=False)
    cfg = pg.Config()
    fields = ("depth_f64", "status", "evals", "P", "G", "X", "bottom_albedo")
    pg.invert(rrs[:65536], cfg, fields=fields)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    out = pg.invert(rrs, cfg, fields=fields)
    e1.record()
    torch.cuda.synchronize()
    pg.sync()
    t = e0.elapsed_time(e1) * 1e-3
    st = out["status"].cpu().numpy()
    conv = ((st & 0xFF) == 0) & ((st >> 8) & 1).astype(bool)
    h = out["depth_f64"].cpu().numpy()
    rng = np.random.default_rng(2)
    idx = np.sort(rng.choice(n, size=min(args.sample, n), replace=False))
    o = O.invert_batch(rrs[torch.tensor(idx, device=dev)].cpu().numpy(),
                       nthreads=os.cpu_count() or 1)
    m = (o[:, 9] == 0) & conv[idx]
    pgxb = {k: out[f].cpu().numpy()[idx] for k, f in
            (("P", "P"), ("G", "G"), ("X", "X"), ("B", "bottom_albedo"))}
    stats = oracle_stats(h[idx], o, m, pgxb)
    ev = out["evals"].cpu().numpy()
    res = {"workload": f"plain method, {args.plain_side}x{args.plain_side} scene, cold start",
           "converged_px_s_within_1cm": float(conv.sum()) * stats["frac_within_1cm"] / t,
           "seconds": t, "evals_per_s": float(ev.sum()) / t,
           "evals_per_pixel": float(ev[conv].mean()), "oracle_sample": stats}
    del rrs, out
    torch.cuda.empty_cache()
    return res


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
    sub = np.sort(rng.choice(n, size=min(n, 1024), replace=False))
    counts = offs_h[1:] - offs_h[:-1]
    so = np.zeros(len(sub) + 1, dtype=np.int32)
    so[1:] = np.cumsum(counts[sub])
    obs = np.concatenate([np.arange(offs_h[p], offs_h[p + 1]) for p in sub])
    res = {"workload": f"{n} pixels of the 4096x4096 temporal grid, k ~ U{{2..8}}",
           "observations": int(n_obs), "mean_scenes": float(n_obs / n)}
    for layout in ("reference", "scene_b"):
        cfg = pg.Config(layout=layout)
        g = pg.JointGraph(n, n_obs, cfg, fields=("depth_f64", "status", "evals", "P", "G", "X",
                                                 "bottom_albedo"))
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
        tsub = torch.tensor(sub, device=dev)
        m = (ref[:, 9] == 0) & conv[tsub].cpu().numpy()
        first = torch.tensor(offs_h[sub], device=dev, dtype=torch.int64)
        pgxb = {"P": out["P"][first].cpu().numpy(), "G": out["G"][first].cpu().numpy(),
                "X": out["X"][first].cpu().numpy(),
                "B": out["bottom_albedo"][tsub].cpu().numpy()}
        stats = oracle_stats(out["depth_f64"][tsub].cpu().numpy(), ref, m, pgxb)
        stats["note"] = "P, G, X of each pixel's first scene"
        within = stats["frac_within_1cm"]
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
            "oracle_sample": stats,
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
    k = min(24, n)
    blk = grid[:k, :k].contiguous()
    g_blk = pg.region_invert(blk, cfg, fields=("depth_f64", "status", "P", "G", "X",
                                               "bottom_albedo"))
    pg.sync()
    t0 = time.perf_counter()
    ref = O.region_invert_batch(blk.cpu().numpy(), nthreads=os.cpu_count() or 1)
    t_cpu = time.perf_counter() - t0
    fit = (g_blk["status"].cpu().numpy() & 0xFF) == 0
    pgxb = {k: g_blk[f].cpu().numpy() for k, f in
            (("P", "P"), ("G", "G"), ("X", "X"), ("B", "bottom_albedo"))}
    stats = oracle_stats(g_blk["depth_f64"].cpu().numpy(), ref, fit, pgxb)
    within = stats["frac_within_1cm"]
    return {"workload": f"{n}x{n} grid, 3x3 regions per pixel (n = 3R + 3 <= 30 unknowns)",
            "converged_px_s_within_1cm": float(conv.sum().item()) * within / t, "seconds": t,
            "converged_share": float(conv.float().mean().item()),
            "mean_evals": float(out["evals"].float().mean().item()),
            "oracle_sample": stats,
            "cpu_oracle_px_s": k * k / t_cpu, "cpu_threads": os.cpu_count() or 1}


def lut_leg(args, dev):
    """samodel()'s pixel loop with its dynamic lookup table (LUT 1) on a
    spatially coherent scene at the reference's tolerances: the GPU's chains
    against the plain cold-start inversion of the same scene, per-chain
    parity against the oracle run on the same slices (each slice is the
    reference's loop on one thread, pinned bit for bit to the reference's
    samodel()), and that loop's CPU rate on one thread."""
    import ctypes as C
    import torch
    import photic_gb300 as pg
    from oracle import oracle as O
    n = args.lut_side
    cfg = pg.Config.reference_default()
    rrs, _ = pg.generate_field(n, n, seed=SEED + 11, device=dev, with_truth=False)
    small, _ = pg.generate_field(64, 64, seed=SEED + 12, device=dev, with_truth=False)
    pg.lut_invert(small, cfg)  # warm-up
    pg.invert(small, cfg, fields=("status",))
    pg.sync()

    def timed(fn):
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        o = fn()
        e1.record()
        torch.cuda.synchronize()
        pg.sync()
        return o, e0.elapsed_time(e1) * 1e-3

    fields = ("depth_f64", "status", "evals", "P", "G", "X", "bottom_albedo", "K_min")
    # fewer, longer chains: more of each chain's history to serve from, but
    # the kernel lasts as long as its busiest lane
    lanes = int(pg.api.L.lib().photic_lut_default_chains(C.byref(cfg.to_c()))) // 8
    other = {}
    for per_lane in (1, 32):
        o, t = timed(lambda: pg.lut_invert(rrs, cfg, n_chains=per_lane * lanes,
                                           fields=("status",)))
        s_ = o["status"].cpu().numpy()
        sr = o["source"].cpu().numpy()
        f_ = (s_ & 0xFF) == 0
        other[f"{per_lane}_per_lane"] = {"chains": int(o["chain_stats"].shape[0]),
                                         "px_s": float(f_.sum()) / t,
                                         "served_share": float(np.mean(sr[f_] >= 0))}
        del o
    lut, t_lut = timed(lambda: pg.lut_invert(rrs, cfg, fields=fields))
    plain, t_plain = timed(lambda: pg.invert(rrs, cfg, fields=("depth_f64", "status", "evals")))
    st = lut["status"].cpu().numpy()
    src = lut["source"].cpu().numpy()
    fit = (st & 0xFF) == 0
    fitted = fit & (src == -1)
    ev = lut["evals"].cpu().numpy()
    pev = plain["evals"].cpu().numpy()
    pst = plain["status"].cpu().numpy()
    order = lut["order"].cpu().numpy()
    C = int(lut["chain_stats"].shape[0])
    S = order.size
    h = lut["depth_f64"].cpu().numpy()
    # parity: a sample of chains re-run by the oracle on the same slices
    rng = np.random.default_rng(3)
    chains = np.sort(rng.choice(C, size=min(args.lut_oracle_chains, C), replace=False))
    r_np = rrs.cpu().numpy()
    d_all, srv_g, srv_o = [], [], []
    for c in chains:
        sl = order[c * S // C:(c + 1) * S // C]
        o, so, _, _ = O.lut_invert(r_np[sl], n_chains=1, nthreads=1)
        d_all.append(np.abs(h[sl] - o[:, 0]))
        srv_g.append(src[sl] >= 0)
        srv_o.append(so >= 0)
    d = np.concatenate(d_all) if d_all else np.zeros(0)
    # the loop on the host, one chain on one thread (the reference's own
    # schedule with OMP_NUM_THREADS=1), on a bounded crop of the scene
    crop = r_np.reshape(n, n, 4)[:args.lut_cpu_side, :args.lut_cpu_side].reshape(-1, 4)
    t0 = time.perf_counter()
    oc, sc, _, _ = O.lut_invert(crop, n_chains=1, nthreads=1)
    t_cpu = time.perf_counter() - t0
    shallow_cpu = int(np.sum(oc[:, 9] == 0))
    return {"workload": f"{n}x{n} spatially coherent scene (one water mass, smooth depth, "
                        f"three bottom classes, noise 1e-4, 10 % masked), reference "
                        f"tolerances (reqmin 1e-2, konvge 100, kcount 5000), LUT of 16000 "
                        f"slots per chain",
            "chains": C, "shallow_pixels": S, "pixels_per_chain": S / max(C, 1),
            "px_s": float(fit.sum()) / t_lut, "seconds": t_lut,
            "served_share": float(np.mean(src[fit] >= 0)),
            "hot_share_of_fits": float(np.mean((st[fitted] & 0x400) != 0)),
            "evals_per_fit": float(ev[fitted].mean()) if fitted.any() else 0.0,
            "evals_per_pixel": float(ev[fit].mean()),
            "plain_px_s": float(((pst & 0xFF) == 0).sum()) / t_plain, "plain_seconds": t_plain,
            "plain_evals_per_pixel": float(pev[(pst & 0xFF) == 0].mean()),
            "speedup_vs_plain": t_plain / t_lut,
            "other_chain_counts": other,
            "oracle_chains": {"chains": int(len(chains)), "pixels": int(d.size),
                              "identical_depth": float(np.mean(d == 0)) if d.size else None,
                              "median_abs_dH_m": float(np.median(d)) if d.size else None,
                              "served_share_gpu": float(np.mean(np.concatenate(srv_g)))
                              if srv_g else None,
                              "served_share_oracle": float(np.mean(np.concatenate(srv_o)))
                              if srv_o else None},
            "cpu_one_thread": {"px_s": shallow_cpu / t_cpu, "seconds": t_cpu,
                               "served_share": float(np.mean(sc[oc[:, 9] == 0] >= 0)),
                               "sample": f"{args.lut_cpu_side}x{args.lut_cpu_side} corner of "
                                         f"the scene, one chain, the oracle port (pinned bit "
                                         f"for bit to the reference's samodel())"}}


def glut_leg(args, dev):
    """samodel()'s pixel loop with its lookup table in the reference's
    default configuration (3 x 3 regions, sand, seagrass and coral mixed in
    each: model/bam.c:3236-3241, model/common.c:152) on a spatially
    coherent scene at the reference's tolerances: the GPU's chains (eight
    and one per resident warp) against the general fit of every pixel, and
    on a corner crop the loop on one chain against the oracle's (pinned bit
    for bit to the reference's samodel()), whose time is the CPU rate."""
    import ctypes as C
    import torch
    import photic_gb300 as pg
    from oracle import oracle as O
    n = args.glut_side
    cfg = pg.Config.reference_default()
    rrs, _ = pg.generate_field(n, n, seed=SEED + 13, device=dev, with_truth=False)
    grid = rrs.reshape(1, n, n, 4).contiguous()
    small = grid[:, :8, :8].contiguous()
    pg.region_lut_invert(small, cfg, fields=("status",))  # warm-up
    pg.region_fit(small, cfg, fields=("status",))
    pg.sync()

    def timed(fn):
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        o = fn()
        e1.record()
        torch.cuda.synchronize()
        pg.sync()
        return o, e0.elapsed_time(e1) * 1e-3

    fields = ("depth_f64", "status", "evals")
    warps = int(pg.api.L.lib().photic_region_lut_default_chains(C.byref(cfg.to_c()), 1, 2,
                                                                 3)) // 8
    one, t_one = timed(lambda: pg.region_lut_invert(grid, cfg, n_chains=warps, fields=fields))
    lut, t_lut = timed(lambda: pg.region_lut_invert(grid, cfg, fields=fields))
    plain, t_plain = timed(lambda: pg.region_fit(grid, cfg, fields=fields))

    def summary(o, t):
        st = o["status"].cpu().numpy()
        src = o["source"].cpu().numpy()
        ev = o["evals"].cpu().numpy()
        fit = (st & 0xFF) == 0
        fitted = fit & (src == -1)
        return {"chains": int(o["chain_stats"].shape[0]), "px_s": float(fit.sum()) / t,
                "seconds": t, "served_share": float(np.mean(src[fit] >= 0)),
                "hot_share_of_fits": float(np.mean((st[fitted] & 0x400) != 0)),
                "evals_per_pixel": float(ev[fit].mean())}

    pst = plain["status"].cpu().numpy()
    pfit = (pst & 0xFF) == 0
    res = summary(lut, t_lut)
    res.update({"workload": f"{n}x{n} spatially coherent scene, 3x3 regions, sand, seagrass "
                            f"and coral (n = 66 unknowns), reference tolerances, LUT of 16000 "
                            f"slots per chain",
                "one_chain_per_warp": summary(one, t_one),
                "plain_px_s": float(pfit.sum()) / t_plain, "plain_seconds": t_plain,
                "plain_evals_per_pixel": float(plain["evals"].cpu().numpy()[pfit].mean()),
                "speedup_vs_plain": t_plain / t_lut})
    # one chain on a corner crop: the GPU against the oracle, and the
    # oracle's time as the loop's CPU rate on one thread
    k = args.glut_cpu_side
    crop = grid[:, :k, :k].contiguous()
    g1 = pg.region_lut_invert(crop, cfg, n_chains=1, fields=("depth_f64", "status"))
    pg.sync()
    t0 = time.perf_counter()
    oc, sc, _, _ = O.glut_invert(crop.cpu().numpy(), n_spatial=2, n_bottoms=3, n_chains=1,
                                 nthreads=1)
    t_cpu = time.perf_counter() - t0
    f1 = (g1["status"].cpu().numpy() & 0xFF) == 0
    d = np.abs(g1["depth_f64"].cpu().numpy()[f1] - oc[f1, 0])
    s1 = g1["source"].cpu().numpy()
    res["one_chain_crop"] = {"pixels": int(f1.sum()), "identical_depth": float(np.mean(d == 0)),
                             "median_abs_dH_m": float(np.median(d)),
                             "served_share_gpu": float(np.mean(s1[f1] >= 0)),
                             "served_share_oracle": float(np.mean(sc[oc[:, 9] == 0] >= 0))}
    res["cpu_one_thread"] = {"px_s": float(np.sum(oc[:, 9] == 0)) / t_cpu, "seconds": t_cpu,
                             "sample": f"{k}x{k} corner of the scene, one chain, the oracle "
                                       f"port (pinned bit for bit to the reference's "
                                       f"samodel())"}
    return res


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

# FP64 thread instructions per cost evaluation of the seeded headline fit
# (cost + Nelder-Mead bookkeeping): 160.6 G over 307.75 M evaluations in the
# ncu capture of invert_kernel<PrecF64, 4, 256> on a 1024 x 1024 tile
# (profiles/invert_kernel_warm_1024x1024_full.md); issued as 741 lane-slots
# of FP64 warp instructions (70 % of lanes live).
FP64_INST_PER_EVAL = 522

# dram__bytes_read.sum + dram__bytes_write.sum of the same capture
# (76.75 MB + 5.47 MB over 1 048 576 seeded pixels), per pixel: the spectra
# (16 B) and seed vector (48 B) read, depth, status and evaluation count
# (16 B) written -- the algorithm's 80 B, no re-reads.
TRAFFIC_BYTES_PER_PIXEL = (76.754688e6 + 5.472256e6) / 1048576
TRAFFIC_NOTE = ("DRAM bytes per launch scaled by pixels from an ncu capture of this kernel on a "
                "1048576-pixel seeded tile (78.2 B/pixel, against the 80 B/pixel the algorithm "
                "moves: 16 B spectra + 48 B seed read, 16 B written)")


if __name__ == "__main__":
    main()
