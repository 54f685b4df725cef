"""Serving loop for tile requests: Poisson arrivals of square tiles of
uneven size, admission by free HBM, batched Nelder-Mead with an optional
learned warm start, per-request latency.

The reference has no serving path; this is the GPU-side caller of the
batched inversion (photic_invert_batch) for a stream of tile requests.

Structure
  * :class:`TileScheduler` -- host logic only: arrivals in schedule order,
    FIFO admission while the device-state budget has room, batches of the
    admitted tiles (up to ``max_batch_pixels``; smallest tiles first under
    the ``sjf`` policy, arrival order under ``fifo``), up to ``depth``
    batches in flight, completions taken in whatever order they finish,
    latency bookkeeping.  The clock and the sleep are injectable so the
    logic is testable without a GPU.
  * :class:`GpuTileExecutor` -- device side: a tile's spectra are created
    on the device at admission (the request's state lives in HBM from then
    on), a batch is one concatenation + optional surrogate seeding + one
    persistent-kernel inversion, results come back to pinned host memory.
    Consecutive batches go to different compute streams, so the next
    batch's blocks take the SMs that the previous batch's ragged tail
    leaves idle.

A request's latency is the time from its arrival to the moment the host
sees its batch complete.
"""
from __future__ import annotations

import dataclasses
import math
import time
from collections import deque
from dataclasses import dataclass, field
from typing import Callable, List, Optional, Sequence

import numpy as np

TILE_BANDS = 4


@dataclass
class TileRequest:
    rid: int
    side: int
    arrival: float           # seconds after the start of the run
    seed: int
    admitted: float = math.nan
    launched: float = math.nan
    done: float = math.nan
    batch: int = -1
    converged: int = 0
    fitted: int = 0
    state: dict = field(default_factory=dict, repr=False)

    @property
    def npix(self) -> int:
        return self.side * self.side

    @property
    def latency(self) -> float:
        return self.done - self.arrival


def poisson_schedule(n: int, rate: float = 50.0, side_lo: int = 256, side_hi: int = 4096,
                     seed: int = 20260404) -> List[TileRequest]:
    """n requests with exponential inter-arrival times (mean 1/rate) and
    square sides log-uniform in [side_lo, side_hi]."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, n))
    side = np.exp(rng.uniform(math.log(side_lo), math.log(side_hi), n))
    side = np.clip(np.rint(side), side_lo, side_hi).astype(int)
    return [TileRequest(rid=i, side=int(side[i]), arrival=float(t[i]), seed=int(seed * 1000 + i))
            for i in range(n)]


class TileScheduler:
    """FIFO admission by a byte budget, batching and latency bookkeeping.

    ``executor`` provides ``footprint(npix) -> bytes``, ``admit(req)``,
    ``launch(reqs) -> token``, ``done(token) -> bool`` and
    ``collect(token, reqs)`` (which fills ``converged``/``fitted`` and
    releases the requests' device state)."""

    def __init__(self, executor, budget_bytes: int, max_batch_pixels: int = 1 << 22,
                 depth: int = 2, policy: str = "sjf",
                 clock: Callable[[], float] = time.perf_counter,
                 sleep: Callable[[float], None] = time.sleep, poll: float = 5e-4):
        if budget_bytes <= 0 or max_batch_pixels <= 0 or depth < 1:
            raise ValueError("budget, batch size and depth must be positive")
        if policy not in ("sjf", "fifo"):
            raise ValueError("policy must be 'sjf' or 'fifo'")
        self.policy = policy
        self.ex = executor
        self.budget = int(budget_bytes)
        self.max_batch_pixels = int(max_batch_pixels)
        self.depth = int(depth)
        self.clock = clock
        self.sleep = sleep
        self.poll = poll
        self.used = 0
        self.peak_used = 0
        self.n_batches = 0
        self.rejected: List[TileRequest] = []

    def run(self, schedule: Sequence[TileRequest]) -> List[TileRequest]:
        pending = deque(sorted(schedule, key=lambda r: r.arrival))
        waiting: deque = deque()
        admitted: List[TileRequest] = []
        inflight: List = []         # (token, [requests])
        finished: List[TileRequest] = []
        t0 = self.clock()
        while pending or waiting or admitted or inflight:
            now = self.clock() - t0
            while pending and pending[0].arrival <= now:
                waiting.append(pending.popleft())
            # admission, FIFO: the head waits until its state fits
            while waiting:
                r = waiting[0]
                need = self.ex.footprint(r.npix)
                if need > self.budget:           # can never fit: refuse it
                    waiting.popleft()
                    r.done = now
                    self.rejected.append(r)
                    continue
                if self.used + need > self.budget:
                    break
                waiting.popleft()
                self.used += need
                self.peak_used = max(self.peak_used, self.used)
                r.admitted = now
                self.ex.admit(r)
                admitted.append(r)
            # completions, in the order they finish
            for item in [it for it in inflight if self.ex.done(it[0])]:
                inflight.remove(item)
                tok, reqs = item
                self.ex.collect(tok, reqs)
                now = self.clock() - t0
                for r in reqs:
                    r.done = now
                    self.used -= self.ex.footprint(r.npix)
                    finished.append(r)
            # launches: keep up to `depth` batches in flight
            if self.policy == "sjf":
                admitted.sort(key=lambda r: (r.npix, r.arrival))
            while admitted and len(inflight) < self.depth:
                batch, px = [], 0
                while admitted and (not batch or px + admitted[0].npix <= self.max_batch_pixels):
                    r = admitted.pop(0)
                    batch.append(r)
                    px += r.npix
                now = self.clock() - t0
                for r in batch:
                    r.launched = now
                    r.batch = self.n_batches
                inflight.append((self.ex.launch(batch), batch))
                self.n_batches += 1
            if pending or waiting or admitted or inflight:
                now = self.clock() - t0
                wait = self.poll
                if pending and not (waiting or admitted or inflight):
                    wait = max(0.0, pending[0].arrival - now)
                self.sleep(wait)
        return finished


def report(finished: Sequence[TileRequest], rejected: Sequence[TileRequest] = ()) -> dict:
    """Latency percentiles and throughput of a finished run."""
    if not finished:
        return {"requests": 0, "rejected": len(rejected)}
    lat = np.array([r.latency for r in finished])
    t_first = min(r.arrival for r in finished)
    t_last = max(r.done for r in finished)
    px = sum(r.npix for r in finished)
    conv = sum(r.converged for r in finished)
    span = max(t_last - t_first, 1e-9)
    return {"requests": len(finished), "rejected": len(rejected), "pixels": int(px),
            "makespan_s": span, "px_s": px / span, "converged_px_s": conv / span,
            "converged_share": conv / max(1, sum(r.fitted for r in finished)),
            "latency_p50_s": float(np.quantile(lat, 0.5)),
            "latency_p99_s": float(np.quantile(lat, 0.99)),
            "latency_max_s": float(lat.max()),
            "queue_wait_p50_s": float(np.quantile([r.launched - r.arrival for r in finished], 0.5)),
            "batches": len({r.batch for r in finished})}


class GpuTileExecutor:
    """Device side of the serving loop (one CUDA device, one compute
    stream, one stream for tile creation)."""

    # device bytes per pixel held by an admitted tile: spectra (16), their
    # copy in the batch (16), seeds (48) and residual (4), outputs (8), the
    # network's features and outputs (44) and the inversion's work queue
    BYTES_PER_PIXEL = 144

    def __init__(self, config=None, surrogate=None, mask_frac: float = 0.15,
                 device=None, n_streams: int = 2, polish_iters: int = 25,
                 seed_step_scale: float = 0.1):
        import torch
        from . import api
        self.torch = torch
        self.api = api
        self.cfg = config or api.Config()
        self.net = surrogate
        self.polish_iters = polish_iters
        self.wcfg = dataclasses.replace(self.cfg, seed_step_scale=seed_step_scale)
        self.mask_frac = mask_frac
        self.device = device or torch.device("cuda", torch.cuda.current_device())
        self.streams = [torch.cuda.Stream(self.device) for _ in range(max(1, n_streams))]
        self.create = torch.cuda.Stream(self.device)
        self.n_launched = 0

    def footprint(self, npix: int) -> int:
        return npix * self.BYTES_PER_PIXEL

    def admit(self, r: TileRequest) -> None:
        torch = self.torch
        with torch.cuda.stream(self.create):
            rrs, _ = self.api.generate_scene(r.npix, seed=r.seed, config=self.cfg,
                                             mask_frac=self.mask_frac, device=self.device,
                                             with_truth=False, stream=self.create)
            ev = torch.cuda.Event()
            ev.record(self.create)
        r.state["rrs"] = rrs
        r.state["ready"] = ev

    def launch(self, reqs: List[TileRequest]):
        torch = self.torch
        s = self.streams[self.n_launched % len(self.streams)]
        self.n_launched += 1
        for r in reqs:
            s.wait_event(r.state["ready"])
        with torch.cuda.stream(s):
            rrs = reqs[0].state["rrs"] if len(reqs) == 1 else \
                torch.cat([r.state["rrs"] for r in reqs])
            for r in reqs:
                r.state["rrs"].record_stream(s)
            seeds = order = None
            if self.net is not None:
                seeds, _ = self.net.seeds(rrs, self.cfg, polish_iters=self.polish_iters)
                order = self.api.fallbacks_first(seeds)
            out = self.api.invert(rrs, self.wcfg if seeds is not None else self.cfg,
                                  seeds=seeds, order=order, fields=("depth", "status"),
                                  stream=s)
            st = out["status"]
            fitted = (st & 0xFF) == 0
            conv = fitted & ((st >> 8) & 1).bool()
            offs = np.cumsum([0] + [r.npix for r in reqs])
            seg = torch.tensor(np.repeat(np.arange(len(reqs)), [r.npix for r in reqs]),
                               device=self.device)
            counts = torch.zeros(2, len(reqs), dtype=torch.int64, device=self.device)
            counts[0].index_add_(0, seg, conv.long())
            counts[1].index_add_(0, seg, fitted.long())
            depth_h = torch.empty(int(offs[-1]), dtype=torch.float32, pin_memory=True)
            counts_h = torch.empty(2, len(reqs), dtype=torch.int64, pin_memory=True)
            depth_h.copy_(out["depth"], non_blocking=True)
            counts_h.copy_(counts, non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(s)
        # keep the batch's device tensors alive until the event completes
        return {"event": ev, "stream": s, "depth": depth_h, "counts": counts_h, "offs": offs,
                "keep": (rrs, seeds, order, out, counts)}

    def done(self, tok) -> bool:
        return tok["event"].query()

    def collect(self, tok, reqs: List[TileRequest]) -> None:
        tok["event"].synchronize()
        self.api.sync(tok["stream"])
        c = tok["counts"].numpy()
        for i, r in enumerate(reqs):
            r.converged = int(c[0, i])
            r.fitted = int(c[1, i])
            r.state["depth"] = tok["depth"][tok["offs"][i]:tok["offs"][i + 1]]
            r.state.pop("rrs", None)
            r.state.pop("ready", None)
        tok.pop("keep", None)


def serve(schedule: Sequence[TileRequest], *, config=None, surrogate=None,
          budget_bytes: Optional[int] = None, budget_frac: float = 0.5,
          max_batch_pixels: int = 1 << 22, depth: int = 2, policy: str = "sjf",
          n_streams: int = 2) -> dict:
    """Run a schedule through the GPU executor; returns :func:`report`
    plus the configuration used.  ``budget_bytes`` defaults to
    ``budget_frac`` of the device memory free at the start."""
    import torch
    ex = GpuTileExecutor(config=config, surrogate=surrogate, n_streams=n_streams)
    if budget_bytes is None:
        free, _ = torch.cuda.mem_get_info()
        budget_bytes = int(free * budget_frac)
    sch = TileScheduler(ex, budget_bytes, max_batch_pixels=max_batch_pixels, depth=depth,
                        policy=policy)
    done = sch.run(schedule)
    torch.cuda.synchronize()
    rep = report(done, sch.rejected)
    rep.update({"budget_bytes": budget_bytes, "peak_admitted_bytes": sch.peak_used,
                "max_batch_pixels": max_batch_pixels, "depth": depth, "policy": policy,
                "streams": n_streams,
                "warm_start": surrogate is not None})
    return rep
