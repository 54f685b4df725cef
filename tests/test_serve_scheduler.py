"""Host logic of the serving loop (photic_gb300/serve.py) with a simulated
clock and a fake executor: FIFO admission by the byte budget, batching
under the pixel cap, in-flight depth, latency bookkeeping."""
import math

import numpy as np
import pytest

from photic_gb300.serve import TileRequest, TileScheduler, poisson_schedule, report


class SimClock:
    def __init__(self):
        self.t = 0.0

    def now(self):
        return self.t

    def sleep(self, dt):
        self.t += max(dt, 1e-4)


class FakeExecutor:
    """Runs batches back to back at `rate` pixels/s on the simulated clock."""

    def __init__(self, clock, rate=1e6, bpp=100):
        self.clock = clock
        self.rate = rate
        self.bpp = bpp
        self.busy_until = 0.0
        self.admitted = []
        self.batches = []
        self.live = 0
        self.peak_live = 0

    def footprint(self, npix):
        return npix * self.bpp

    def admit(self, r):
        self.admitted.append(r.rid)
        self.live += self.footprint(r.npix)
        self.peak_live = max(self.peak_live, self.live)

    def launch(self, reqs):
        px = sum(r.npix for r in reqs)
        start = max(self.clock.now(), self.busy_until)
        self.busy_until = start + px / self.rate
        self.batches.append([r.rid for r in reqs])
        return self.busy_until

    def done(self, tok):
        return self.clock.now() >= tok

    def collect(self, tok, reqs):
        for r in reqs:
            r.fitted = r.npix
            r.converged = r.npix - 1
            self.live -= self.footprint(r.npix)


def _run(schedule, budget, **kw):
    clk = SimClock()
    ex = FakeExecutor(clk)
    sch = TileScheduler(ex, budget, clock=clk.now, sleep=clk.sleep, **kw)
    done = sch.run(schedule)
    return clk, ex, sch, done


def test_schedule_distribution():
    s = poisson_schedule(4000, rate=50.0, seed=7)
    gaps = np.diff([0.0] + [r.arrival for r in s])
    assert abs(gaps.mean() - 1 / 50.0) < 0.002
    sides = np.array([r.side for r in s])
    assert sides.min() >= 256 and sides.max() <= 4096
    # log-uniform: the median side is near sqrt(256 * 4096) = 1024
    assert 900 < np.median(sides) < 1150
    assert poisson_schedule(5, seed=3)[2].side == poisson_schedule(5, seed=3)[2].side


def test_all_finish_in_fifo_admission_order():
    s = poisson_schedule(40, rate=50.0, side_lo=64, side_hi=512, seed=11)
    clk, ex, sch, done = _run(s, budget=10 ** 12, policy="fifo")
    assert len(done) == 40 and not sch.rejected
    assert ex.admitted == sorted(ex.admitted)
    flat = [rid for b in ex.batches for rid in b]
    assert flat == list(range(40))          # FIFO batches
    for r in done:
        assert r.arrival <= r.admitted <= r.launched <= r.done
        assert r.latency > 0


def test_sjf_launches_small_tiles_first():
    sides = [300, 50, 200, 20, 100]
    s = [TileRequest(rid=i, side=sd, arrival=0.0, seed=i) for i, sd in enumerate(sides)]
    clk, ex, sch, done = _run(s, budget=10 ** 12, max_batch_pixels=1, depth=1)
    assert [b[0] for b in ex.batches] == [3, 1, 4, 2, 0]
    lat = {r.rid: r.latency for r in done}
    assert lat[3] < lat[1] < lat[4] < lat[2] < lat[0]


def test_budget_bounds_device_state():
    s = [TileRequest(rid=i, side=100, arrival=0.001 * i, seed=i) for i in range(20)]
    budget = 3 * 100 * 100 * 100 + 5           # room for three tiles
    clk, ex, sch, done = _run(s, budget=budget)
    assert len(done) == 20
    assert ex.peak_live <= budget and sch.peak_used <= budget
    assert sch.used == 0


def test_oversize_request_is_refused():
    s = [TileRequest(rid=0, side=1000, arrival=0.0, seed=0),
         TileRequest(rid=1, side=10, arrival=0.0, seed=1)]
    clk, ex, sch, done = _run(s, budget=10 ** 6)
    assert [r.rid for r in sch.rejected] == [0]
    assert [r.rid for r in done] == [1]


def test_batch_pixel_cap_and_depth():
    s = [TileRequest(rid=i, side=64, arrival=0.0, seed=i) for i in range(10)]
    clk, ex, sch, done = _run(s, budget=10 ** 12, max_batch_pixels=3 * 64 * 64, depth=2)
    assert all(len(b) <= 3 for b in ex.batches)
    assert sum(len(b) for b in ex.batches) == 10
    # a single tile larger than the cap still goes out, alone
    s = [TileRequest(rid=0, side=200, arrival=0.0, seed=0)]
    clk, ex, sch, done = _run(s, budget=10 ** 12, max_batch_pixels=100)
    assert ex.batches == [[0]]


def test_report_numbers():
    s = [TileRequest(rid=i, side=100, arrival=float(i), seed=i) for i in range(4)]
    clk, ex, sch, done = _run(s, budget=10 ** 12)
    rep = report(done)
    assert rep["requests"] == 4 and rep["pixels"] == 40000
    # each tile runs alone at 1e6 px/s: 10 ms of service, no queueing
    assert rep["latency_p50_s"] == pytest.approx(0.01, abs=2e-3)
    assert rep["converged_share"] == pytest.approx(9999 / 10000)
    assert math.isfinite(rep["px_s"])


def test_invalid_arguments():
    with pytest.raises(ValueError):
        TileScheduler(FakeExecutor(SimClock()), 0)
