"""The serving loop on the GPU: every request of a small Poisson schedule
completes, and each tile's depths equal a direct photic_invert_batch of the
same tile bit for bit (a pixel's fit does not depend on its batch), cold
and with the learned warm start."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _direct(pg, r, cfg, net=None, polish_iters=0, seed_step_scale=1.0):
    rrs, _ = pg.generate_scene(r.npix, seed=r.seed, config=cfg, mask_frac=0.15,
                               with_truth=False)
    seeds = None
    if net is not None:
        seeds, _ = net.seeds(rrs, cfg, polish_iters=polish_iters)
        cfg = pg.Config(seed_step_scale=seed_step_scale)
    out = pg.invert(rrs, cfg, seeds=seeds, fields=("depth", "status"))
    pg.sync()
    return out["depth"].cpu().numpy(), out["status"].cpu().numpy()


@pytest.mark.parametrize("warm", [False, True])
def test_serving_matches_direct(gpu, warm):
    from photic_gb300 import serve as S
    from photic_gb300 import surrogate as SU
    pg = gpu
    cfg = pg.Config()
    net = None
    if warm:
        net = SU.Surrogate(seed=3)
        x, t = SU.training_data(1 << 16, 0, seed=5)
        SU.train(net, x, t, epochs=1, batch=4096)
    sched = S.poisson_schedule(10, rate=200.0, side_lo=48, side_hi=200, seed=99)
    ex = S.GpuTileExecutor(config=cfg, surrogate=net)
    sch = S.TileScheduler(ex, budget_bytes=3 * 200 * 200 * ex.BYTES_PER_PIXEL,
                          max_batch_pixels=150 * 150, depth=2)
    done = sch.run(sched)
    torch.cuda.synchronize()
    assert len(done) == 10 and not sch.rejected
    assert sch.n_batches >= 2
    for r in done:
        d, st = _direct(pg, r, cfg, net, ex.polish_iters, ex.wcfg.seed_step_scale)
        np.testing.assert_array_equal(r.state["depth"].numpy(), d)
        conv = ((st & 0xFF) == 0) & ((st >> 8) & 1).astype(bool)
        assert r.converged == int(conv.sum())
        assert r.fitted == int(((st & 0xFF) == 0).sum())
    rep = S.report(done)
    assert rep["requests"] == 10 and rep["latency_p99_s"] >= rep["latency_p50_s"] > 0
