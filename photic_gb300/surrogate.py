"""The learned warm start: host side of the surrogate MLP (include/photic.h,
photic_surrogate_*).  The network maps observed Rrs (4 bands) and the
subsurface sun / view zenith to (ln P, ln G, ln X, B, H); its prediction
seeds the plain Nelder-Mead fit (photic_invert_batch with d_seeds), which
still converges to the plain tolerance.  Pixels whose seed does not
reproduce the measured spectrum to within 3 sigma of the noise keep the
cold multi-start.

Training data come from photic itself: forward-model samples of the
synthetic prior (the on-device generator) and converged inversions.
"""
from __future__ import annotations

import ctypes as C
import time
from typing import Optional

import numpy as np
import torch

from . import _lib as L
from .api import Config, _stream_handle, generate_scene, invert

NOISE_SIGMA = 2.0e-4


class Surrogate:
    """Owns one network on the current CUDA device."""

    def __init__(self, seed: int = 1):
        h = C.c_void_p()
        L.check(L.lib().photic_surrogate_create(C.byref(h), seed))
        self.h = h
        self.n_params = int(L.lib().photic_surrogate_num_params())

    def close(self):
        if self.h is not None and self.h.value:
            L.lib().photic_surrogate_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> np.ndarray:
        p = np.zeros(self.n_params, dtype=np.float32)
        L.check(L.lib().photic_surrogate_params(self.h, p.ctypes.data, self.n_params, 0))
        return p

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        L.check(L.lib().photic_surrogate_params(self.h, p.ctypes.data, self.n_params, 1))

    def grads(self, x: torch.Tensor, t: torch.Tensor):
        g = torch.empty(self.n_params, dtype=torch.float32, device=x.device)
        loss = torch.zeros(1, dtype=torch.float32, device=x.device)
        L.check(L.lib().photic_surrogate_grads(self.h, x.data_ptr(), t.data_ptr(), x.shape[0],
                                               g.data_ptr(), loss.data_ptr(),
                                               _stream_handle(None)))
        return g, loss

    def train_step(self, x: torch.Tensor, t: torch.Tensor, lr: float,
                   loss: Optional[torch.Tensor] = None) -> None:
        L.check(L.lib().photic_surrogate_train_step(
            self.h, x.data_ptr(), t.data_ptr(), x.shape[0], lr,
            loss.data_ptr() if loss is not None else None, _stream_handle(None)))

    def infer(self, x: torch.Tensor) -> torch.Tensor:
        y = torch.empty(x.shape[0], 5, dtype=torch.float32, device=x.device)
        L.check(L.lib().photic_surrogate_infer(self.h, x.data_ptr(), x.shape[0], y.data_ptr(),
                                               _stream_handle(None)))
        return y

    def seeds(self, rrs: torch.Tensor, config: Optional[Config] = None,
              resid_max: float = 3.0 * NOISE_SIGMA, polish_iters: int = 0):
        """Start vectors [npix, 6] (NaN in column 0 = cold start) and the
        seed's spectral RMS residual [npix].  ``polish_iters`` > 0 refines
        each prediction with that many Levenberg-Marquardt steps on the
        spectral misfit before the residual test."""
        cfg = config or Config()
        npix = rrs.shape[0]
        sd = torch.empty(npix, 6, dtype=torch.float64, device=rrs.device)
        res = torch.empty(npix, dtype=torch.float32, device=rrs.device)
        c = cfg.to_c()
        L.check(L.lib().photic_surrogate_seed_polished(
            self.h, C.byref(c), rrs.data_ptr(), npix, resid_max, int(polish_iters),
            sd.data_ptr(), res.data_ptr(), _stream_handle(None)))
        return sd, res


def heuristic_seeds(rrs: torch.Tensor, config: Optional[Config] = None,
                    resid_max: float = 3.0 * NOISE_SIGMA, polish_iters: int = 25,
                    h_guess: float = 10.0):
    """Seeds from the same Levenberg-Marquardt polish and residual test as
    :meth:`Surrogate.seeds`, started without the network from the
    reference's cold-start guess of B, P, G, X (model/samodel.c:2266-2273,
    2342-2351) at depth ``h_guess`` (and 0.4 / 2.5 times it): the baseline
    that isolates what the trained network adds."""
    cfg = config or Config()
    npix = rrs.shape[0]
    sd = torch.empty(npix, 6, dtype=torch.float64, device=rrs.device)
    res = torch.empty(npix, dtype=torch.float32, device=rrs.device)
    c = cfg.to_c()
    L.check(L.lib().photic_seed_polished_heuristic(
        C.byref(c), rrs.data_ptr(), npix, float(h_guess), resid_max, int(polish_iters),
        sd.data_ptr(), res.data_ptr(), _stream_handle(None)))
    return sd, res


def features(rrs: torch.Tensor, theta_sun: float = 35.0, theta_view: float = 0.0) -> torch.Tensor:
    x = torch.empty(rrs.shape[0], 6, dtype=torch.float32, device=rrs.device)
    x[:, :4] = rrs[:, :4]
    x[:, 4] = theta_sun
    x[:, 5] = theta_view
    return x


def targets(P, G, X, B, H) -> torch.Tensor:
    return torch.stack([torch.log(P), torch.log(G), torch.log(X), B, H], dim=1).float()


def training_data(n_forward: int, n_inverted: int, seed: int = 777, device="cuda"):
    """Forward-model samples of the synthetic prior plus converged
    inversions of further samples (features, targets)."""
    cfg = Config()
    xs, ts = [], []
    if n_forward:
        rrs, tr = generate_scene(n_forward, seed=seed, config=cfg, mask_frac=0.0,
                                 noise_sigma=NOISE_SIGMA, device=device)
        ok = (rrs > 0).all(dim=1)
        H, P, G, X, B = (tr[:, i] for i in range(5))
        xs.append(features(rrs[ok]))
        ts.append(targets(P, G, X, B, H)[ok])
    if n_inverted:
        rrs, _ = generate_scene(n_inverted, seed=seed + 1, config=cfg, mask_frac=0.0,
                                noise_sigma=NOISE_SIGMA, device=device)
        out = invert(rrs, cfg, fields=("depth_f64", "P", "G", "X", "bottom_albedo", "status"))
        st = out["status"]
        # converged fits inside a physical range (a fit on the solution curve
        # of an underdetermined pixel can wander to P -> 0 or H -> 100 m,
        # which would dominate a squared loss)
        P, G, X = out["P"], out["G"], out["X"]
        B, H = out["bottom_albedo"], out["depth_f64"]
        ok = ((st & 0xFF) == 0) & ((st >> 8) & 1).bool() \
            & (P > 1e-4) & (P < 1.0) & (G > 1e-4) & (G < 1.0) & (X > 1e-5) & (X < 0.5) \
            & (B > 0.005) & (B < 1.5) & (H > 0.1) & (H < 60.0)
        xs.append(features(rrs[ok]))
        ts.append(targets(out["P"][ok].double(), out["G"][ok].double(), out["X"][ok].double(),
                          out["bottom_albedo"][ok].double(), out["depth_f64"][ok])
                  )
    return torch.cat(xs), torch.cat(ts)


def train(net: Surrogate, x: torch.Tensor, t: torch.Tensor, epochs: int = 2, batch: int = 8192,
          lr: float = 2e-3, seed: int = 0, log=None) -> dict:
    """Adam over shuffled mini-batches; returns loss history and timing."""
    g = torch.Generator(device=x.device).manual_seed(seed)
    n = x.shape[0]
    steps = 0
    hist = []
    loss = torch.zeros(1, dtype=torch.float32, device=x.device)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for ep in range(epochs):
        perm = torch.randperm(n, device=x.device, generator=g)
        loss.zero_()
        nb = 0
        for i in range(0, n - batch + 1, batch):
            idx = perm[i:i + batch]
            lr_t = lr * (0.5 ** ep)
            net.train_step(x[idx].contiguous(), t[idx].contiguous(), lr_t, loss)
            steps += 1
            nb += 1
        hist.append(float(loss.item()) / max(1, nb))
        if log:
            log(f"epoch {ep}: mean loss {hist[-1]:.4f}")
    torch.cuda.synchronize()
    return {"loss": hist, "steps": steps, "seconds": time.perf_counter() - t0,
            "samples": n}
