"""Regenerate the golden fixtures from the reference itself.

Runs the reference's own samodel_optimise / samodel_error / nelmin, compiled
from its sources by oracle/Makefile into oracle/_ref/libphotic_ref.so
(needs the reference sources; run from the repository root):

    make -C oracle all && python tests/golden/make_golden.py [fixture ...]

Inputs are synthetic spectra of the plain-method workload (the reference
publishes no test vectors).  Every fixture stores its inputs next to the
reference outputs, so the tests never need the reference at run time.
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
KEEP = [0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 11, 19, 27]  # H B cost rrs_err Kmin iod evk ev conv status P G X


def single():
    rrs, truth = O.generate_single(20260101, 768, pix0=1000)
    ref = O.invert_batch(rrs, which="reference", nthreads=os.cpu_count())
    # the reference's own hard-coded tolerances on a smaller set
    ref_d = O.invert_batch(rrs[:256], which="reference", reqmin=None, nthreads=os.cpu_count())
    np.savez_compressed(os.path.join(OUT, "single_scene.npz"), rrs=rrs, truth=truth,
                        ref=ref[:, KEEP], ref_default=ref_d[:, KEEP], cols=np.array(KEEP),
                        seed=np.array(20260101), pix0=np.array(1000))


def joint():
    offs, th, rrs, truth = O.generate_joint(20260202, 96)
    ref = O.joint_invert_batch(offs, th, rrs, which="reference", nthreads=os.cpu_count())
    cols = list(range(0, 11)) + list(range(11, 35))
    np.savez_compressed(os.path.join(OUT, "joint.npz"), offsets=offs, theta_sun=th, rrs=rrs,
                        truth=truth, ref=ref[:, cols], cols=np.array(cols))


def cost_and_nelmin():
    rng = np.random.default_rng(7)
    rrs, _ = O.generate_single(20260303, 64, mask_frac=0.0)
    params = np.column_stack([rng.uniform(0.2, 40, 64), rng.uniform(1, 60, 64),
                              rng.uniform(0.2, 2, 64), rng.uniform(0.1, 12, 64),
                              rng.uniform(0.1, 25, 64), rng.uniform(0.05, 6, 64)])
    params[::7] *= -1.0  # the cost takes |x|
    costs, rm, K = [], [], []
    for i in range(64):
        c, r, k = O.cost(rrs[i].astype(np.float64), params[i], which="reference")
        costs.append(c); rm.append(r); K.append(k)
    starts = np.column_stack([np.full(16, 40.0), 400 * rrs[:16, 1], np.ones(16),
                              np.full(16, 0.9), np.full(16, 1.35), 3000 * 0.3108 * rrs[:16, 3]])
    steps = starts * np.array([1.25, 1.5, 0.5, 2, 2, 2])
    nm = [O.nelmin(rrs[i].astype(np.float64), starts[i], steps[i], which="reference")
          for i in range(16)]
    bc = O.band_constants(which="reference")
    np.savez_compressed(os.path.join(OUT, "cost_nelmin.npz"), rrs=rrs, params=params,
                        cost=np.array(costs), rrs_modelled=np.array(rm), K=np.array(K),
                        nm_start=starts, nm_step=steps,
                        nm_xmin=np.array([r[0] for r in nm]),
                        nm_y=np.array([r[1] for r in nm]),
                        nm_counts=np.array([[r[2], r[3], r[4]] for r in nm]),
                        band_constants=bc)


def regions():
    # spatial-region fit (3 x 3 neighbourhoods) of a small grid with masked
    # pixels, edges and a reduced evaluation budget
    nr, nc = 14, 12
    rrs, _ = O.generate_single(20260606, nr * nc, pix0=0, mask_frac=0.15)
    grid = rrs.reshape(nr, nc, rrs.shape[1])
    ref = O.region_invert_batch(grid, kcount=400, which="reference", nthreads=os.cpu_count())
    cols = KEEP + [38, 39]
    np.savez_compressed(os.path.join(OUT, "regions.npz"), grid=grid, ref=ref[:, cols],
                        cols=np.array(cols), kcount=np.array(400))


def bottoms():
    # sand / seagrass / coral mixtures (n_bottoms = 3, the reference's
    # default), pixels alone and with 3 x 3 regions, some with empirical
    # depths; a reduced evaluation budget keeps the fixture quick
    nr, nc = 10, 12
    rrs, truth = O.generate_single(20260707, nr * nc, pix0=4000, mask_frac=0.15)
    grid = rrs.reshape(nr, nc, rrs.shape[1])
    he = truth[:, 0] * np.random.default_rng(9).uniform(0.7, 1.3, truth.shape[0])
    he[::2] = np.nan
    cols = KEEP + [38, 39, 40, 41, 42, 43]
    out = {}
    for ns in (1, 2):
        out[f"ref_s{ns}"] = O.region_invert_batch(grid, kcount=600, n_spatial=ns, n_bottoms=3,
                                                  which="reference", nthreads=os.cpu_count())[:, cols]
        out[f"ref_s{ns}_emp"] = O.region_invert_batch(grid, kcount=600, n_spatial=ns, n_bottoms=3,
                                                      h_empirical=he, which="reference",
                                                      nthreads=os.cpu_count())[:, cols]
    # samodel()'s own call: the reference's hard-coded tolerances
    # (model/samodel.c:2142-2144), for the drop-in test
    for ns in (1, 2):
        out[f"ref_default_s{ns}"] = O.region_invert_batch(grid, reqmin=None, n_spatial=ns,
                                                          n_bottoms=3, which="reference",
                                                          nthreads=os.cpu_count())[:, cols]
    # a two-scene stack of the same place (own sun zeniths and masks), 3 x 3
    # regions and three bottom types: n = 9 + 18 * 3 + 3 * 2 unknowns
    stack = []
    for s in range(2):
        r, _ = O.generate_single(20260808 + s, 6 * 7, pix0=100, mask_frac=0.1,
                                 theta_sun=30.0 + 8.0 * s)
        stack.append(r.reshape(6, 7, r.shape[1]))
    stack = np.stack(stack)
    stack_th = np.array([30.0, 38.0])
    out["ref_stack"] = O.region_invert_batch(stack, theta_sun=stack_th, kcount=600, n_spatial=2,
                                             n_bottoms=3, which="reference",
                                             nthreads=os.cpu_count())[:, cols + [12, 20, 28]]
    np.savez_compressed(os.path.join(OUT, "bottoms.npz"), grid=grid, h_empirical=he,
                        cols=np.array(cols), kcount=np.array(600), stack=stack,
                        stack_theta_sun=stack_th, **out)


def lut():
    """The reference's own samodel() with its dynamic lookup table (LUT 1),
    one thread, reference tolerances, on three spatially coherent scenes:
    64 x 64 ordered by the spectral index alone, 48 x 48 with a noise
    spectrum (R_sigma) so that the spectral angle enters the order, and
    48 x 48 with an empirical depth grid.  Kept grids:
    depth (negative below the datum), model error, bottom albedo, K_min and
    index of optical depth, as samodel() leaves them."""
    keep = [0, 2, 3, 7, 9]
    out = {}
    for name, n, rs in (("plain", 64, None), ("noise", 48, np.array([2e-4, 1.5e-4, 1e-4, 5e-5]))):
        rrs, _ = O.generate_field(20261201 + n, n, n, mask_frac=0.1, noise_sigma=1e-4)
        grid = rrs.reshape(n, n, 4)
        g = O.reference_samodel_grid(grid, r_sigma=rs)
        out[f"{name}_grid"] = grid
        out[f"{name}_ref"] = g[keep]
        if rs is not None:
            out[f"{name}_r_sigma"] = rs
    # an empirical depth grid (negative below the datum, 20 % nodata, some
    # shallower than 1 m): it orders the pixels and starts their fits
    n = 48
    rrs, truth = O.generate_field(20261313, n, n, mask_frac=0.1, noise_sigma=1e-4)
    rng = np.random.default_rng(9)
    emp = (-truth[:, 0] * rng.uniform(0.8, 1.2, n * n)).astype(np.float32)
    emp[rng.random(n * n) < 0.2] = -9999.0
    emp[rng.random(n * n) < 0.05] = -0.5
    grid = rrs.reshape(n, n, 4)
    out["emp_grid"] = grid
    out["emp_empirical"] = emp.reshape(n, n)
    out["emp_ref"] = O.reference_samodel_grid(grid, empirical=emp.reshape(n, n))[keep]
    np.savez_compressed(os.path.join(OUT, "lut.npz"), grids=np.array(keep), **out)


# the general configurations of the lookup-table loop: (name, side,
# n_spatial, n_bottoms, sun zeniths of the scenes, noise, empirical grid)
GLUT_CASES = (("r2b3", 20, 2, 3, (35.0,), False, False),
              ("r1b3", 24, 1, 3, (35.0,), False, False),
              ("r2b2_noise", 18, 2, 2, (35.0,), True, False),
              ("r2b3_emp", 18, 2, 3, (35.0,), False, True),
              ("r2b3_s2", 12, 2, 3, (35.0, 50.0), False, False))


def glut():
    """The reference's own samodel() with LUT 1 in its general
    configurations -- 3 x 3 regions, mixtures of 1-3 bottom types, a noise
    spectrum, an empirical depth grid (15 % nodata), a stack of two scenes
    -- one thread, reference tolerances, on spatially coherent scenes (a
    stack: the same place under two sun zeniths).  Kept grids: all but the
    depth sigma.  The empirical grid's nodata value is positive, so that its
    nodata pixels sort after the pixels with an empirical depth: the
    reference sets h_empirical (which picks sand alone above 8 m) only from
    a pixel with one and never initialises it (model/samodel.c:375,
    960-967), so nodata pixels sorted first would see an undefined value."""
    keep = [0, 2, 3, 4, 5, 6, 7, 8, 9]
    out = {}
    for name, n, ns, nbt, ths, noise, emp in GLUT_CASES:
        grids = np.stack([O.generate_field(20261401 + n, n, n, theta_sun=t, mask_frac=0.1,
                                           noise_sigma=1e-4)[0].reshape(n, n, 4) for t in ths])
        rs = np.array([[2e-4, 1.5e-4, 1e-4, 5e-5]] * len(ths)) if noise else None
        em = None
        if emp:
            _, truth = O.generate_field(20261401 + n, n, n, theta_sun=ths[0])
            rng = np.random.default_rng(11)
            em = (-truth[:, 0] * rng.uniform(0.8, 1.2, n * n)).astype(np.float32)
            em[rng.random(n * n) < 0.15] = 9999.0
            em = em.reshape(n, n)
        g = O.reference_samodel_stack(grids, theta_sun=ths, n_spatial=ns, n_bottoms=nbt,
                                      r_sigma=rs, empirical=em, empirical_nodata=9999.0)
        out[f"{name}_grid"] = grids
        out[f"{name}_theta_sun"] = np.array(ths)
        out[f"{name}_config"] = np.array([ns, nbt])
        out[f"{name}_ref"] = g[keep]
        if rs is not None:
            out[f"{name}_r_sigma"] = rs
        if em is not None:
            out[f"{name}_empirical"] = em
    np.savez_compressed(os.path.join(OUT, "glut.npz"), grids=np.array(keep),
                        cases=np.array([c[0] for c in GLUT_CASES]), **out)


FIXTURES = {"single": single, "joint": joint, "cost_nelmin": cost_and_nelmin,
            "regions": regions, "bottoms": bottoms, "lut": lut, "glut": glut}

if __name__ == "__main__":
    O.build(ref=True)
    if not O.reference_available():
        sys.exit("reference library not built; the reference sources are required")
    for name in (sys.argv[1:] or list(FIXTURES)):
        FIXTURES[name]()
    for f in sorted(os.listdir(OUT)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(OUT, f)), "bytes")
