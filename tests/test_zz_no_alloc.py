"""photic_invert_batch_noalloc, the allocation-free inversion.

Some callers cannot allocate device memory while they run -- a serving
process whose pool allocator owns all of HBM, or a pipeline that forbids
cudaMalloc once started -- so the library offers a variant whose only
scratch is a static device array.  This test calls it through the C ABI
twice in a row (the second call must find the array cleared of the first
call's queue position) and checks that both calls give what the ordinary
entry point gives for the same pixels.  It sits in its own file, collected
last, and needs nothing from the other tests, so it passes alone in a fresh
process or after the rest of the suite.
"""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

FIELDS = ("depth", "depth_f64", "P", "G", "X", "bottom_albedo", "model_error", "rrs_error",
          "K_min", "iod", "evals", "evals_kept", "status")


def _call(entry, rrs, cfg):
    import photic_gb300 as pg
    from photic_gb300 import _lib as L
    out = pg.alloc_outputs(rrs.shape[0], rrs.device, FIELDS)
    os_ = pg.api._outputs_struct(out)
    c = cfg.to_c()
    rc = getattr(L.lib(), entry)(C.byref(c), rrs.data_ptr(), rrs.shape[0], rrs.shape[1], 1,
                                 None, C.byref(os_), torch.cuda.current_stream().cuda_stream)
    L.check(rc)
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in out.items()}


@pytest.mark.parametrize("precision", ["fp64", "df64"])
def test_noalloc_matches_allocating_entry_point(gpu, precision):
    cfg = gpu.Config(precision=precision)
    rrs, _ = gpu.generate_scene(3000, seed=4242, config=cfg)
    rrs2, _ = gpu.generate_scene(1500, seed=4343, config=cfg)
    torch.cuda.synchronize()
    for r in (rrs, rrs2):  # two calls in a row through the static scratch
        ref = _call("photic_invert_batch", r, cfg)
        got = _call("photic_invert_batch_noalloc", r, cfg)
        for k in FIELDS:
            # same kernel, same inputs: the per-pixel results are identical
            np.testing.assert_array_equal(got[k], ref[k], err_msg=k)
        assert np.any((got["status"] & 0xFF) == 0)


def test_noalloc_rejects_what_it_cannot_serve(gpu):
    """Guarded precision needs scratch of its own, and kernel-detected errors
    reach the caller only through the status array: both are refused."""
    from photic_gb300 import _lib as L
    rrs, _ = gpu.generate_scene(64, seed=4444)
    torch.cuda.synchronize()
    out = gpu.alloc_outputs(64, rrs.device, ("depth", "status"))
    for precision, drop_status in (("guarded", False), ("fp64", True)):
        o = dict(out)
        if drop_status:
            o.pop("status")
        os_ = gpu.api._outputs_struct(o)
        c = gpu.Config(precision=precision).to_c()
        rc = L.lib().photic_invert_batch_noalloc(C.byref(c), rrs.data_ptr(), 64, 4, 1, None,
                                                 C.byref(os_),
                                                 torch.cuda.current_stream().cuda_stream)
        assert rc == (L.ERR_UNSUPPORTED if precision == "guarded" else L.ERR_INVALID)
