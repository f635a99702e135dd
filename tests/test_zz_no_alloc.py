"""pmgb_widom_noalloc: the Widom entry point that allocates nothing.

Some callers cannot let the library call cudaMalloc or cudaFree in the middle of a run.
cudaFree synchronises the whole device, so a host that keeps other work in flight on the
same GPU would stall on it.  A process whose device memory is already reserved by another
framework's caching allocator may have nothing left for the library to allocate.  Those
callers use pmgb_widom_noalloc.  It keeps its per-CTA scratch in a fixed device array and
writes only to the output buffers the caller passes in.

This file is collected last on purpose.  It checks, through the C ABI, that two calls in a
row give the results of the allocating entry point pmgb_widom_device on the same inputs.
"""
from __future__ import annotations

import numpy as np
import pytest

import pmgb
from pmgb import synthetic

pytestmark = pytest.mark.gpu


def test_noalloc_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    cr = synthetic.config1()
    ff = synthetic.forcefield()
    sc = pmgb.replicate(cr, pmgb.replication_factors(cr.box, ff))
    ep = pmgb.setup_Ewald_sum(sc.box, ff.r_cutoff, eps=1e-6)
    ctx = pmgb.Context(0)
    system = pmgb.GPUSystem(sc, pmgb.Frac(synthetic.co2(), sc.box), ff, ep, ctx=ctx)
    # the allocating entry point with per-site distances (image lists change FP32 roundings only),
    # so that the two entry points compute the same sums
    system.set_image_lists(False)
    lib = ctx._lib
    n_per_block, n_blocks = 3001, 5
    dev = torch.device("cuda", 0)

    def run(fn, seed):
        # outputs are the caller's device memory; torch.empty enqueues no kernel
        blocks = torch.empty(4 * n_blocks, dtype=torch.float64, device=dev)
        u = torch.empty(2 * n_per_block * n_blocks, dtype=torch.float64, device=dev)
        ctx.check(fn(system.handle, n_per_block, n_blocks, seed, 298.0, blocks.data_ptr(), u.data_ptr()))
        ctx.synchronize()
        return blocks.cpu().numpy().reshape(n_blocks, 4), u.cpu().numpy().reshape(-1, 2)

    first = None
    for seed in (17, 18):  # two calls in a row through the fixed scratch
        ref_b, ref_u = run(lib.pmgb_widom_device, seed)
        got_b, got_u = run(lib.pmgb_widom_noalloc, seed)
        np.testing.assert_allclose(got_b, ref_b, rtol=1e-12, atol=1e-9)
        np.testing.assert_allclose(got_u, ref_u, rtol=1e-12, atol=1e-9)
        if first is None:
            first = (seed, got_b)
    # the scratch keeps the previous call's contents; a repeat of the first call is unaffected
    again_b, _ = run(lib.pmgb_widom_noalloc, first[0])
    np.testing.assert_allclose(again_b, first[1], rtol=1e-12, atol=1e-9)

    # a request larger than the fixed scratch is refused with a clear message, also where the
    # CTA count would wrap a 64-bit product
    out = torch.empty(4 * n_blocks, dtype=torch.float64, device=dev)
    for npb in (65536 * 256, 2 ** 62):
        with pytest.raises(pmgb.PMGBError, match="fixed scratch"):
            ctx.check(lib.pmgb_widom_noalloc(system.handle, npb, n_blocks, 1, 298.0, out.data_ptr(), None))

    # a system that refines its Boltzmann tail in FP64 needs per-run scratch: the call refuses it
    # instead of returning the unrefined K_H, and works again once refinement is off
    system.set_refine(1e-3)
    with pytest.raises(pmgb.PMGBError, match="refines its Boltzmann tail"):
        ctx.check(lib.pmgb_widom_noalloc(system.handle, n_per_block, n_blocks, 17, 298.0, out.data_ptr(), None))
    system.set_refine(0.0)
    got_b, _ = run(lib.pmgb_widom_noalloc, 17)
    ref_b, _ = run(lib.pmgb_widom_device, 17)
    np.testing.assert_allclose(got_b, ref_b, rtol=1e-12, atol=1e-9)
    assert ctx.device_status() == 0
