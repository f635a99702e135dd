"""Failure detection on the device: the kernels' bounded waits report through the status word.

Every wait of the shared-memory staging ring on an mbarrier is bounded in time; when one gives
up, the kernel sets a bit in the context's status word and returns, and the host turns it into
PMGB_ERR_DEVICE_STATUS.  The failure is made without faulting anything: the self-test kernel arms
an mbarrier for a transfer that no copy delivers (no copy is issued, so none is in flight when
the wait gives up) and waits a few microseconds.
"""
from __future__ import annotations

import pytest

import pmgb
from pmgb import synthetic

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_and_reports(ctx):
    assert ctx.device_status() == 0
    # the phase completes: no failure
    ctx.test_bounded_wait(5000, arm=False)
    assert ctx.device_status() == 0
    # nothing completes the phase: the wait gives up after 5 us and the call reports it
    with pytest.raises(pmgb.PMGBError, match="staging wait gave up") as err:
        ctx.test_bounded_wait(5000, arm=True)
    assert err.value.code == -4
    # the status word was read and cleared by that call; the context stays usable
    assert ctx.device_status() == 0
    ctx.test_bounded_wait(5000, arm=False)
    cr, ff = synthetic.config0(), synthetic.forcefield()
    sc = pmgb.replicate(cr, pmgb.replication_factors(cr.box, ff))
    gs = pmgb.GPUSystem(sc, pmgb.Frac(synthetic.ch4(), sc.box), ff, ctx=ctx)
    blocks, _ = gs.widom(1000, 5, 3, 298.0)
    assert blocks.shape == (5, 4)
    assert ctx.device_status() == 0


def test_bounded_wait_rejects_bad_limits(ctx):
    for limit in (0, -1, 10 ** 9):
        with pytest.raises(pmgb.PMGBError, match="limit_ns"):
            ctx.test_bounded_wait(limit, arm=False)
