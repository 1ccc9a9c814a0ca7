"""A device-side bounded wait that runs out is reported, and nothing else breaks.

Every TMA / tcgen05 wait in the library is bounded: on give-up the CTA sets
the handle's device error word, drains the copies it issued and returns, and
nrs_synchronize reports NRS_ERR_TIMEOUT. Here a real column-fold TMA
pipeline launch is given a barrier that nothing completes (the test hook
nrs_test_expire_next_wait leaves the first CTA's first tile unloaded) with a
short probe limit; the call must come back with the timeout status, and the
same handle must then compute correct results again.
"""
import numpy as np
import pytest
import torch

from numrs_gb300 import _lib as L

pytestmark = pytest.mark.gpu


def test_expired_wait_reports_timeout_and_handle_recovers(K, ora):
    lib = L.load()
    h = K.handle()
    x = torch.empty((4096, 1024), dtype=torch.float32, device="cuda")
    K.fill_random(x, L.RNG_NORMAL, 31, 0.0, 1.0)
    want = ora.axis(0, x.cpu().numpy(), 0)          # SUM along axis 0 (lanes = columns)
    K.synchronize()
    assert lib.nrs_test_expire_next_wait(h, 1 << 12) == L.OK
    out = K.reduce(x, L.SUM, 0)                       # column-fold TMA pipeline
    st = lib.nrs_synchronize(h)
    assert st == L.ERR_TIMEOUT, st
    assert b"bounded wait" in lib.nrs_last_error(h)
    # lanes 64.. were folded by CTAs that never waited on the dead barrier
    got = out.cpu().numpy()
    assert np.array_equal(got[64:].view(np.uint32), want[64:].view(np.uint32))
    # the error word was cleared and the context is healthy: the same call
    # again (hook consumed) gives every lane bit for bit
    again = K.reduce(x, L.SUM, 0)
    assert lib.nrs_synchronize(h) == L.OK
    assert np.array_equal(again.cpu().numpy().view(np.uint32), want.view(np.uint32))
    assert torch.isfinite(K.sum(x)).item()
    assert lib.nrs_synchronize(h) == L.OK


def test_expire_hook_arguments(K):
    lib = L.load()
    assert lib.nrs_test_expire_next_wait(K.handle(), 0) == L.ERR_INVALID
    assert lib.nrs_test_expire_next_wait(None, 5) == L.ERR_INVALID
