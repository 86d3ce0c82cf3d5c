"""Bounded device-side waits run out cleanly.

Every spin of the frame kernels is bounded: the ordered look-back of the
instance and meshlet culls, the grid barrier of the persistent frame kernel
and the mbarrier wait of the TMA-staged resolve.  lh_check_bounded_wait runs
each of them in a one-block launch against a condition that nothing meets
(a predecessor tile that never publishes, a block that never arrives, an
arrival that never comes) with a small poll limit.  The launch must finish,
report LH_FLAG_TIMEOUT in the status word, and leave the context usable --
no fault, no hang.  The same waits with the condition met must not flag.
"""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("which", [0, 1, 2], ids=["lookback", "grid_barrier", "mbarrier"])
def test_bounded_wait_expires_with_flag(native, which):
    import torch
    lh = native
    L = lh.lib()
    words = torch.zeros(8, dtype=torch.int64, device="cuda")
    for satisfied in (0, 1, 0):
        t0 = time.perf_counter()
        st = L.lh_check_bounded_wait(which, 2000, satisfied, words.data_ptr(), None)
        assert st == 0
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        w = words.cpu().numpy().view(np.uint64)
        flags = int(w[3] & np.uint64(0xFFFFFFFF))
        if satisfied:
            assert flags == 0, "wait %d flagged although its condition was met" % which
            assert int(w[4]) == (5 if which == lh.WAIT_LOOKBACK else 1)
        else:
            assert flags == lh.FLAG_TIMEOUT, "wait %d did not report its expiry (flags %#x)" % (which, flags)
            # the look-back counts the missing predecessor as zero
            assert int(w[4]) == 0
        assert dt < 5.0, "a 2,000-poll wait took %.1f s" % dt
    # the context is still usable: an ordinary kernel runs and syncs
    x = torch.arange(1024, device="cuda", dtype=torch.float32)
    assert float(x.sum().item()) == 1023 * 1024 / 2


def test_bounded_wait_rejects_bad_arguments(native):
    import torch
    L = native.lib()
    words = torch.zeros(8, dtype=torch.int64, device="cuda")
    assert L.lh_check_bounded_wait(3, 100, 0, words.data_ptr(), None) == 1
    assert L.lh_check_bounded_wait(0, 0, 0, words.data_ptr(), None) == 1
    assert L.lh_check_bounded_wait(0, (1 << 22) + 1, 0, words.data_ptr(), None) == 1
    assert L.lh_check_bounded_wait(0, 100, 0, None, None) == 1
