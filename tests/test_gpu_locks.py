"""Failure detection without a GPU fault: a point-API lock left held (as by a
thread that died inside its critical section) makes every operation that
needs it give up after a bounded wait with QF_TIMEOUT and set the filter's
timeout status; nothing hangs, the filter is untouched, and the same calls
succeed once the lock is free."""
import numpy as np
import pytest

import oracle
from tests.gpu_util import dev, host, zeros_dev

pytestmark = pytest.mark.gpu

QF_ITEM_INSERTED, QF_TIMEOUT = 0, 3


@pytest.fixture(scope="module")
def gq():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import cqf_gb300
    from cqf_gb300 import build

    build.build()
    cqf_gb300.load()
    return cqf_gb300


def test_held_lock_times_out_then_recovers(gq):
    import torch

    nbits = 14  # two 8192-slot lock regions (and the tail's)
    rng = np.random.default_rng(1)
    q = rng.integers(100, 8000, size=300).astype(np.uint64)  # lock pair (0, 1)
    hs = np.unique((q << np.uint64(8)) | rng.integers(0, 256, size=q.size).astype(np.uint64))
    flags = gq.QF_KEY_IS_HASH
    with gq.QF(nbits, bulk_config=False) as qf:
        empty = qf.export()
        qf.set_lock_wait(64)
        qf.debug_hold_lock(1)
        rets = torch.zeros(hs.size, dtype=torch.int8, device="cuda")
        qf.point_insert_batch(dev(hs), rets, flags=flags)
        torch.cuda.synchronize()
        assert (rets.cpu().numpy() == QF_TIMEOUT).all()
        assert qf.status() & gq.STATUS_TIMEOUT
        assert np.array_equal(qf.export(), empty)
        counts = zeros_dev(hs.size)
        qf.point_query_batch(dev(hs), counts, flags=flags, concurrent=True)
        assert (host(counts) == 0).all()
        # the lock comes back: the same calls now succeed (with the default
        # wait: 300 threads queue on one lock pair, longer than 64 attempts)
        qf.debug_hold_lock(1, False)
        qf.set_lock_wait(1 << 20)
        qf.clear_status()
        qf.point_insert_batch(dev(hs), rets, flags=flags)
        torch.cuda.synchronize()
        assert (rets.cpu().numpy() == QF_ITEM_INSERTED).all()
        assert qf.status() == 0
        o = oracle.Oracle(nbits)
        o.bulk_insert(hs, key_is_hash=True)
        assert np.array_equal(qf.export(), o.dump())
        qf.point_query_batch(dev(hs), counts, flags=flags, concurrent=True)
        assert (host(counts) == 1).all()


def test_lock_wait_bounds_are_checked(gq):
    with gq.QF(10) as qf:
        with pytest.raises(RuntimeError):
            qf.set_lock_wait(0)
        with pytest.raises(RuntimeError):
            qf.debug_hold_lock(1 << 20)
