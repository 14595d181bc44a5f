"""gqf_bulk_insert_noalloc: bulk_insert for callers that cannot allocate.

Callers such as a serving process with a device budget fixed at start-up, or
a plugin whose host framework owns every device allocation, may not call
cudaMalloc while they run.  This entry point partitions each batch into a
fixed array inside the library instead of growing scratch on demand.  The
tests call it through the C ABI twice in a row and check, after each call,
that the filter is byte-for-byte the one the regular bulk_insert builds from
the same batches (the tolerance of all parity tests here: exact), and that a
batch larger than the fixed array is refused without touching the filter.

Kept in its own file, named to be collected last.
"""
import numpy as np
import pytest

import oracle
from tests.gpu_util import dev, gpu_get

pytestmark = pytest.mark.gpu


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


@pytest.mark.parametrize("nbits", [16, 22])
def test_noalloc_insert_matches_bulk_insert_twice(gq, nbits):
    import torch

    n = int(0.42 * (1 << nbits))
    batches = [oracle.splitmix64(1, n), oracle.skewed_keys(7, n, nbits - 3)]
    probe = np.concatenate([batches[0], batches[1][:1000], oracle.splitmix64(2, 1 << 12)])
    with gq.QF(nbits) as ref, gq.QF(nbits) as na:
        for b in batches:
            kb = dev(b)
            ref.bulk_insert(kb)
            na.bulk_insert_noalloc(kb)
            torch.cuda.synchronize()
            assert np.array_equal(na.export(), ref.export())
            assert np.array_equal(gpu_get(na, probe), gpu_get(ref, probe))
        assert na.status() & ~gq.STATUS_DEFERRED == 0


def test_noalloc_rejects_batches_beyond_its_scratch(gq):
    nbits = 20
    with gq.QF(nbits) as na:
        # 16 MiB of scratch holds about 4.19 million region-local hashes here
        too_many = (16 << 20) // 4
        kb = dev(oracle.splitmix64(5, too_many))
        with pytest.raises(RuntimeError, match="exceeds"):
            na.bulk_insert_noalloc(kb)
        assert np.array_equal(na.export(), oracle.Oracle(nbits).dump())
        na.bulk_insert_noalloc(kb, n=1000)
        assert gpu_get(na, oracle.splitmix64(5, 1000)).min() == 1
