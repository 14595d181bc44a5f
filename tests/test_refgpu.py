"""The reference's own CUDA build (its kernels compiled from its sources,
baseline/refgpu.py) agrees with the oracle and with the product on small
filters.  Skipped where the cubin was not built (it needs the reference
tree on an x86 host)."""
import numpy as np
import pytest

import oracle
from tests.gpu_util import dev, first_diff, host, zeros_dev

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def refgpu():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from baseline import refgpu

    if not refgpu.available():
        pytest.skip("reference cubin not built here")
    return refgpu


@pytest.mark.parametrize("nbits", [12, 16])
def test_reference_cuda_build_matches_oracle(refgpu, nbits):
    n = int(0.9 * (1 << nbits))
    keys = oracle.splitmix64(1, n)
    absent = oracle.splitmix64(2, 1 << nbits)
    r = refgpu.RefGPU(nbits)
    o = oracle.Oracle(nbits)
    try:
        r.bulk_insert(dev(keys))
        o.bulk_insert(keys)
        a, b = o.dump(), r.dump()
        assert np.array_equal(a, b), first_diff(a, b)
        for probe in (keys, absent):
            out = zeros_dev(probe.size)
            r.bulk_get(dev(probe), out)
            assert np.array_equal(host(out), o.bulk_get(probe))
        r.bulk_delete(dev(keys[: n // 2]))
        o.bulk_delete(keys[: n // 2])
        a, b = o.dump(), r.dump()
        assert np.array_equal(a, b), first_diff(a, b)
    finally:
        r.close()


@pytest.mark.parametrize("nbits", [12, 16])
def test_reference_cuda_reduce_matches_oracle_and_product(refgpu, nbits):
    import cqf_gb300
    from cqf_gb300 import build, synth

    keys = synth.zipf_keys(3, 1 << (nbits + 1), 1 << (nbits - 4))
    r = refgpu.RefGPU(nbits)
    o = oracle.Oracle(nbits)
    try:
        r.bulk_insert_reduce(dev(keys))
        o.bulk_insert_reduce(keys)
        a, b = o.dump(), r.dump()
        assert np.array_equal(a, b), first_diff(a, b)
    finally:
        r.close()
    build.build()
    with cqf_gb300.QF(nbits) as qf:
        qf.bulk_insert_reduce(dev(keys))
        c = qf.export()
        assert np.array_equal(a, c), first_diff(a, c)


@pytest.mark.slow
def test_product_matches_reference_cuda_build_at_2_26_slots_90_percent(refgpu):
    """The headline workload's shape at 2^26 slots: 90% of the slots filled in
    2^22-key bulk_insert batches (256 keys per 4096-quotient region, as at
    2^28 slots with 2^24-key batches), then 2^24 present and 2^24 absent gets
    and 2^24 deletes.  The product's packed filter after the inserts and after
    the deletes, and both count arrays (the false-positive set on the absent
    keys), equal the reference's CUDA build word for word.  At this load the
    short-window rebuild hands regions to the full-window pass, which is
    checked to have run."""
    import torch

    import cqf_gb300
    from cqf_gb300 import build, synth

    build.build()
    nbits, batch, nget = 26, 1 << 22, 1 << 24
    n = int(0.9 * (1 << nbits))
    keys = synth.splitmix64_dev(1, n)
    absent = synth.splitmix64_dev(2, nget)
    r = refgpu.RefGPU(nbits)
    try:
        with cqf_gb300.QF(nbits) as qf:
            scratch = torch.empty(batch, dtype=torch.int64, device="cuda")
            for s in range(0, n, batch):
                m = min(batch, n - s)
                qf.bulk_insert(keys[s:s + m], n=m)
                scratch[:m].copy_(keys[s:s + m])
                r.bulk_insert(scratch, m)  # overwrites its input with hashes
            a, b = qf.export(), r.dump()
            assert np.array_equal(a, b), first_diff(a, b)
            assert qf.counters()["full_window_regions"] > 0
            for probe in (keys[:nget], absent):
                o1, o2 = zeros_dev(nget), zeros_dev(nget)
                qf.bulk_get(probe, o1)
                r.bulk_get(probe, o2)
                torch.cuda.synchronize()
                assert torch.equal(o1, o2)
            for s in range(0, nget, batch):
                qf.bulk_delete(keys[s:s + batch], n=batch)
                scratch.copy_(keys[s:s + batch])
                r.bulk_delete(scratch, batch)
            a, b = qf.export(), r.dump()
            assert np.array_equal(a, b), first_diff(a, b)
            assert qf.status() & ~cqf_gb300.STATUS_DEFERRED == 0
    finally:
        r.close()
