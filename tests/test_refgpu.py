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
