"""Enumeration and the operations built on it (the reference's iterator,
qf_merge, qf_multi_merge, qf_intersect, qf_inner_product), on the GPU,
against multisets computed on the host and against the oracle."""
from collections import Counter

import numpy as np
import pytest

import oracle
from tests.gpu_util import dev, first_diff

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


def _multiset(keys, nbits):
    return Counter(oracle.hash64(keys, nbits).tolist())


def _filled(gq, nbits, keys):
    qf = gq.QF(nbits)
    qf.bulk_insert_reduce(dev(keys))
    return qf


@pytest.mark.parametrize("nbits,n", [(10, 700), (14, 12000), (20, 900000)])
def test_enumerate_lists_the_multiset_in_hash_order(gq, nbits, n):
    keys = oracle.skewed_keys(nbits, n, nbits - 2)
    ms = _multiset(keys, nbits)
    with _filled(gq, nbits, keys) as qf:
        h, c = qf.enumerate()
        want = np.array(sorted(ms), dtype=np.uint64)
        assert np.array_equal(h, want)
        assert np.array_equal(c, np.array([ms[int(x)] for x in want], dtype=np.uint64))
        k, c2 = qf.enumerate(as_keys=True)
        assert np.array_equal(oracle.hash64(k, nbits), h) and np.array_equal(c, c2)
        assert np.array_equal(k, k & np.uint64((1 << (nbits + 8)) - 1))
    with gq.QF(nbits) as empty:
        h, c = empty.enumerate()
        assert h.size == 0


def test_merge_and_multi_merge(gq):
    nbits = 14
    A = oracle.skewed_keys(1, 5000, 12)
    B = oracle.skewed_keys(2, 4000, 12)
    C = oracle.splitmix64(3, 3000)
    o = oracle.Oracle(nbits)
    o.bulk_insert_reduce(np.concatenate([A, B]))
    with _filled(gq, nbits, A) as a, _filled(gq, nbits, B) as b, gq.QF(nbits) as out:
        out.merge_from(a, b)
        got, want = out.export(), o.dump()
        assert np.array_equal(got, want), first_diff(got, want)
        a.merge_from(a, b)  # the output may be an input: every input is read first
        o2 = oracle.Oracle(nbits)
        o2.bulk_insert_reduce(np.concatenate([A, A, B]))  # a held A already
        assert np.array_equal(a.export(), o2.dump())
        with _filled(gq, nbits, C) as c, gq.QF(nbits) as out3:
            out3.merge_from(b, c, out)
            o.bulk_insert_reduce(np.concatenate([B, C]))
            got, want = out3.export(), o.dump()
            assert np.array_equal(got, want), first_diff(got, want)


@pytest.mark.parametrize("na,nb", [(14, 14), (12, 14), (14, 12)])
def test_intersect_and_inner_product(gq, na, nb):
    A = oracle.skewed_keys(4, 6000, 11)
    B = np.concatenate([A[:2500], oracle.skewed_keys(5, 3000, 11)])
    ma, mb = _multiset(A, na), _multiset(B, nb)
    # the reference iterates the larger table (ties: the second) and probes the other
    disk, mem, mem_bits = (ma, mb, nb) if na > nb else (mb, ma, na)
    mem_range = 1 << (mem_bits + 8)
    common = {h: c for h, c in disk.items() if h < mem_range and mem.get(h, 0) > 0}
    ip = sum(c * mem[h] for h, c in common.items())
    out_bits = max(na, nb)
    with _filled(gq, na, A) as a, _filled(gq, nb, B) as b, gq.QF(out_bits) as r:
        assert a.inner_product(b) == ip
        r.intersect_from(a, b)
        h, c = r.enumerate()
        assert dict(zip(h.tolist(), c.tolist())) == common
        want = oracle.canonical_dump(out_bits, common)
        got = r.export()
        assert np.array_equal(got, want), first_diff(got, want)
