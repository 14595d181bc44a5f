"""Enumeration and the operations built on it (the reference's iterator,
qf_merge, qf_multi_merge, qf_intersect, qf_inner_product), on the GPU,
against multisets computed on the host and against the oracle."""
from collections import Counter

import numpy as np
import pytest

import oracle
from tests.gpu_util import dev, first_diff, gpu_get

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


@pytest.mark.parametrize("old,new", [(12, 13), (16, 19), (20, 22)])
def test_resize_equals_the_filter_built_at_the_new_size(gq, old, new):
    """Keys that fit nbits + 8 bits (with repeats and one hot key): the
    resized filter is word for word the oracle's filter built at the new size
    from the same multiset, and the handle keeps working for gets and inserts."""
    mask = np.uint64((1 << (old + 8)) - 1)
    n = int(0.8 * (1 << old))
    keys = np.concatenate([oracle.splitmix64(31, n) & mask, oracle.skewed_keys(32, n // 4, old - 4) & mask,
                           np.full(300, 12345, dtype=np.uint64)])
    qf = gq.QF(old)
    try:
        qf.bulk_insert(dev(keys))
        qf.resize(new)
        o = oracle.Oracle(new)
        o.bulk_insert(keys)
        a, b = qf.export(), o.dump()
        assert np.array_equal(a, b), first_diff(a, b)
        more = oracle.splitmix64(33, 1 << (new - 3)) & np.uint64((1 << (new + 8)) - 1)
        qf.bulk_insert(dev(more))
        o.bulk_insert(more)
        assert np.array_equal(qf.export(), o.dump())
        probe = np.concatenate([keys[:5000], oracle.splitmix64(34, 5000)])
        assert np.array_equal(gpu_get(qf, probe), o.bulk_get(probe))
        assert qf.status() & ~gq.STATUS_DEFERRED == 0
    finally:
        qf.close()


def test_resize_keeps_the_low_bits_of_wider_keys(gq):
    """Keys wider than nbits + 8 bits are stored by their low bits: after the
    resize the filter equals one built at the new size from those low bits."""
    old, new = 14, 16
    keys = oracle.splitmix64(35, int(0.7 * (1 << old)))
    low = keys & np.uint64((1 << (old + 8)) - 1)
    qf = gq.QF(old)
    try:
        qf.bulk_insert(dev(keys))
        qf.resize(new)
        o = oracle.Oracle(new)
        o.bulk_insert(low)
        assert np.array_equal(qf.export(), o.dump())
        with pytest.raises(RuntimeError):
            qf.resize(new - 1)
    finally:
        qf.close()

