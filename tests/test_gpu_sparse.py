"""Sparse regions (few keys per region) take the key-by-key path
(k_sparse); the result is the same filter, byte for byte, as the canonical
layout of the multiset, as the oracle's, and as rebuilding every region."""
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


@pytest.mark.parametrize("seed", range(4))
@pytest.mark.parametrize("nbits,lr", [(14, 11), (18, 12), (20, 13)])
def test_small_batches_match_canonical_layout(gq, seed, nbits, lr):
    """Many small batches until the counters fill 85% of the slots.  The
    filter is compared with the canonical layout of the multiset inserted so
    far (oracle.canonical_dump, pinned to the oracle in the CPU tests), and
    with the oracle itself as long as the oracle has not met the reference's
    offset defect (a delete storing an offset above 255 truncated to 8 bits,
    src/gqf.cu:1180-1186, after which the reference's own layout goes
    wrong)."""
    from collections import Counter

    rng = np.random.default_rng(seed * 31 + nbits)
    o = oracle.Oracle(nbits)
    ms = Counter()
    used = 0  # slots the multiset's counters take

    def add(h, d):
        nonlocal used
        old = ms[h]
        new = max(0, old + d)
        ms[h] = new
        used += len(oracle.encode_counter(h & 255, new)) - len(oracle.encode_counter(h & 255, old))

    oracle_sound = True
    inserted = []
    with gq.QF(nbits, log_region=lr) as qf:
        assert 16 <= qf.sparse_max() <= 256
        step = 0
        mark = 0.1  # compare at every further tenth of the slots filled
        while used < 0.85 * (1 << nbits):
            m = int(2 ** rng.uniform(0, np.log2(max(2, (1 << nbits) >> 6))))
            if rng.random() < 0.6 or not inserted:
                k = oracle.splitmix64(int(rng.integers(1 << 40)), m)
                if rng.random() < 0.3:
                    k = np.concatenate([k, k[: m // 2 + 1]])
                    o.bulk_insert_reduce(k)
                    qf.bulk_insert_reduce(dev(k))
                else:
                    o.bulk_insert(k)
                    qf.bulk_insert(dev(k))
                for h in oracle.hash64(k, nbits).tolist():
                    add(h, 1)
                inserted.append(k)
            else:
                pool = np.concatenate(inserted)
                k = pool[rng.integers(0, pool.size, size=min(m, pool.size))]
                o.bulk_delete(k)
                qf.bulk_delete(dev(k))
                for h in oracle.hash64(k, nbits).tolist():
                    add(h, -1)
            step += 1
            if used >= mark * (1 << nbits) or (nbits <= 14 and step % 7 == 0):
                mark = used / (1 << nbits) + 0.1
                want, got = oracle.canonical_dump(nbits, ms), qf.export()
                assert np.array_equal(want, got), (step, first_diff(want, got))
                oracle_sound = oracle_sound and np.array_equal(o.dump(), want)
                if oracle_sound:
                    assert np.array_equal(o.dump(), got)
        want, got = oracle.canonical_dump(nbits, ms), qf.export()
        assert np.array_equal(want, got), first_diff(want, got)
        probe = np.concatenate(inserted[-3:] + [oracle.splitmix64(5, 2048)])
        exp = np.array([ms[h] for h in oracle.hash64(probe, nbits).tolist()], dtype=np.uint64)
        assert np.array_equal(gpu_get(qf, probe), exp)
        assert qf.status() & gq.STATUS_FULL == 0


@pytest.mark.parametrize("sparse", [0, 1 << 20])
def test_all_sparse_or_all_rebuilt_agree(gq, sparse):
    nbits = 16
    keys = oracle.splitmix64(8, int(0.9 * (1 << nbits)))
    with gq.QF(nbits) as a, gq.QF(nbits) as b:
        b.set_sparse_max(sparse)
        for chunk in np.array_split(keys, 5):
            a.bulk_insert(dev(chunk))
            b.bulk_insert(dev(chunk))
        b.bulk_delete(dev(keys[::3]))
        a.bulk_delete(dev(keys[::3]))
        da, db = a.export(), b.export()
        assert np.array_equal(da, db), first_diff(da, db)


def test_sparse_region_past_its_window_is_deferred(gq):
    """A cluster running past a region's window makes the sparse pre-check
    refuse the region; the serial pass applies it, byte-exact."""
    nbits, lr = 14, 11
    reg = 1 << lr
    rng = np.random.default_rng(3)
    q = np.arange(reg - 300, reg + 2600, dtype=np.uint64)  # one key per slot, no gaps
    fill = (q << np.uint64(8)) | rng.integers(0, 256, size=q.size).astype(np.uint64)
    extra = (np.arange(reg - 280, reg - 270, dtype=np.uint64) << np.uint64(8)) | np.uint64(7)
    o = oracle.Oracle(nbits)
    o.bulk_insert(fill, key_is_hash=True)
    o.bulk_insert(extra, key_is_hash=True)
    flags = gq.QF_NO_LOCK | gq.QF_KEY_IS_HASH
    with gq.QF(nbits, log_region=lr) as qf:
        qf.set_sparse_max(0)
        qf.bulk_insert(dev(fill), flags=flags)
        qf.set_sparse_max(32)
        before = qf.counters()["deferred_regions"]
        qf.bulk_insert(dev(extra), flags=flags)  # 10 keys: a sparse region
        assert qf.counters()["deferred_regions"] > before
        a, b = o.dump(), qf.export()
        assert np.array_equal(a, b), first_diff(a, b)


@pytest.mark.parametrize("lr", [11, 12, 13])
def test_region_past_its_short_window_takes_the_full_one(gq, lr):
    """A cluster that runs 500 slots past its region: the first rebuild
    window (the region plus 256 slots) cannot hold the shift, the full one
    (plus 2048, or 1024 for 2048-quotient regions) can; the region is retried
    there, not left to the serial pass, and the filter matches the oracle
    after the insert and after the delete that shifts the cluster back."""
    nbits = 16
    reg = 1 << lr
    rng = np.random.default_rng(lr)
    q = np.arange(reg - 200, reg + 500, dtype=np.uint64)  # one key per slot, no gaps
    fill = (q << np.uint64(8)) | rng.integers(0, 256, size=q.size).astype(np.uint64)
    extra = (np.arange(reg - 180, reg - 170, dtype=np.uint64) << np.uint64(8)) | np.uint64(7)
    o = oracle.Oracle(nbits)
    o.bulk_insert(fill, key_is_hash=True)
    flags = gq.QF_NO_LOCK | gq.QF_KEY_IS_HASH
    with gq.QF(nbits, log_region=lr) as qf:
        qf.set_sparse_max(0)
        qf.bulk_insert(dev(fill), flags=flags)
        c0 = qf.counters()
        o.bulk_insert(extra, key_is_hash=True)
        qf.bulk_insert(dev(extra), flags=flags)
        c1 = qf.counters()
        assert c1["full_window_regions"] > c0["full_window_regions"]
        assert c1["deferred_regions"] == c0["deferred_regions"]
        a, b = o.dump(), qf.export()
        assert np.array_equal(a, b), first_diff(a, b)
        o.bulk_delete(extra, key_is_hash=True)
        qf.bulk_delete(dev(extra), flags=flags)
        c2 = qf.counters()
        assert c2["full_window_regions"] > c1["full_window_regions"]
        assert c2["deferred_regions"] == c0["deferred_regions"]
        a, b = o.dump(), qf.export()
        assert np.array_equal(a, b), first_diff(a, b)
