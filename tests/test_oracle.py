"""The CPU oracle pinned against the reference (CPU only).

The oracle (oracle/gqf_oracle.c) restates src/gqf.cu on the reference's own
packed format.  It is pinned two ways: against the committed fixtures that
tests/golden/make_golden.py produced from the reference itself, and, where
oracle/_ref can be built (x86 host with the reference tree), live against the
reference on fresh randomised histories.
"""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.fixture(scope="module")
def golden():
    with open(os.path.join(GOLDEN, "golden.json")) as fh:
        meta = json.load(fh)
    arrays = np.load(os.path.join(GOLDEN, "golden.npz"))
    return meta, arrays


def test_hash64_is_a_bijection_under_the_mask():
    L = oracle.lib()
    for nbits in (10, 20, 28):
        mask = (1 << (nbits + 8)) - 1
        keys = oracle.splitmix64(3, 2000)
        h = oracle.hash64(keys, nbits)
        for k, x in zip(keys[:200], h[:200]):
            assert L.hash64(int(k), mask) == int(x)
            assert L.hash64i(int(x), mask) == int(k) & mask
        # only key mod 2^(nbits+8) matters (src/hashutil.cu:132-140)
        assert np.array_equal(h, oracle.hash64(keys & np.uint64(mask), nbits))


@pytest.mark.parametrize("nbits", [10, 12, 14, 16, 20])
def test_oracle_matches_golden_uniform(golden, nbits):
    meta, arrays = golden
    m = meta[f"uniform{nbits}"]
    n = m["n"]
    present = oracle.splitmix64(1, n)
    absent = oracle.splitmix64(2, 1 << nbits)
    f = oracle.Oracle(nbits)
    f.bulk_insert(present)
    d = f.dump()
    assert sha(d) == m["dump_insert_sha256"]
    if f"uniform{nbits}_dump_insert" in arrays:
        assert np.array_equal(d, arrays[f"uniform{nbits}_dump_insert"])
    cp = f.bulk_get(present)
    ca = f.bulk_get(absent)
    assert sha(cp) == m["counts_present_sha256"]
    assert sha(ca) == m["counts_absent_sha256"]
    assert int((ca > 0).sum()) == m["false_positives"]
    assert np.array_equal(np.nonzero(ca)[0].astype(np.uint32), arrays[f"uniform{nbits}_fp_index"])
    f.bulk_delete(present[: n // 2])
    assert sha(f.dump()) == m["dump_delete_sha256"]
    assert sha(f.bulk_get(present)) == m["counts_after_delete_sha256"]


def test_oracle_matches_golden_skew(golden):
    meta, arrays = golden
    nbits = 12
    n = meta["skew12"]["n"]
    k1 = oracle.skewed_keys(5, n, nbits - 2)
    k2 = oracle.skewed_keys(9, n // 4, nbits - 2)
    f = oracle.Oracle(nbits)
    f.bulk_insert_reduce(k1)
    assert np.array_equal(f.dump(), arrays["skew12_dump_reduce"])
    f.bulk_insert(k2)
    assert np.array_equal(f.dump(), arrays["skew12_dump_insert"])
    f.bulk_delete(k1[: n // 3])
    assert np.array_equal(f.dump(), arrays["skew12_dump_delete"])
    probe = np.concatenate([np.unique(k1), oracle.splitmix64(77, 1 << 10)])
    assert np.array_equal(f.bulk_get(probe), arrays["skew12_counts"])


def test_oracle_matches_golden_point(golden):
    _, arrays = golden
    nbits = 10
    f = oracle.Oracle(nbits)
    mask = (1 << (nbits + 8)) - 1
    hs = oracle.splitmix64(21, 600) & np.uint64(mask)
    for h in hs[:100]:
        f.insert_hash(int(h), 3)
    rets = []
    for h in np.concatenate([hs, hs[:300]]):
        r, v = f.insert_not_exists_hash(int(h))
        rets.append(r * 256 + v)
    assert np.array_equal(np.array(rets, dtype=np.uint32), arrays["point10_rets"])
    q = [f.query_hash(int(h))[0] for h in np.concatenate([hs, oracle.splitmix64(22, 200) & np.uint64(mask)])]
    assert np.array_equal(np.array(q, dtype=np.uint64), arrays["point10_query"])
    assert np.array_equal(f.dump(), arrays["point10_dump"])


def test_threaded_oracle_matches_single_thread():
    nbits = 18
    n = int(0.9 * (1 << nbits))
    keys = oracle.splitmix64(4, n)
    a, b = oracle.Oracle(nbits, threads=1), oracle.Oracle(nbits, threads=6)
    for f in (a, b):
        f.bulk_insert(keys)
        f.bulk_delete(keys[: n // 3])
    assert np.array_equal(a.dump(), b.dump())


def _ref_available():
    try:
        return oracle.build_ref() is not None and os.path.exists(oracle.REF_LIB_PATH)
    except Exception:
        return False


@pytest.mark.skipif(not _ref_available(), reason="oracle/_ref needs an x86 host with the reference tree")
@pytest.mark.parametrize("seed", [1, 2, 3, 4])
def test_oracle_matches_reference_live(seed):
    rng = np.random.default_rng(seed)
    for nbits in (10, 13, 16):
        r, o = oracle.RefFilter(nbits), oracle.Oracle(nbits)
        n = 1 << nbits
        for step in range(4):
            kind = rng.integers(0, 4)
            m = int(rng.integers(1, n // 2))
            if kind == 0:
                k = oracle.splitmix64(int(rng.integers(1 << 30)), m)
                r.bulk_insert(k); o.bulk_insert(k)
            elif kind == 1:
                k = oracle.skewed_keys(int(rng.integers(1 << 30)), m, max(4, nbits - 3))
                r.bulk_insert_reduce(k); o.bulk_insert_reduce(k)
            elif kind == 2:
                k = oracle.skewed_keys(int(rng.integers(1 << 30)), m, max(4, nbits - 3))
                r.bulk_insert(k); o.bulk_insert(k)
            else:
                k = oracle.splitmix64(int(rng.integers(1 << 30)), m)
                r.bulk_delete(k); o.bulk_delete(k)
            assert np.array_equal(r.dump(), o.dump()), (nbits, step, kind)
        probe = oracle.splitmix64(seed + 1000, n)
        assert np.array_equal(r.bulk_get(probe), o.bulk_get(probe))
        r.close()


@pytest.mark.parametrize("nbits", [8, 11])
def test_canonical_dump_matches_oracle(nbits):
    """oracle.canonical_dump (the layout as a function of the multiset) equals
    the oracle after insert, counted-insert and delete histories that keep
    every block offset below 255."""
    from collections import Counter

    rng = np.random.default_rng(nbits)
    o = oracle.Oracle(nbits)
    ms = Counter()
    checked = 0
    for step in range(12):
        n = int(rng.integers(1, 1 << (nbits - 2)))
        k = oracle.skewed_keys(int(rng.integers(1 << 30)), n, nbits - 2)
        if step % 3 == 2:
            o.bulk_delete(k)
            for h in oracle.hash64(k, nbits).tolist():
                ms[h] = max(0, ms[h] - 1)
        else:
            (o.bulk_insert_reduce if step % 3 else o.bulk_insert)(k)
            ms.update(oracle.hash64(k, nbits).tolist())
        d = o.dump()
        if oracle.parse_dump(d)[1].max() < 255:
            assert np.array_equal(d, oracle.canonical_dump(nbits, ms)), step
            checked += 1
    assert checked >= 4
    assert oracle.encode_counter(7, 1) == [7] and oracle.encode_counter(0, 3) == [0, 0, 0]
