"""Skewed counting on the GPU: bulk_insert_reduce (tile and region merging,
the counted rebuild) and the device k-mer path, bit-exact against the oracle
and against exact multiplicities.

Exact counts identify keys modulo 2^(nbits+8): hash_64 reads only those bits
(src/hashutil.cu:132-140), so keys equal there share a counter in the
reference's filter as in this one.
"""
import numpy as np
import pytest

import oracle
from cqf_gb300 import synth
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


def _dev_u8(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.uint8)).cuda()


@pytest.mark.parametrize("nbits,lr", [(16, 11), (20, 12), (20, 13)])
def test_zipf_reduce_matches_oracle_and_exact_counts(gq, nbits, lr):
    keys = synth.zipf_keys(3, 1 << (nbits + 1), 1 << (nbits - 5))
    o = oracle.Oracle(nbits)
    o.bulk_insert_reduce(keys)
    with gq.QF(nbits, log_region=lr) as qf:
        qf.bulk_insert_reduce(dev(keys))
        a, b = o.dump(), qf.export()
        assert np.array_equal(a, b), first_diff(a, b)
        probe = np.concatenate([np.unique(keys), synth.splitmix64(99, 4096)])
        got = gpu_get(qf, probe)
        assert np.array_equal(got[: np.unique(keys).size], oracle.exact_counts(keys, nbits, np.unique(keys)))
        assert np.array_equal(got, o.bulk_get(probe))
        assert qf.status() & ~gq.STATUS_DEFERRED == 0


def test_reduce_equals_insert(gq):
    """The layout depends only on the multiset: reduce and plain insert of a
    skewed batch (whose hot regions the plain path takes in many rounds)
    give the same filter."""
    nbits = 21
    keys = dev(synth.zipf_keys(5, 1 << 21, 1 << 15))
    with gq.QF(nbits) as a, gq.QF(nbits) as b:
        a.bulk_insert_reduce(keys)
        b.bulk_insert(keys)
        da, db = a.export(), b.export()
        assert np.array_equal(da, db), first_diff(da, db)


def _region_hashes(seed, q_hi, distinct, copies, nbits=None, filler=0):
    """`distinct` hashes with quotients below q_hi, `copies` of each, mixed
    with `filler` single hashes far above the window of region 0 so that the
    copies land in different merge tiles."""
    rng = np.random.default_rng(seed)
    q = rng.integers(0, q_hi, size=distinct * 4).astype(np.uint64)
    r = rng.integers(0, 256, size=distinct * 4).astype(np.uint64)
    h = np.unique((q << np.uint64(8)) | r)
    h = rng.permutation(h)[:distinct]
    parts = [np.repeat(h, copies)]
    if filler:
        fq = rng.integers(q_hi + 4096, 1 << nbits, size=filler).astype(np.uint64)
        fr = rng.integers(0, 256, size=filler).astype(np.uint64)
        parts.append((fq << np.uint64(8)) | fr)
    out = np.concatenate(parts)
    rng.shuffle(out)
    return out


@pytest.mark.parametrize("nbits,lr,q_hi,distinct,copies", [
    (16, 11, 2048, 1300, 2),   # region merge succeeds: one rebuild round
    (16, 13, 8192, 4500, 2),   # too many distinct for the region table: counted rounds
    (16, 11, 2048, 1700, 2),   # the region overflows its window: serial path with counts
])
def test_region_merge_paths_match_oracle(gq, nbits, lr, q_hi, distinct, copies):
    h = _region_hashes(nbits + distinct, q_hi, distinct, copies, nbits, 20000)
    o = oracle.Oracle(nbits)
    o.bulk_insert_reduce(h, key_is_hash=True)
    with gq.QF(nbits, log_region=lr) as qf:
        qf.bulk_insert_reduce(dev(h), flags=gq.QF_NO_LOCK | gq.QF_KEY_IS_HASH)
        a, b = o.dump(), qf.export()
        assert np.array_equal(a, b), first_diff(a, b)
        assert qf.status() & gq.STATUS_FULL == 0
        if distinct == 1700:
            assert qf.counters()["deferred_regions"] >= 1


def test_reduce_bad_key_is_skipped(gq):
    nbits = 12
    h = _region_hashes(1, 1 << nbits, 300, 2)
    bad = np.array([1 << (nbits + 8), (1 << 63) + 5], dtype=np.uint64)
    o = oracle.Oracle(nbits)
    o.bulk_insert_reduce(h, key_is_hash=True)
    with gq.QF(nbits) as qf:
        qf.bulk_insert_reduce(dev(np.concatenate([h, bad])), flags=gq.QF_NO_LOCK | gq.QF_KEY_IS_HASH)
        assert qf.status() & gq.STATUS_BAD_KEY
        assert np.array_equal(o.dump(), qf.export())


@pytest.mark.parametrize("k", [31, 21, 32, 9])
def test_kmers_extract_matches_oracle(gq, k):
    import torch

    reads = synth.dna_reads(4, 700, 150, 1 << 15)
    reads[3, 40] = ord("N")
    reads[7, :] = np.frombuffer(b"acgt" * 37 + b"AC", dtype=np.uint8)
    rd = _dev_u8(reads)
    nk = 150 - k + 1
    out = torch.zeros(700 * nk, dtype=torch.int64, device="cuda")
    gq.kmers_extract(rd, k, out)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy().view(np.uint64), oracle.canonical_kmers(reads, k))


@pytest.mark.parametrize("nbits,read_len,k", [(18, 150, 31), (16, 100, 21), (16, 64, 32)])
def test_kmer_counting_matches_oracle(gq, nbits, read_len, k):
    reads = synth.dna_reads(4, 1 << (nbits - 7), read_len, 1 << (nbits - 3))
    reads[5, 10] = ord("N")
    km = oracle.canonical_kmers(reads, k)
    km = km[km != np.uint64(0xFFFFFFFFFFFFFFFF)]
    o = oracle.Oracle(nbits)
    o.bulk_insert_reduce(km)
    with gq.QF(nbits) as qf:
        qf.bulk_insert_kmers(_dev_u8(reads), k)
        a, b = o.dump(), qf.export()
        assert np.array_equal(a, b), first_diff(a, b)
        u = np.unique(km)
        assert np.array_equal(gpu_get(qf, u), oracle.exact_counts(km, nbits, u))


def test_kmer_shape_errors(gq):
    import torch

    reads = _dev_u8(np.zeros((4, 20), dtype=np.uint8))
    out = torch.zeros(100, dtype=torch.int64, device="cuda")
    with pytest.raises(RuntimeError):
        gq.kmers_extract(reads, 33, out)
    with pytest.raises(RuntimeError):
        gq.kmers_extract(reads, 21, out)
    with gq.QF(10) as qf:
        with pytest.raises(RuntimeError):
            qf.bulk_insert_kmers(reads, 0)


@pytest.mark.slow
def test_two_level_partition_matches_oracle(gq):
    """Batches of at least 2^18 keys into at least 4096 regions take the
    two-level partition (tile histograms, staged scatter, one pass per
    super-bucket).  Plain inserts with out-of-range pre-hashed keys mixed in,
    a skewed counted batch with one hot key, and deletes: each equals the
    oracle word for word, and the bad keys are skipped and flagged."""
    nbits = 24
    o = oracle.Oracle(nbits, threads=8)
    with gq.QF(nbits) as qf:
        h = oracle.hash64(oracle.splitmix64(41, 1 << 20), nbits)
        bad = np.array([1 << (nbits + 8), (1 << 63) + 7, 1 << 40], dtype=np.uint64)
        qf.bulk_insert(dev(np.concatenate([h[:1000], bad, h[1000:]])), flags=gq.QF_NO_LOCK | gq.QF_KEY_IS_HASH)
        o.bulk_insert(h, key_is_hash=True)
        assert qf.status() & gq.STATUS_BAD_KEY
        assert np.array_equal(qf.export(), o.dump())
        skew = np.concatenate([synth.zipf_keys(42, 1 << 21, 1 << 14), np.full(1 << 18, 777, dtype=np.uint64)])
        qf.bulk_insert_reduce(dev(skew))
        o.bulk_insert_reduce(skew)
        a, b = o.dump(), qf.export()
        assert np.array_equal(a, b), first_diff(a, b)
        gone = oracle.hash64(oracle.splitmix64(41, 1 << 19), nbits)
        qf.bulk_delete(dev(gone), flags=gq.QF_NO_LOCK | gq.QF_KEY_IS_HASH)
        o.bulk_delete(gone, key_is_hash=True)
        a, b = o.dump(), qf.export()
        assert np.array_equal(a, b), first_diff(a, b)
        assert qf.status() & gq.STATUS_FULL == 0
