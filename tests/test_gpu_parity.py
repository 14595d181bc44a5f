"""Parity of the CUDA path with the oracle and the reference's golden vectors.

Every comparison is bit-exact: exported filter bytes (the reference's packed
81-byte blocks), per-key counts, and false-positive sets.  The GPU is driven
through the C ABI (include/gqf.h) via ctypes.
"""
import json
import os

import numpy as np
import pytest

import oracle
from tests.gpu_util import dev, first_diff, gpu_get, host, sha, zeros_dev

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


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


@pytest.fixture(scope="module")
def golden():
    with open(os.path.join(GOLDEN, "golden.json")) as fh:
        meta = json.load(fh)
    return meta, np.load(os.path.join(GOLDEN, "golden.npz"))


def _sync():
    import torch

    torch.cuda.synchronize()


@pytest.mark.parametrize("nbits", [10, 12, 14, 16, 20])
@pytest.mark.parametrize("lr", [0, 11, 13])
def test_uniform_matches_reference_golden(gq, golden, nbits, lr):
    meta, arrays = golden
    m = meta[f"uniform{nbits}"]
    n = m["n"]
    present = oracle.splitmix64(1, n)
    absent = oracle.splitmix64(2, 1 << nbits)
    with gq.QF(nbits) as qf:
        if lr:
            qf.set_region_log(lr)
        kp = dev(present)
        qf.bulk_insert(kp)
        d = qf.export()
        assert sha(d) == m["dump_insert_sha256"], first_diff(d, arrays[f"uniform{nbits}_dump_insert"]) \
            if f"uniform{nbits}_dump_insert" in arrays else "dump differs"
        # keys are left unmodified by bulk_insert
        assert np.array_equal(host(kp), present)
        cp = gpu_get(qf, present)
        ca = gpu_get(qf, absent)
        assert sha(cp) == m["counts_present_sha256"]
        assert sha(ca) == m["counts_absent_sha256"]
        assert np.array_equal(np.nonzero(ca)[0].astype(np.uint32), arrays[f"uniform{nbits}_fp_index"])
        assert qf.bulk_get_misses(dev(present)) == 0
        assert qf.bulk_get_misses(dev(absent)) == (1 << nbits) - m["false_positives"]
        qf.bulk_delete(dev(present[: n // 2]))
        assert sha(qf.export()) == m["dump_delete_sha256"]
        assert sha(gpu_get(qf, present)) == m["counts_after_delete_sha256"]
        assert qf.status() & ~gq.STATUS_DEFERRED == 0


def test_skew_matches_reference_golden(gq, golden):
    meta, arrays = golden
    nbits = 12
    n = meta["skew12"]["n"]
    k1 = oracle.skewed_keys(5, n, nbits - 2)
    k2 = oracle.skewed_keys(9, n // 4, nbits - 2)
    with gq.QF(nbits) as qf:
        qf.bulk_insert_reduce(dev(k1))
        d = qf.export()
        assert np.array_equal(d, arrays["skew12_dump_reduce"]), first_diff(d, arrays["skew12_dump_reduce"])
        qf.bulk_insert(dev(k2))
        d = qf.export()
        assert np.array_equal(d, arrays["skew12_dump_insert"]), first_diff(d, arrays["skew12_dump_insert"])
        qf.bulk_delete(dev(k1[: n // 3]))
        d = qf.export()
        assert np.array_equal(d, arrays["skew12_dump_delete"]), first_diff(d, arrays["skew12_dump_delete"])
        probe = np.concatenate([np.unique(k1), oracle.splitmix64(77, 1 << 10)])
        assert np.array_equal(gpu_get(qf, probe), arrays["skew12_counts"])


def _history(seed, nbits, steps):
    rng = np.random.default_rng(seed)
    n = 1 << nbits
    ops = []
    for _ in range(steps):
        kind = int(rng.integers(0, 5))
        m = int(rng.integers(1, max(2, n // 3)))
        s = int(rng.integers(1, 1 << 30))
        if kind == 0:
            ops.append(("insert", oracle.splitmix64(s, m)))
        elif kind == 1:
            ops.append(("insert", oracle.skewed_keys(s, m, max(4, nbits - 3))))
        elif kind == 2:
            ops.append(("reduce", oracle.skewed_keys(s, m, max(4, nbits - 4))))
        elif kind == 3:
            ops.append(("delete", oracle.splitmix64(s, m)))
        else:
            # delete a sample of what may be present
            prev = [k for op, k in ops if op != "delete"]
            if prev:
                pool = np.concatenate(prev)
                ops.append(("delete", pool[rng.integers(0, pool.size, size=min(m, pool.size))]))
    return ops


@pytest.mark.parametrize("seed", range(6))
@pytest.mark.parametrize("nbits,lr", [(11, 11), (13, 11), (14, 12), (16, 13), (17, 11)])
def test_random_histories_match_oracle(gq, seed, nbits, lr):
    o = oracle.Oracle(nbits)
    with gq.QF(nbits, log_region=lr) as qf:
        for step, (op, keys) in enumerate(_history(seed * 7 + nbits, nbits, 6)):
            getattr(o, {"insert": "bulk_insert", "reduce": "bulk_insert_reduce", "delete": "bulk_delete"}[op])(keys)
            getattr(qf, {"insert": "bulk_insert", "reduce": "bulk_insert_reduce", "delete": "bulk_delete"}[op])(dev(keys))
            a, b = o.dump(), qf.export()
            assert np.array_equal(a, b), (step, op, len(keys), first_diff(a, b))
        probe = np.concatenate([oracle.splitmix64(seed + 99, 1 << nbits), oracle.skewed_keys(seed + 5, 4096, 8)])
        assert np.array_equal(o.bulk_get(probe), gpu_get(qf, probe))
        assert qf.status() & ~gq.STATUS_DEFERRED == 0


def _clustered_hashes(seed, nbits, n, q_lo, q_hi):
    """Hashes whose quotients fall in [q_lo, q_hi): builds one long cluster."""
    rng = np.random.default_rng(seed)
    q = rng.integers(q_lo, q_hi, size=n).astype(np.uint64)
    r = rng.integers(0, 256, size=n).astype(np.uint64)
    return (q << np.uint64(8)) | r


def _one_per_quotient(q_lo, q_hi, seed):
    rng = np.random.default_rng(seed)
    q = np.arange(q_lo, q_hi, dtype=np.uint64)
    r = rng.integers(0, 256, size=q.size).astype(np.uint64)
    return (q << np.uint64(8)) | r


@pytest.mark.parametrize("lr", [11, 12])
def test_long_cluster_defers_and_matches_oracle(gq, lr):
    """A push that is not absorbed inside the rebuild window (here ~2900
    slots with no gap, longer than any push window) takes the serial path;
    the result is still the reference's layout, byte for byte."""
    nbits = 14
    reg = 1 << lr
    fill = _one_per_quotient(reg - 300, reg + 2600, 1)  # one key per slot, no gaps
    extra = _clustered_hashes(2, nbits, 100, reg - 300, reg - 250)
    o = oracle.Oracle(nbits)
    with gq.QF(nbits, log_region=lr) as qf:
        for batch in (fill, extra):
            o.bulk_insert(batch, key_is_hash=True)
            qf.bulk_insert(dev(batch), flags=gq.QF_KEY_IS_HASH)
            a, b = o.dump(), qf.export()
            assert np.array_equal(a, b), first_diff(a, b)
        assert qf.status() & gq.STATUS_DEFERRED
        assert oracle.parse_dump(o.dump())[1].max() < 255
        qf.clear_status()
        o.bulk_delete(extra[:60], key_is_hash=True)
        qf.bulk_delete(dev(extra[:60]), flags=gq.QF_KEY_IS_HASH)
        a, b = o.dump(), qf.export()
        assert np.array_equal(a, b), first_diff(a, b)
        assert qf.status() & gq.STATUS_DEFERRED


def _exact_offsets(occ: np.ndarray, run: np.ndarray) -> np.ndarray:
    """Block offsets recomputed from the bits: the k-th occupied quotient's
    run ends at the k-th runend; offset(b) = max(0, end of the last run of a
    quotient < 64 b, minus 64 b, plus 1)."""
    qs = np.nonzero(np.unpackbits(occ.view(np.uint8), bitorder="little"))[0]
    ends = np.nonzero(np.unpackbits(run.view(np.uint8), bitorder="little"))[0]
    assert qs.size == ends.size
    out = np.zeros(occ.size, dtype=np.int64)
    for b in range(1, occ.size):
        k = np.searchsorted(qs, 64 * b) - 1
        if k >= 0:
            out[b] = max(0, int(ends[k]) - 64 * b + 1)
    return out


def test_offsets_beyond_255_after_delete(gq):
    """Known reference defect: a delete inside a cluster whose block offset
    exceeds 255 stores the offset truncated to 8 bits (src/gqf.cu:1180-1186),
    which corrupts the reference's later lookups.  The device keeps exact
    offsets and exports the saturated 255 the reference's insert path
    stores; slots, occupieds and runends stay identical and counts stay
    right."""
    nbits = 14
    h = _clustered_hashes(3, nbits, 3000, 100, 600)  # offsets reach ~2500
    h2 = _clustered_hashes(4, nbits, 800, 300, 700)
    o = oracle.Oracle(nbits)
    truth = {}
    with gq.QF(nbits, log_region=11) as qf:
        for batch in (h, h2):
            o.bulk_insert(batch, key_is_hash=True)
            qf.bulk_insert(dev(batch), flags=gq.QF_KEY_IS_HASH)
            for x in batch:
                truth[int(x)] = truth.get(int(x), 0) + 1
        a, b = o.dump(), qf.export()
        assert np.array_equal(a, b), first_diff(a, b)
        o.bulk_delete(h[:1500], key_is_hash=True)
        qf.bulk_delete(dev(h[:1500]), flags=gq.QF_KEY_IS_HASH)
        for x in h[:1500]:
            truth[int(x)] -= 1
        A, B = oracle.parse_dump(o.dump()), oracle.parse_dump(qf.export())
        for i in (0, 2, 3, 4):  # metadata, occupieds, runends, slots
            assert np.array_equal(A[i], B[i])
        assert (A[1] != B[1]).any()  # the reference's offsets are corrupted here
        assert np.array_equal(B[1], np.minimum(255, _exact_offsets(B[2], B[3])))
        keys = np.array(sorted(truth), dtype=np.uint64)
        out = zeros_dev(keys.size)
        qf.bulk_get_async(dev(keys), out, keys.size, flags=gq.QF_KEY_IS_HASH)
        assert np.array_equal(host(out), np.array([truth[int(k)] for k in keys], dtype=np.uint64))


def test_key_is_hash_out_of_range_is_reported(gq):
    nbits = 10
    with gq.QF(nbits) as qf:
        bad = np.array([1 << 20, (1 << 18) + 5], dtype=np.uint64)
        good = oracle.splitmix64(5, 100) & np.uint64((1 << 18) - 1)
        qf.bulk_insert(dev(np.concatenate([bad, good])), flags=gq.QF_KEY_IS_HASH)
        assert qf.status() & gq.STATUS_BAD_KEY
        o = oracle.Oracle(nbits)
        o.bulk_insert(good, key_is_hash=True)
        assert np.array_equal(o.dump(), qf.export())


def test_serial_device_path_matches_oracle(gq):
    """The single-key device algorithms (point API, fallback) alone."""
    import torch

    nbits = 12
    rng = np.random.default_rng(11)
    o = oracle.Oracle(nbits)
    with gq.QF(nbits) as qf:
        mask = np.uint64((1 << (nbits + 8)) - 1)
        # ~75% of xnslots: offsets stay below 255, where deletes are exact
        hs = oracle.splitmix64(12, 2600) & mask
        dup = hs[rng.integers(0, hs.size, size=900)]
        for batch in (hs, dup):
            for h in batch:
                o.insert_hash(int(h), 1)
            qf.serial_apply(dev(batch), 0)
            torch.cuda.synchronize()
            a, b = o.dump(), qf.export()
            assert np.array_equal(a, b), first_diff(a, b)
        assert oracle.parse_dump(o.dump())[1].max() < 255
        rm = np.concatenate([hs[:1200], dup[:500]])
        for h in rm:
            o.remove_hash(int(h), 1)
        qf.serial_apply(dev(rm), 1)
        a, b = o.dump(), qf.export()
        assert np.array_equal(a, b), first_diff(a, b)


def test_point_api_matches_reference_golden(gq, golden):
    """point_insert_not_exists / point_query, one key per launch so the
    sequence is the reference's sequential one."""
    import torch

    _, arrays = golden
    nbits = 10
    mask = np.uint64((1 << (nbits + 8)) - 1)
    hs = oracle.splitmix64(21, 600) & mask
    with gq.QF(nbits) as qf:
        # count-3 entries for the first 100 hashes, as the golden run made them
        qf.bulk_insert(dev(np.repeat(hs[:100], 3)), flags=gq.QF_KEY_IS_HASH)
        seq = np.concatenate([hs, hs[:300]])
        kd = dev(seq)
        rets = torch.zeros(seq.size, dtype=torch.int8, device="cuda")
        vals = torch.zeros(seq.size, dtype=torch.uint8, device="cuda")
        for i in range(seq.size):
            qf.point_insert_not_exists_batch(kd[i:], rets[i:], vals[i:], n=1, flags=gq.QF_KEY_IS_HASH)
        got = rets.cpu().numpy().astype(np.uint32) * 256 + vals.cpu().numpy().astype(np.uint32)
        assert np.array_equal(got, arrays["point10_rets"])
        q = np.concatenate([hs, oracle.splitmix64(22, 200) & mask])
        counts = zeros_dev(q.size)
        qf.point_query_batch(dev(q), counts, flags=gq.QF_KEY_IS_HASH)
        assert np.array_equal(host(counts), arrays["point10_query"])
        counts2 = zeros_dev(q.size)
        qf.point_query_batch(dev(q), counts2, flags=gq.QF_KEY_IS_HASH, concurrent=True)
        assert np.array_equal(host(counts2), arrays["point10_query"])
        d = qf.export()
        assert np.array_equal(d, arrays["point10_dump"]), first_diff(d, arrays["point10_dump"])


@pytest.mark.parametrize("nbits", [12, 16])
def test_concurrent_point_inserts_match_bulk(gq, nbits):
    """point_bulk_insert runs one thread per key under the region locks;
    distinct keys commute, so the result is the bulk layout."""
    keys = np.unique(oracle.splitmix64(31, int(0.8 * (1 << nbits))))
    o = oracle.Oracle(nbits)
    o.bulk_insert(keys)
    with gq.QF(nbits, bulk_config=False) as qf:
        qf.point_bulk_insert(dev(keys))
        assert qf.status() == 0
        a, b = o.dump(), qf.export()
        assert np.array_equal(a, b), first_diff(a, b)
        assert qf.point_get_misses(dev(keys)) == 0


def test_export_import_roundtrip(gq):
    nbits = 14
    o = oracle.Oracle(nbits)
    o.bulk_insert(oracle.splitmix64(41, int(0.85 * (1 << nbits))))
    o.bulk_insert_reduce(oracle.skewed_keys(42, 1 << 13, 10))
    img = o.dump()
    probe = np.concatenate([oracle.splitmix64(41, 5000), oracle.splitmix64(43, 5000)])
    with gq.QF(nbits) as qf:
        qf.import_(img)
        assert np.array_equal(qf.export(), img)
        assert np.array_equal(gpu_get(qf, probe), o.bulk_get(probe))
        # keep working on the imported filter
        more = oracle.splitmix64(44, 1000)
        o.bulk_insert(more)
        qf.bulk_insert(dev(more))
        assert np.array_equal(qf.export(), o.dump())


def test_saturated_offsets(gq):
    """Clusters longer than 255 slots: the packed offsets saturate at 255 as
    in the reference, while the device keeps exact ones."""
    nbits = 12
    h = _clustered_hashes(7, nbits, 2500, 2000, 2400)
    o = oracle.Oracle(nbits)
    o.bulk_insert(h, key_is_hash=True)
    img = o.dump()
    assert (oracle.parse_dump(img)[1] == 255).any()
    with gq.QF(nbits) as qf:
        qf.bulk_insert(dev(h), flags=gq.QF_KEY_IS_HASH)
        assert np.array_equal(qf.export(), img), first_diff(qf.export(), img)
        probe = np.concatenate([h, _clustered_hashes(8, nbits, 2000, 1900, 2500)])
        import torch

        out = zeros_dev(probe.size)
        qf.bulk_get_async(dev(probe), out, probe.size, flags=gq.QF_KEY_IS_HASH)
        torch.cuda.synchronize()
        assert np.array_equal(host(out), np.array([o.count_hash(int(x)) for x in probe], dtype=np.uint64))
    with gq.QF(nbits) as qf2:
        qf2.import_(img)
        assert np.array_equal(qf2.export(), img)


def test_empty_and_tiny_batches(gq):
    nbits = 10
    with gq.QF(nbits) as qf:
        z = dev(np.zeros(1, dtype=np.uint64))
        qf.bulk_insert(z, n=0)
        qf.bulk_delete(z, n=0)
        assert qf.bulk_get_misses(z, n=0) == 0
        assert np.array_equal(qf.export(), oracle.Oracle(nbits).dump())
        one = np.array([12345], dtype=np.uint64)
        qf.bulk_insert(dev(one))
        assert gpu_get(qf, one)[0] == 1
        qf.bulk_delete(dev(one))
        assert gpu_get(qf, one)[0] == 0
        assert np.array_equal(qf.export(), oracle.Oracle(nbits).dump())


@pytest.mark.slow
@pytest.mark.parametrize("nbits", [22, 24])
def test_batched_fill_matches_oracle(gq, nbits):
    """Config-2 shape at a size the oracle finishes in seconds: fill to 90% in
    batches of 2^(nbits-4), get present + absent, delete a quarter."""
    n = int(0.9 * (1 << nbits))
    keys = oracle.splitmix64(1, n)
    o = oracle.Oracle(nbits, threads=8)
    bs = 1 << (nbits - 4)
    with gq.QF(nbits) as qf:
        for i in range(0, n, bs):
            o.bulk_insert(keys[i:i + bs])
            qf.bulk_insert(dev(keys[i:i + bs]))
        a, b = o.dump(), qf.export()
        assert np.array_equal(a, b), first_diff(a, b)
        probe = np.concatenate([keys[: 1 << 20], oracle.splitmix64(2, 1 << 20)])
        assert np.array_equal(gpu_get(qf, probe), o.bulk_get(probe))
        o.bulk_delete(keys[: n // 4])
        qf.bulk_delete(dev(keys[: n // 4]))
        a, b = o.dump(), qf.export()
        assert np.array_equal(a, b), first_diff(a, b)


def test_serialize_roundtrip_and_reference_image(gq, golden, tmp_path):
    """gqf_serialize / gqf_deserialize: a file round trip keeps the filter,
    and an image of the reference's own filter (the golden dump) loads."""
    meta, arrays = golden
    nbits = 14
    keys = oracle.splitmix64(1, meta["uniform14"]["n"])
    path = str(tmp_path / "f.gqf")
    with gq.QF(nbits) as qf:
        qf.bulk_insert(dev(keys))
        n = qf.save(path)
        assert n == 120 + 81 * qf.nblocks
        with gq.QF.load_file(path) as back:
            assert back.nbits == nbits
            assert np.array_equal(back.export(), qf.export())
            assert np.array_equal(gpu_get(back, keys), gpu_get(qf, keys))
    ref = arrays["uniform14_dump_insert"] if "uniform14_dump_insert" in arrays else None
    if ref is not None:
        (tmp_path / "ref.gqf").write_bytes(np.ascontiguousarray(ref).tobytes())
        with gq.QF.load_file(str(tmp_path / "ref.gqf")) as r:
            assert np.array_equal(r.export(), ref)
    (tmp_path / "bad.gqf").write_bytes(b"not a filter")
    with pytest.raises(RuntimeError):
        gq.QF.load_file(str(tmp_path / "bad.gqf"))
