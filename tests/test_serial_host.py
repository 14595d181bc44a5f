"""The device's single-key algorithms (gqf_device.cuh, gqf::Serial) compiled
for the host and compared with the oracle on random histories (CPU only).

These are the algorithms behind the point API and the bulk path's serial
fallback; on the device they run the same source."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    from cqf_gb300 import build

    nv = build.nvcc()
    out = str(tmp_path_factory.mktemp("serial") / "libserial_host.so")
    subprocess.check_call([nv, "-std=c++17", "-O1", "-Xcompiler", "-fPIC", "-shared", "-x", "cu",
                           os.path.join(HERE, "serial_host.cu"), "-o", out])
    L = ctypes.CDLL(out)
    vp, u64 = ctypes.c_void_p, ctypes.c_uint64
    L.sh_new.restype = vp
    L.sh_new.argtypes = [ctypes.c_int]
    L.sh_insert1.argtypes = [vp, u64]
    L.sh_remove.argtypes = [vp, u64]
    L.sh_insert.argtypes = [vp, u64, u64]
    L.sh_count.restype = u64
    L.sh_count.argtypes = [vp, u64]
    L.sh_export.argtypes = [vp, vp]
    L.sh_sparse_fits.argtypes = [vp, u64, u64, u64]
    L.sh_insert_growth.restype = u64
    L.sh_insert_growth.argtypes = [u64]
    L.sh_snapshot.restype = ctypes.c_int64
    L.sh_snapshot.argtypes = [vp, vp]
    L.sh_highest_change.restype = ctypes.c_int64
    L.sh_highest_change.argtypes = [vp, vp]
    return L


@pytest.mark.parametrize("seed", range(24))
def test_serial_algorithms_match_oracle(lib, seed):
    rng = np.random.default_rng(seed)
    nbits = int(rng.integers(8, 13))
    o = oracle.Oracle(nbits)
    q = lib.sh_new(nbits)
    mask = (1 << (nbits + 8)) - 1
    cap = int(0.4 * o.xnslots)
    pool = oracle.splitmix64(seed + 1, cap) & np.uint64(mask)
    for _ in range(int(rng.integers(200, 2000))):
        h = int(pool[rng.integers(0, int(rng.integers(1, cap)))])
        r = rng.random()
        if r < 0.55:
            o.insert_hash(h, 1)
            lib.sh_insert1(q, h)
        elif r < 0.7:
            c = int(rng.choice([2, 3, 4, 5, 254, 255, 256, 1000, 65536]))
            o.insert_hash(h, c)
            lib.sh_insert(q, h, c)
        else:
            o.remove_hash(h, 1)
            lib.sh_remove(q, h)
    a = o.dump()
    assert oracle.parse_dump(a)[1].max() < 255
    b = np.zeros(o.nblocks * 81, dtype=np.uint8)
    lib.sh_export(q, b.ctypes.data)
    assert np.array_equal(a[120:], b)
    for h in pool[:500]:
        assert lib.sh_count(q, int(h)) == o.count_hash(int(h))


def test_walks_stop_at_the_table_end(lib):
    """A table pushed far past full (where the reference's walks run off its
    allocation) still terminates."""
    nbits = 10
    o = oracle.Oracle(nbits)
    q = lib.sh_new(nbits)
    rng = np.random.default_rng(31)
    mask = (1 << (nbits + 8)) - 1
    pool = oracle.splitmix64(32, 1075) & np.uint64(mask)
    for _ in range(1700):
        h = int(pool[rng.integers(0, 1075)])
        r = rng.random()
        if r < 0.55:
            o.insert_hash(h, 1)
            lib.sh_insert1(q, h)
        elif r < 0.7:
            c = int(rng.choice([1000, 70000]))
            o.insert_hash(h, c)
            lib.sh_insert(q, h, c)
        else:
            o.remove_hash(h, 1)
            lib.sh_remove(q, h)


@pytest.mark.parametrize("seed", range(12))
def test_sparse_window_check_bounds_every_change(lib, seed):
    """The key-by-key path's pre-check (Serial::sparse_fits): whenever it
    accepts a region's batch, applying the batch changes nothing at or past
    the bound.  Regions of 256 quotients with a 384-slot window, driven to
    93% of the slots with counted inserts and deletes; the end state is the
    canonical layout of the multiset."""
    from collections import Counter

    rng = np.random.default_rng(seed)
    nbits, lr = 13, 8
    reg = 1 << lr
    o = oracle.Oracle(nbits)
    q = lib.sh_new(nbits)
    snap = np.zeros(o.nblocks * 96, dtype=np.uint8)
    ms = Counter()
    used = 0  # slots the multiset's counters take
    live = []
    accepted = rejected = 0

    def slots(h, c):
        return len(oracle.encode_counter(h & 255, c))

    while used < int(0.93 * (1 << nbits)) and accepted + rejected < 6000:
        r = int(rng.integers(0, (1 << nbits) >> lr))
        k = int(rng.integers(1, 12))
        delete = live and rng.random() < 0.25
        if delete:
            hs = [live[int(i)] for i in rng.integers(0, len(live), size=k)]
            counts = [1] * k
        else:
            qs = rng.integers(r * reg, (r + 1) * reg, size=k).astype(np.uint64)
            rs = rng.integers(0, 256, size=k).astype(np.uint64)
            hs = [int(x) for x in (qs << np.uint64(8)) | rs]
            counts = [int(rng.choice([1, 1, 1, 2, 3, 300, 70000])) for _ in hs]
        rr = (hs[0] >> 8) >> lr
        keep = [i for i, h in enumerate(hs) if ((h >> 8) >> lr) == rr]
        hs, counts = [hs[i] for i in keep], [counts[i] for i in keep]
        grow = 0 if delete else sum(int(lib.sh_insert_growth(c)) for c in counts)
        bound = min(rr * reg + reg + reg // 2, o.xnslots)
        fits = lib.sh_sparse_fits(q, (rr + 1) * reg, grow, bound)
        lib.sh_snapshot(q, snap.ctypes.data)
        for h, c in zip(hs, counts):
            old = ms[h]
            if delete:
                lib.sh_remove(q, h)
                ms[h] = max(0, old - 1)
                if h in live:
                    live.remove(h)
            else:
                lib.sh_insert(q, h, c) if c > 1 else lib.sh_insert1(q, h)
                ms[h] = old + c
                live.append(h)
            used += slots(h, ms[h]) - slots(h, old)
        hi = lib.sh_highest_change(q, snap.ctypes.data)
        if fits:
            accepted += 1
            assert hi < bound, (hi, bound, grow, delete)
        else:
            rejected += 1
    assert accepted > 500
    # the canonical layout of the multiset (the oracle itself meets the
    # reference's 8-bit offset defect on such long clusters)
    b = np.zeros(o.nblocks * 81, dtype=np.uint8)
    lib.sh_export(q, b.ctypes.data)
    assert np.array_equal(oracle.canonical_dump(nbits, ms)[120:], b)
