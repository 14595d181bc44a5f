"""The serving loop's host policy (staging ring and launch grouping,
cqf_gb300/csrc/serve_sched.h) on the CPU, against a byte-level model."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GET, INSERT, DELETE, REDUCE = 0, 1, 2, 3


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("needs a C++ compiler")
    out = str(tmp_path_factory.mktemp("sched") / "libsched.so")
    subprocess.check_call([cxx, "-std=c++17", "-O1", "-fPIC", "-shared",
                           os.path.join(HERE, "serve_sched_host.cpp"), "-o", out])
    L = ctypes.CDLL(out)
    vp, u64 = ctypes.c_void_p, ctypes.c_uint64
    L.ring_new.restype = vp
    L.ring_new.argtypes = [u64]
    L.ring_free.argtypes = [vp]
    L.ring_alloc.argtypes = [vp, u64, ctypes.POINTER(u64)]
    L.ring_release.argtypes = [vp, u64, u64]
    L.ring_used.restype = u64
    L.ring_used.argtypes = [vp]
    L.plan.restype = u64
    L.plan.argtypes = [vp, vp, vp, u64, u64, u64]
    L.split.restype = u64
    L.split.argtypes = [ctypes.c_int, u64]
    L.req_bytes.restype = u64
    L.req_bytes.argtypes = [ctypes.c_int, u64]
    return L


@pytest.mark.parametrize("seed", range(8))
def test_ring_never_overlaps_and_frees_in_order(lib, seed):
    rng = np.random.default_rng(seed)
    cap = int(rng.integers(1, 64)) * 256
    r = lib.ring_new(cap)
    owner = np.zeros(cap, dtype=np.int64)  # byte -> live block id (0 = free)
    live = []  # FIFO of (id, off, bytes)
    nid = 0
    for _ in range(3000):
        if live and (rng.random() < 0.45 or len(live) > 40):
            bid, off, b = live.pop(0)
            assert lib.ring_release(r, off, b) == 1
            assert (owner[off:off + b] == bid).all()
            owner[off:off + b] = 0
            if not live:
                assert lib.ring_used(r) == 0
            continue
        b = int(rng.integers(1, cap // 256 + 1)) * 256
        off = ctypes.c_uint64(0)
        ok = lib.ring_alloc(r, b, ctypes.byref(off))
        if not live:
            assert ok  # an empty ring takes any block up to its size
        if ok:
            o = off.value
            assert o + b <= cap
            assert (owner[o:o + b] == 0).all()
            nid += 1
            owner[o:o + b] = nid
            live.append((nid, o, b))
        else:
            # refusal only when neither free run (after the newest block,
            # before the oldest one) can hold the block
            head = live[-1][1] + live[-1][2]
            tail = live[0][1]
            runs = [cap - head, tail] if head > tail else [tail - head]
            assert max(runs) < b
        assert lib.ring_used(r) >= int((owner > 0).sum())
        assert lib.ring_used(r) <= cap
    if live:  # a release out of order is refused
        assert lib.ring_release(r, live[0][1] + 1, live[0][2]) == 0
    lib.ring_free(r)


def _plan(lib, reqs, max_keys, max_bytes):
    ops = np.array([q[0] for q in reqs], dtype=np.int32)
    kih = np.array([q[1] for q in reqs], dtype=np.int32)
    ns = np.array([q[2] for q in reqs], dtype=np.uint64)
    return int(lib.plan(ops.ctypes.data, kih.ctypes.data, ns.ctypes.data, len(reqs), max_keys, max_bytes))


def test_grouping_by_class_and_limits(lib):
    big = 1 << 40
    assert _plan(lib, [], big, big) == 0
    # inserts and counted inserts coalesce; a get ends the group
    assert _plan(lib, [(INSERT, 0, 10), (REDUCE, 0, 5), (INSERT, 0, 7), (GET, 0, 3)], big, big) == 3
    # QF_KEY_IS_HASH batches stay apart
    assert _plan(lib, [(INSERT, 0, 10), (INSERT, 1, 5)], big, big) == 1
    assert _plan(lib, [(DELETE, 0, 1), (DELETE, 0, 1), (INSERT, 0, 1)], big, big) == 2
    assert _plan(lib, [(GET, 0, 4), (GET, 0, 4), (GET, 0, 4)], big, big) == 3
    # key limit, byte limit; the first request always goes
    assert _plan(lib, [(GET, 0, 100), (GET, 0, 100), (GET, 0, 100)], 250, big) == 2
    assert _plan(lib, [(INSERT, 0, 1000)], 10, 10) == 1
    per = int(lib.req_bytes(GET, 100))
    assert per == 1792  # 100 keys + 100 counts, rounded up to 256 bytes
    assert _plan(lib, [(GET, 0, 100)] * 5, big, 3 * per) == 3


def test_split_keeps_parts_within_a_quarter_ring(lib):
    for op, per in ((GET, 16), (INSERT, 8), (DELETE, 8)):
        for ring in (1 << 20, 1 << 30, 3 << 28):
            k = int(lib.split(op, ring))
            assert k % 32 == 0 and 0 < k * per <= ring // 4
