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
