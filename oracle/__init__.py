"""CPU oracle for the GQF bulk hot path -- TEST INFRASTRUCTURE ONLY.

Python bindings for ``oracle/gqf_oracle.c`` (a plain-C restatement of the
reference counting quotient filter, src/gqf.cu) and for ``oracle/_ref`` (the
reference's own host path compiled from its sources on an x86 host).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg may import this package, and only as the test oracle or the timed CPU
baseline.  The product (``cqf_gb300``) never imports it.
"""
from __future__ import annotations

import ctypes
import os
import platform
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
LIB_PATH = os.path.join(BUILD_DIR, "liboracle.so")
REF_LIB_PATH = os.path.join(REF_DIR, "libgqf_ref.so")
# The reference tree: $GQF_REFERENCE_TREE, else a checkout named "reference"
# beside this repository.  Only the build recipes read it.
REFERENCE_TREE = os.environ.get("GQF_REFERENCE_TREE") or os.path.join(os.path.dirname(os.path.dirname(HERE)),
                                                                       "reference")

_vp, _u64, _int = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int


def build(force: bool = False) -> str:
    """Compile the C restatement with gcc (portable C11, no intrinsics)."""
    src = os.path.join(HERE, "gqf_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < max(
        os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "gqf_oracle.h"))
    ):
        os.makedirs(BUILD_DIR, exist_ok=True)
        tmp = LIB_PATH + ".tmp"
        subprocess.check_call(
            ["gcc", "-O2", "-std=c11", "-Wall", "-shared", "-fPIC", src, "-lpthread", "-lm", "-o", tmp]
        )
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


def build_ref() -> str | None:
    """Compile the reference host path from its sources (x86 only; needs the
    reference tree).  Returns the library path or None when not possible."""
    if platform.machine() not in ("x86_64", "AMD64") or not os.path.isdir(REFERENCE_TREE):
        return REF_LIB_PATH if os.path.exists(REF_LIB_PATH) else None
    subprocess.check_call(["make", "-s", "-C", os.path.join(HERE, "ref"), f"REF={REFERENCE_TREE}"])
    return REF_LIB_PATH


def splitmix64(seed: int, n: int) -> np.ndarray:
    """splitmix64 stream: out[i] = mix(seed + (i + 1) * golden)."""
    x = np.uint64(seed) + np.arange(1, n + 1, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15)
    z = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def hash64(keys: np.ndarray, nbits: int) -> np.ndarray:
    """hash_64 (src/hashutil.cu:132) under BITMASK(nbits + 8), vectorised."""
    m = np.uint64((1 << (nbits + 8)) - 1)
    k = np.asarray(keys, dtype=np.uint64)
    with np.errstate(over="ignore"):
        k = (~k + (k << np.uint64(21))) & m
        k = k ^ (k >> np.uint64(24))
        k = ((k + (k << np.uint64(3))) + (k << np.uint64(8))) & m
        k = k ^ (k >> np.uint64(14))
        k = ((k + (k << np.uint64(2))) + (k << np.uint64(4))) & m
        k = k ^ (k >> np.uint64(28))
        k = (k + (k << np.uint64(31))) & m
    return k


def skewed_keys(seed: int, n: int, pool_bits: int) -> np.ndarray:
    """Deterministic skewed multiset: the product of three uniforms picks an
    index into a pool of 2^pool_bits distinct splitmix64 keys (small indices
    are far more frequent).  Integer-only, so identical on every host."""
    a = splitmix64(seed, n) >> np.uint64(44)
    b = splitmix64(seed + 1, n) >> np.uint64(44)
    c = splitmix64(seed + 2, n) >> np.uint64(44)
    idx = (a * b * c) >> np.uint64(60 - pool_bits)
    pool = splitmix64(seed + 3, 1 << pool_bits)
    return pool[idx.astype(np.int64)]


def _bind(lib: ctypes.CDLL, name: str, res, args):
    f = getattr(lib, name)
    f.restype = res
    f.argtypes = args
    return f


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data if a is not None and a.size else 0


class _OracleLib:
    def __init__(self, path: str):
        L = ctypes.CDLL(path)
        self.new = _bind(L, "oqf_new", _vp, [_int])
        self.free = _bind(L, "oqf_free", None, [_vp])
        self.dump = _bind(L, "oqf_dump", _u64, [_vp, _vp, _u64])
        self.load = _bind(L, "oqf_load", _int, [_vp, _vp, _u64])
        self.nslots = _bind(L, "oqf_nslots", _u64, [_vp])
        self.xnslots = _bind(L, "oqf_xnslots", _u64, [_vp])
        self.nblocks = _bind(L, "oqf_nblocks", _u64, [_vp])
        self.insert = _bind(L, "oqf_insert", _int, [_vp, _u64, _u64])
        self.remove = _bind(L, "oqf_remove", _int, [_vp, _u64, _u64])
        self.count = _bind(L, "oqf_count", _u64, [_vp, _u64])
        self.insert_not_exists = _bind(
            L, "oqf_insert_not_exists", _int, [_vp, _u64, ctypes.POINTER(ctypes.c_uint8)]
        )
        self.query = _bind(L, "oqf_query", _u64, [_vp, _u64, ctypes.POINTER(ctypes.c_uint64)])
        self.hash64 = _bind(L, "oqf_hash64", _u64, [_u64, _u64])
        self.hash64i = _bind(L, "oqf_hash64i", _u64, [_u64, _u64])
        for name in ("oqf_bulk_insert", "oqf_bulk_insert_reduce", "oqf_bulk_delete"):
            setattr(self, name[4:], _bind(L, name, None, [_vp, _u64, _vp, _int, _int]))
        self.bulk_get = _bind(L, "oqf_bulk_get", None, [_vp, _u64, _vp, _vp, _int])
        self.bulk_get_misses = _bind(L, "oqf_bulk_get_misses", _u64, [_vp, _u64, _vp, _int])


_LIB: _OracleLib | None = None


def lib() -> _OracleLib:
    global _LIB
    if _LIB is None:
        _LIB = _OracleLib(build())
    return _LIB


class Oracle:
    """The reference filter restated on the CPU (packed 81-byte blocks)."""

    def __init__(self, nbits: int, threads: int = 1):
        self.L = lib()
        self.nbits = nbits
        self.threads = threads
        self.h = self.L.new(nbits)

    def close(self):
        if self.h:
            self.L.free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def nslots(self):
        return self.L.nslots(self.h)

    @property
    def xnslots(self):
        return self.L.xnslots(self.h)

    @property
    def nblocks(self):
        return self.L.nblocks(self.h)

    def dump(self) -> np.ndarray:
        n = self.L.dump(self.h, None, 0)
        out = np.zeros(n, dtype=np.uint8)
        self.L.dump(self.h, out.ctypes.data, n)
        return out

    def load(self, buf: np.ndarray):
        buf = np.ascontiguousarray(buf, dtype=np.uint8)
        if self.L.load(self.h, buf.ctypes.data, buf.size) != 0:
            raise ValueError("dump size does not match this filter")

    def bulk_insert(self, keys, key_is_hash=False):
        k = np.ascontiguousarray(keys, dtype=np.uint64)
        self.L.bulk_insert(self.h, k.size, _ptr(k), int(key_is_hash), self.threads)

    def bulk_insert_reduce(self, keys, key_is_hash=False):
        k = np.ascontiguousarray(keys, dtype=np.uint64)
        self.L.bulk_insert_reduce(self.h, k.size, _ptr(k), int(key_is_hash), self.threads)

    def bulk_delete(self, keys, key_is_hash=False):
        k = np.ascontiguousarray(keys, dtype=np.uint64)
        self.L.bulk_delete(self.h, k.size, _ptr(k), int(key_is_hash), self.threads)

    def bulk_get(self, keys) -> np.ndarray:
        k = np.ascontiguousarray(keys, dtype=np.uint64)
        out = np.zeros(k.size, dtype=np.uint64)
        self.L.bulk_get(self.h, k.size, _ptr(k), _ptr(out), self.threads)
        return out

    def bulk_get_misses(self, keys) -> int:
        k = np.ascontiguousarray(keys, dtype=np.uint64)
        return int(self.L.bulk_get_misses(self.h, k.size, _ptr(k), self.threads))

    def insert_hash(self, h, count=1):
        return self.L.insert(self.h, int(h), int(count))

    def remove_hash(self, h, count=1):
        return self.L.remove(self.h, int(h), int(count))

    def count_hash(self, h):
        return int(self.L.count(self.h, int(h)))

    def insert_not_exists_hash(self, h):
        v = ctypes.c_uint8(0)
        r = self.L.insert_not_exists(self.h, int(h), ctypes.byref(v))
        return r, v.value

    def query_hash(self, h):
        v = ctypes.c_uint64(0)
        r = self.L.query(self.h, int(h), ctypes.byref(v))
        return int(r), v.value


class RefFilter:
    """The reference host path itself (oracle/_ref), x86 only."""

    def __init__(self, nbits: int):
        path = REF_LIB_PATH
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        L = ctypes.CDLL(path)
        self._new = _bind(L, "ref_new", _vp, [_int])
        self._free = _bind(L, "ref_free", None, [_vp])
        self._dump = _bind(L, "ref_dump", _u64, [_vp, _vp, _u64])
        self._bi = _bind(L, "ref_bulk_insert", None, [_vp, _u64, _vp, _int])
        self._br = _bind(L, "ref_bulk_insert_reduce", None, [_vp, _u64, _vp, _int])
        self._bd = _bind(L, "ref_bulk_delete", None, [_vp, _u64, _vp, _int])
        self._bg = _bind(L, "ref_bulk_get", None, [_vp, _u64, _vp, _vp])
        self._ine = _bind(L, "ref_insert_not_exists_hash", _int, [_vp, _u64, ctypes.POINTER(ctypes.c_uint8)])
        self._q = _bind(L, "ref_query_hash", _u64, [_vp, _u64])
        self._ins = _bind(L, "ref_insert_hash", _int, [_vp, _u64, _u64])
        self._rem = _bind(L, "ref_remove_hash", _int, [_vp, _u64, _u64])
        self.nbits = nbits
        self.h = self._new(nbits)

    def close(self):
        if self.h:
            self._free(self.h)
            self.h = None

    def dump(self) -> np.ndarray:
        n = self._dump(self.h, None, 0)
        out = np.zeros(n, dtype=np.uint8)
        self._dump(self.h, out.ctypes.data, n)
        return out

    def bulk_insert(self, keys, key_is_hash=False):
        k = np.ascontiguousarray(keys, dtype=np.uint64)
        self._bi(self.h, k.size, _ptr(k), int(key_is_hash))

    def bulk_insert_reduce(self, keys, key_is_hash=False):
        k = np.ascontiguousarray(keys, dtype=np.uint64)
        self._br(self.h, k.size, _ptr(k), int(key_is_hash))

    def bulk_delete(self, keys, key_is_hash=False):
        k = np.ascontiguousarray(keys, dtype=np.uint64)
        self._bd(self.h, k.size, _ptr(k), int(key_is_hash))

    def bulk_get(self, keys) -> np.ndarray:
        k = np.ascontiguousarray(keys, dtype=np.uint64)
        out = np.zeros(k.size, dtype=np.uint64)
        self._bg(self.h, k.size, _ptr(k), _ptr(out))
        return out

    def insert_hash(self, h, count=1):
        return self._ins(self.h, int(h), int(count))

    def remove_hash(self, h, count=1):
        return self._rem(self.h, int(h), int(count))

    def insert_not_exists_hash(self, h):
        v = ctypes.c_uint8(0)
        r = self._ine(self.h, int(h), ctypes.byref(v))
        return r, v.value

    def query_hash(self, h):
        return int(self._q(self.h, int(h)))


def parse_dump(buf: np.ndarray):
    """Split a reference-format dump into (metadata u64[15], offsets u8[nb],
    occupieds u64[nb], runends u64[nb], slots u8[nb, 64])."""
    buf = np.ascontiguousarray(buf, dtype=np.uint8)
    meta = buf[:120]
    blocks = buf[120:].reshape(-1, 81)
    offsets = blocks[:, 0].copy()
    occ = np.ascontiguousarray(blocks[:, 1:9]).view(np.uint64).reshape(-1)
    run = np.ascontiguousarray(blocks[:, 9:17]).view(np.uint64).reshape(-1)
    slots = blocks[:, 17:].copy()
    return meta, offsets, occ, run, slots


_BASE_CODE = np.full(256, 255, dtype=np.uint8)
for _c, _v in zip(b"ACGTacgt", (0, 1, 2, 3, 0, 1, 2, 3)):
    _BASE_CODE[_c] = _v


def canonical_kmers(reads: np.ndarray, k: int) -> np.ndarray:
    """Canonical k-mers of fixed-length ASCII reads, uint64 [nreads * nk].

    The reference cuts k-mers as substrings of each read line
    (src/gqf_verify.cu:158-170); here each window is 2-bit packed (A=0 C=1
    G=2 T=3, first base in the high bits) and replaced by the smaller of
    itself and its reverse complement.  Windows holding a byte other than
    ACGT (either case) give all ones.  Vectorised over reads."""
    reads = np.ascontiguousarray(reads, dtype=np.uint8)
    nreads, length = reads.shape
    nk = length - k + 1
    codes = _BASE_CODE[reads]
    bad = codes == 255
    c = np.where(bad, 0, codes).astype(np.uint64)
    fw = np.zeros((nreads, nk), dtype=np.uint64)
    rc = np.zeros((nreads, nk), dtype=np.uint64)
    badw = np.zeros((nreads, nk), dtype=bool)
    for j in range(k):
        cj = c[:, j:j + nk]
        fw = (fw << np.uint64(2)) | cj
        rc = rc | ((np.uint64(3) - cj) << np.uint64(2 * j))
        badw |= bad[:, j:j + nk]
    out = np.minimum(fw, rc)
    out[badw] = np.uint64(0xFFFFFFFFFFFFFFFF)
    return out.reshape(-1)


def exact_counts(keys: np.ndarray, nbits: int, probe: np.ndarray) -> np.ndarray:
    """Exact multiplicity of each probe key among keys, with keys identified
    modulo 2^(nbits+8): hash_64 (src/hashutil.cu:132-140) reads only those
    bits, so keys equal there share one counter in any filter."""
    m = np.uint64((1 << (nbits + 8)) - 1)
    u, cnt = np.unique(np.asarray(keys, dtype=np.uint64) & m, return_counts=True)
    p = np.asarray(probe, dtype=np.uint64) & m
    i = np.searchsorted(u, p)
    i = np.minimum(i, max(0, u.size - 1))
    hit = (u.size > 0) & (u[i] == p) if u.size else np.zeros(p.shape, dtype=bool)
    return np.where(hit, cnt[i] if u.size else 0, 0).astype(np.uint64)


def encode_counter(rem: int, count: int) -> list:
    """Slots of one counter (src/gqf.cu:1216-1273), first slot first: count 1
    is [rem], 2 is [rem, rem], 3 is [rem, 0, rem]; larger counts store
    count - 3 (count - 4 for remainder 0) in base 254 (255) digits between
    two copies of rem, digits shifted past rem, a 0 escape when the leading
    digit is not below rem, and a trailing 0 for remainder 0."""
    if count == 0:
        return []
    if count == 1:
        return [rem]
    if count == 2:
        return [rem, rem]
    if count == 3:
        return [rem, 0, rem]
    base = 254 if rem else 255
    c = count - (3 if rem else 4)
    digits = []
    while True:
        d = c % base + 1
        if rem and d >= rem:
            d += 1
        digits.append(d)
        c //= base
        if not c:
            break
    out = [rem]
    if rem and digits[-1] >= rem:
        out.append(0)
    out += digits[::-1]
    if rem == 0:
        out.append(0)
    out.append(rem)
    return out


def canonical_dump(nbits: int, counts: dict) -> np.ndarray:
    """The packed filter (120-byte metadata + 81-byte blocks) that any history
    leaving the multiset `counts` (hash -> count) produces in the reference's
    insert path: runs in quotient order, counters in remainder order, each run
    at max(quotient, end of the previous run + 1), offsets min(255, exact).
    The metadata is taken from an empty oracle filter.  Raises if the runs
    do not fit the table."""
    o = Oracle(nbits)
    meta = o.dump()[:120].copy()
    nblocks, xn = o.nblocks, o.xnslots
    o.close()
    slots = np.zeros(64 * nblocks, dtype=np.uint8)
    occ = np.zeros(64 * nblocks, dtype=np.uint8)
    run = np.zeros(64 * nblocks, dtype=np.uint8)
    by_q = {}
    for h, c in counts.items():
        if c:
            by_q.setdefault(int(h) >> 8, []).append((int(h) & 255, int(c)))
    end = -1
    ends = {}
    for q in sorted(by_q):
        s = max(q, end + 1)
        body = []
        for rem, c in sorted(by_q[q]):
            body += encode_counter(rem, c)
        if s + len(body) > xn:
            raise ValueError("multiset does not fit the table")
        slots[s:s + len(body)] = body
        end = s + len(body) - 1
        occ[q] = 1
        run[end] = 1
        ends[q] = end
    offs = np.zeros(nblocks, dtype=np.int64)
    qs = np.array(sorted(ends), dtype=np.int64)
    es = np.array([ends[q] for q in qs], dtype=np.int64)
    for b in range(1, nblocks):
        k = np.searchsorted(qs, 64 * b) - 1
        if k >= 0:
            offs[b] = max(0, int(es[k]) - 64 * b + 1)
    blk = np.zeros((nblocks, 81), dtype=np.uint8)
    blk[:, 0] = np.minimum(255, offs)
    blk[:, 1:9] = np.packbits(occ.reshape(nblocks, 64), axis=1, bitorder="little")
    blk[:, 9:17] = np.packbits(run.reshape(nblocks, 64), axis=1, bitorder="little")
    blk[:, 17:] = slots.reshape(nblocks, 64)
    return np.concatenate([meta, blk.reshape(-1)])
