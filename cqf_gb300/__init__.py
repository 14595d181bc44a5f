"""GB300-native counting quotient filter: Python view of the C ABI.

The product is ``cqf_gb300/_lib/libgqf_gb300.so`` (C ABI in ``include/gqf.h``)
and ``libgqf_gb300_device.a`` (device point API, ``include/gqf.cuh``), both
built by :func:`cqf_gb300.build.build`.  This module binds the C ABI with
ctypes and mirrors the reference's host API (PASSIONLab/cqf include/gqf.cuh)
for tests and benchmarks: same function names, same argument meaning, same
asynchronous behaviour.  Device buffers are passed as raw pointers; the
helpers accept torch CUDA tensors for convenience (torch is only plumbing
here: device memory and streams).

There is no CPU fallback.  If the native library is missing or cannot be
loaded, every entry point raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

QF_NO_LOCK = 0x01
QF_TRY_ONCE_LOCK = 0x02
QF_WAIT_FOR_LOCK = 0x04
QF_KEY_IS_HASH = 0x08

QF_ITEM_INSERTED, QF_ITEM_FOUND, QF_FULL, QF_TIMEOUT = 0, 1, 2, 3

STATUS_FULL = 1 << 0
STATUS_TIMEOUT = 1 << 1
STATUS_BAD_KEY = 1 << 2
STATUS_DEFERRED = 1 << 3
STATUS_OVERFLOW = 1 << 4

LIB_PATH = _build.SO_PATH

_vp, _u64, _u32, _int, _u8 = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int, ctypes.c_uint8

# name -> (restype, argtypes); mirrors include/gqf.h
SIGNATURES = {
    "qf_malloc_device": (None, [ctypes.POINTER(_vp), _int, ctypes.c_bool]),
    "qf_destroy_device": (None, [_vp]),
    "bulk_insert": (None, [_vp, _u64, _vp, _u8]),
    "bulk_insert_reduce": (None, [_vp, _u64, _vp, _u8]),
    "bulk_delete": (None, [_vp, _u64, _vp, _u8]),
    "bulk_get": (None, [_vp, _u64, _vp, _vp]),
    "bulk_get_misses_wrapper": (_u64, [_vp, _vp, _u64]),
    "point_get_wrapper": (_u64, [_vp, _vp, _u64]),
    "gqf_point_bulk_insert": (_int, [_vp, _vp, _u64]),
    "gqf_point_insert_batch": (_int, [_vp, _vp, _u64, _u8, _vp]),
    "gqf_point_insert_not_exists_batch": (_int, [_vp, _vp, _u64, _u8, _vp, _vp]),
    "gqf_point_query_batch": (_int, [_vp, _vp, _u64, _u8, _int, _vp]),
    "gqf_bulk_insert_async": (_int, [_vp, _u64, _vp, _u8, _vp]),
    "gqf_bulk_insert_reduce_async": (_int, [_vp, _u64, _vp, _u8, _vp]),
    "gqf_bulk_delete_async": (_int, [_vp, _u64, _vp, _u8, _vp]),
    "gqf_bulk_get_async": (_int, [_vp, _u64, _vp, _vp, _u8, _vp]),
    "gqf_bulk_insert_noalloc": (_int, [_vp, _u64, _vp, _u8, _vp]),
    "gqf_bulk_insert_kmers": (_int, [_vp, _vp, _u64, _u32, _u32, _vp]),
    "gqf_kmers_extract": (_int, [_vp, _u64, _u32, _u32, _vp, _vp]),
    "gqf_enumerate": (_int, [_vp, _vp, _vp, _u64, ctypes.POINTER(_u64), _int]),
    "gqf_merge": (_int, [_vp, _vp, _vp]),
    "gqf_multi_merge": (_int, [_vp, _int, _vp]),
    "gqf_intersect": (_int, [_vp, _vp, _vp]),
    "gqf_inner_product": (_u64, [_vp, _vp]),
    "gqf_resize": (_int, [_vp, _int]),
    "gqf_set_create": (_int, [_u32, _vp, _u64, ctypes.POINTER(_vp)]),
    "gqf_set_destroy": (None, [_vp]),
    "gqf_set_insert": (_int, [_vp, _vp, _vp, _u64, _u8, _vp]),
    "gqf_set_delete": (_int, [_vp, _vp, _vp, _u64, _u8, _vp]),
    "gqf_set_get": (_int, [_vp, _vp, _vp, _u64, _vp, _u8, _vp]),
    "gqf_set_reset": (_int, [_vp, _vp]),
    "gqf_set_tune": (_int, [_vp, _vp, _vp, _u64, _u8, ctypes.POINTER(ctypes.c_double)]),
    "gqf_set_config": (_int, [_vp, _int, _u32]),
    "gqf_set_get_config": (_int, [_vp, ctypes.POINTER(_int), ctypes.POINTER(_u32)]),
    "gqf_set_export_size": (_u64, [_vp, _u32]),
    "gqf_set_export": (_int, [_vp, _u32, _vp, _u64]),
    "gqf_set_get_status": (_int, [_vp, ctypes.POINTER(_u32)]),
    "gqf_server_create": (_int, [_vp, _u64, ctypes.POINTER(_vp)]),
    "gqf_server_submit": (ctypes.c_int64, [_vp, _int, _vp, _u64, _vp, _u32]),
    "gqf_server_poll": (_int, [_vp, ctypes.c_int64]),
    "gqf_server_wait": (_int, [_vp, ctypes.c_int64, ctypes.POINTER(ctypes.c_double)]),
    "gqf_server_drain": (_int, [_vp]),
    "gqf_server_stats": (_int, [_vp, _vp, _int]),
    "gqf_server_reset_stats": (_int, [_vp]),
    "gqf_server_destroy": (None, [_vp]),
    "gqf_set_stream": (_int, [_vp, _vp]),
    "gqf_set_region_log": (_int, [_vp, _int]),
    "gqf_get_region_log": (_int, [_vp]),
    "gqf_serialize": (_u64, [_vp, ctypes.c_char_p]),
    "gqf_deserialize": (_u64, [ctypes.POINTER(_vp), ctypes.c_char_p]),
    "gqf_set_lock_wait": (_int, [_vp, _u32]),
    "gqf_debug_hold_lock": (_int, [_vp, _u64, _int]),
    "gqf_set_sparse_max": (_int, [_vp, _u32]),
    "gqf_get_sparse_max": (ctypes.c_int64, [_vp]),
    "gqf_nslots": (_u64, [_vp]),
    "gqf_xnslots": (_u64, [_vp]),
    "gqf_nblocks": (_u64, [_vp]),
    "gqf_device_bytes": (_u64, [_vp]),
    "gqf_get_status": (_int, [_vp, ctypes.POINTER(_u32)]),
    "gqf_clear_status": (_int, [_vp]),
    "gqf_get_counters": (_int, [_vp, _vp, _int]),
    "gqf_reset": (_int, [_vp]),
    "gqf_export_size": (_u64, [_vp]),
    "gqf_export": (_int, [_vp, _vp, _u64]),
    "gqf_import": (_int, [_vp, _vp, _u64]),
    "gqf_debug_serial_apply": (_int, [_vp, _vp, _u64, _int]),
    "gqf_profile": (_int, [_vp, _int]),
    "gqf_profile_read": (_int, [_vp, _vp, _vp, _vp]),
    "gqf_launch_count": (_u64, []),
    "gqf_last_error": (ctypes.c_char_p, []),
    "gqf_version": (ctypes.c_char_p, []),
}

_LIB = None


def load(path: str | None = None, build_if_missing: bool = False) -> ctypes.CDLL:
    """Load the native library (raising if it is absent)."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = path or LIB_PATH
    if not os.path.exists(p):
        if build_if_missing:
            _build.build()
        else:
            raise RuntimeError(f"cqf_gb300 native library not built: {p} (run cqf_gb300.build.build())")
    lib = ctypes.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _LIB = lib
    return lib


def last_error() -> str:
    return load().gqf_last_error().decode()


def _ptr(x) -> int:
    """Device pointer of a torch tensor, an int, or None."""
    if x is None:
        return 0
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    raise TypeError(f"expected a device tensor or pointer, got {type(x)}")


def _stream_ptr(stream) -> int:
    if stream is None:
        return 0
    if hasattr(stream, "cuda_stream"):
        return stream.cuda_stream
    return int(stream)


class QF:
    """One filter on the current GPU (the reference's QF* handle)."""

    def __init__(self, nbits: int, bulk_config: bool = True, log_region: int | None = None):
        self.L = load()
        h = _vp()
        self.L.qf_malloc_device(ctypes.byref(h), int(nbits), bool(bulk_config))
        if not h.value:
            raise RuntimeError("qf_malloc_device failed: " + last_error())
        self.h = h.value
        self.nbits = nbits
        if log_region is not None:
            self.set_region_log(log_region)

    def close(self):
        if getattr(self, "h", None):
            self.L.qf_destroy_device(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- geometry
    @property
    def nslots(self) -> int:
        return int(self.L.gqf_nslots(self.h))

    @property
    def xnslots(self) -> int:
        return int(self.L.gqf_xnslots(self.h))

    @property
    def nblocks(self) -> int:
        return int(self.L.gqf_nblocks(self.h))

    def set_region_log(self, lr: int):
        if self.L.gqf_set_region_log(self.h, int(lr)) != 0:
            raise ValueError(last_error())

    def save(self, path: str) -> int:
        """Writes the filter image to `path` (gqf_serialize)."""
        n = int(self.L.gqf_serialize(self.h, os.fsencode(path)))
        if n == 0:
            raise RuntimeError(last_error())
        return n

    @classmethod
    def load_file(cls, path: str) -> "QF":
        """A new filter read from a gqf_serialize image (gqf_deserialize)."""
        L = load()
        h = _vp()
        if int(L.gqf_deserialize(ctypes.byref(h), os.fsencode(path))) == 0:
            raise RuntimeError(last_error())
        q = cls.__new__(cls)
        q.L = L
        q.h = h.value
        q.nbits = int(L.gqf_nslots(q.h)).bit_length() - 1
        return q

    def set_lock_wait(self, max_spins: int):
        self._ok(self.L.gqf_set_lock_wait(self.h, max_spins))

    def debug_hold_lock(self, index: int, held: bool = True):
        self._ok(self.L.gqf_debug_hold_lock(self.h, index, int(held)))

    def set_sparse_max(self, n: int):
        self._ok(self.L.gqf_set_sparse_max(self.h, n))

    def sparse_max(self) -> int:
        return int(self.L.gqf_get_sparse_max(self.h))

    def region_log(self) -> int:
        return int(self.L.gqf_get_region_log(self.h))

    # ---- reference bulk API (device buffers)
    def bulk_insert(self, keys, n: int | None = None, flags: int = QF_NO_LOCK):
        n = keys.numel() if n is None else n
        self.L.bulk_insert(self.h, n, _ptr(keys), flags)

    def bulk_insert_reduce(self, keys, n: int | None = None, flags: int = QF_NO_LOCK):
        n = keys.numel() if n is None else n
        self.L.bulk_insert_reduce(self.h, n, _ptr(keys), flags)

    def bulk_delete(self, keys, n: int | None = None, flags: int = QF_NO_LOCK):
        n = keys.numel() if n is None else n
        self.L.bulk_delete(self.h, n, _ptr(keys), flags)

    def bulk_get(self, vals, returns, n: int | None = None):
        n = vals.numel() if n is None else n
        self.L.bulk_get(self.h, n, _ptr(vals), _ptr(returns))

    def bulk_get_misses(self, vals, n: int | None = None) -> int:
        n = vals.numel() if n is None else n
        return int(self.L.bulk_get_misses_wrapper(self.h, _ptr(vals), n))

    def point_get_misses(self, keys, n: int | None = None) -> int:
        n = keys.numel() if n is None else n
        return int(self.L.point_get_wrapper(self.h, _ptr(keys), n))

    # ---- extensions
    def bulk_insert_async(self, keys, n, flags=QF_NO_LOCK, stream=None):
        self._ok(self.L.gqf_bulk_insert_async(self.h, n, _ptr(keys), flags, _stream_ptr(stream)))

    def bulk_insert_noalloc(self, keys, n=None, flags=QF_NO_LOCK, stream=None):
        """bulk_insert that allocates nothing (fixed scratch; see include/gqf.h)."""
        n = keys.numel() if n is None else n
        self._ok(self.L.gqf_bulk_insert_noalloc(self.h, n, _ptr(keys), flags, _stream_ptr(stream)))

    def bulk_insert_reduce_async(self, keys, n, flags=QF_NO_LOCK, stream=None):
        self._ok(self.L.gqf_bulk_insert_reduce_async(self.h, n, _ptr(keys), flags, _stream_ptr(stream)))

    def bulk_insert_kmers(self, reads, k: int, stream=None):
        """Counts the canonical k-mers of a device uint8 tensor [nreads, read_len]."""
        nreads, read_len = reads.shape
        self._ok(self.L.gqf_bulk_insert_kmers(self.h, _ptr(reads), nreads, read_len, k, _stream_ptr(stream)))

    def bulk_delete_async(self, keys, n, flags=QF_NO_LOCK, stream=None):
        self._ok(self.L.gqf_bulk_delete_async(self.h, n, _ptr(keys), flags, _stream_ptr(stream)))

    def bulk_get_async(self, vals, returns, n, flags=0, stream=None):
        self._ok(self.L.gqf_bulk_get_async(self.h, n, _ptr(vals), _ptr(returns), flags, _stream_ptr(stream)))

    def point_bulk_insert(self, keys, n=None):
        n = keys.numel() if n is None else n
        self._ok(self.L.gqf_point_bulk_insert(self.h, _ptr(keys), n))

    def point_insert_batch(self, keys, rets, n=None, flags=0):
        n = keys.numel() if n is None else n
        self._ok(self.L.gqf_point_insert_batch(self.h, _ptr(keys), n, flags, _ptr(rets)))

    def point_insert_not_exists_batch(self, keys, rets, vals, n=None, flags=0):
        n = keys.numel() if n is None else n
        self._ok(self.L.gqf_point_insert_not_exists_batch(self.h, _ptr(keys), n, flags, _ptr(rets), _ptr(vals)))

    def point_query_batch(self, keys, counts, n=None, flags=0, concurrent=False):
        n = keys.numel() if n is None else n
        self._ok(self.L.gqf_point_query_batch(self.h, _ptr(keys), n, flags, int(concurrent), _ptr(counts)))

    def serial_apply(self, hashes, op: int, n=None):
        n = hashes.numel() if n is None else n
        self._ok(self.L.gqf_debug_serial_apply(self.h, _ptr(hashes), n, op))

    def set_stream(self, stream):
        self._ok(self.L.gqf_set_stream(self.h, _stream_ptr(stream)))

    def status(self) -> int:
        s = _u32(0)
        self._ok(self.L.gqf_get_status(self.h, ctypes.byref(s)))
        return int(s.value)

    def counters(self) -> dict:
        c = np.zeros(3, dtype=np.uint64)
        self._ok(self.L.gqf_get_counters(self.h, c.ctypes.data, 3))
        return {"deferred_regions": int(c[0]), "serial_keys": int(c[1]), "full_window_regions": int(c[2])}

    def clear_status(self):
        self._ok(self.L.gqf_clear_status(self.h))

    def reset(self):
        self._ok(self.L.gqf_reset(self.h))

    def enumerate(self, as_keys: bool = False):
        """(hashes, counts) as host uint64 arrays, in increasing hash order."""
        import torch

        n = _u64(0)
        self._ok(self.L.gqf_enumerate(self.h, 0, 0, 0, ctypes.byref(n), 0))
        m = max(1, n.value)
        h = torch.empty(m, dtype=torch.int64, device="cuda")
        c = torch.empty(m, dtype=torch.int64, device="cuda")
        self._ok(self.L.gqf_enumerate(self.h, h.data_ptr(), c.data_ptr(), m, ctypes.byref(n), int(as_keys)))
        k = n.value
        return h[:k].cpu().numpy().view(np.uint64), c[:k].cpu().numpy().view(np.uint64)

    def merge_from(self, *others: "QF"):
        """Inserts every (hash, count) of the other filters (gqf_multi_merge)."""
        arr = (_vp * len(others))(*[o.h for o in others])
        self._ok(self.L.gqf_multi_merge(arr, len(others), self.h))

    def intersect_from(self, a: "QF", b: "QF"):
        self._ok(self.L.gqf_intersect(a.h, b.h, self.h))

    def inner_product(self, other: "QF") -> int:
        return int(self.L.gqf_inner_product(self.h, other.h))

    def resize(self, new_nbits: int):
        """Grows the table to 2^new_nbits slots under the same handle, keeping
        every stored key (modulo 2^(nbits + 8)) and its count."""
        self._ok(self.L.gqf_resize(self.h, int(new_nbits)))
        self.nbits = int(new_nbits)

    def export(self) -> np.ndarray:
        n = int(self.L.gqf_export_size(self.h))
        out = np.zeros(n, dtype=np.uint8)
        self._ok(self.L.gqf_export(self.h, out.ctypes.data, n))
        return out

    def import_(self, buf: np.ndarray):
        buf = np.ascontiguousarray(buf, dtype=np.uint8)
        self._ok(self.L.gqf_import(self.h, buf.ctypes.data, buf.size))

    def profile(self, enable: bool = True):
        self._ok(self.L.gqf_profile(self.h, int(enable)))

    PHASES = ("partition", "insert", "delete", "get")

    def profile_read(self) -> dict:
        ms = np.zeros(8, dtype=np.float64)
        calls = np.zeros(8, dtype=np.uint64)
        keys = np.zeros(8, dtype=np.uint64)
        self._ok(self.L.gqf_profile_read(self.h, ms.ctypes.data, calls.ctypes.data, keys.ctypes.data))
        return {p: {"ms": float(ms[i]), "calls": int(calls[i]), "keys": int(keys[i])}
                for i, p in enumerate(self.PHASES)}

    def _ok(self, rc: int):
        if rc != 0:
            raise RuntimeError(last_error())


SPARSE_AUTO = 0xFFFFFFFF


class FilterSet:
    """n independent filters served by one launch per phase (gqf_set_* in
    include/gqf.h).  Batches are device tensors: keys (int64) with CSR
    offsets (int64, n + 1 entries) on the device."""

    def __init__(self, nbits, max_batch_keys: int):
        self.L = load()
        nb = np.ascontiguousarray(nbits, dtype=np.int32)
        self.n = int(nb.size)
        self.nbits = nb.copy()
        h = _vp()
        if self.L.gqf_set_create(self.n, nb.ctypes.data, int(max_batch_keys), ctypes.byref(h)) != 0:
            raise RuntimeError("gqf_set_create failed: " + last_error())
        self.h = h

    def _ok(self, rc):
        if rc != 0:
            raise RuntimeError(last_error())

    def insert(self, keys, offsets, n=None, flags=QF_NO_LOCK, stream=None):
        n = keys.numel() if n is None else n
        self._ok(self.L.gqf_set_insert(self.h, _ptr(keys), _ptr(offsets), n, flags, _stream_ptr(stream)))

    def delete(self, keys, offsets, n=None, flags=QF_NO_LOCK, stream=None):
        n = keys.numel() if n is None else n
        self._ok(self.L.gqf_set_delete(self.h, _ptr(keys), _ptr(offsets), n, flags, _stream_ptr(stream)))

    def get(self, keys, offsets, counts, n=None, flags=0, stream=None):
        n = keys.numel() if n is None else n
        self._ok(self.L.gqf_set_get(self.h, _ptr(keys), _ptr(offsets), n, _ptr(counts), flags, _stream_ptr(stream)))

    def reset(self, stream=None):
        self._ok(self.L.gqf_set_reset(self.h, _stream_ptr(stream)))

    def tune(self, keys, offsets, n=None, flags=QF_NO_LOCK) -> float:
        """Picks region size and key-by-key threshold by timing inserts of
        this batch; leaves the set empty.  Returns the best insert time (ms)."""
        n = keys.numel() if n is None else n
        ms = ctypes.c_double(0)
        self._ok(self.L.gqf_set_tune(self.h, _ptr(keys), _ptr(offsets), n, flags, ctypes.byref(ms)))
        return ms.value

    def config(self, log_region: int | None = None, sparse_max: int | None = None):
        lr, sp = _int(0), _u32(0)
        self._ok(self.L.gqf_set_get_config(self.h, ctypes.byref(lr), ctypes.byref(sp)))
        if log_region is None and sparse_max is None:
            return {"log_region": lr.value, "sparse_max": sp.value}
        self._ok(self.L.gqf_set_config(self.h, lr.value if log_region is None else log_region,
                                       sp.value if sparse_max is None else sparse_max))

    def export(self, i: int) -> np.ndarray:
        size = int(self.L.gqf_set_export_size(self.h, i))
        out = np.zeros(size, dtype=np.uint8)
        self._ok(self.L.gqf_set_export(self.h, i, out.ctypes.data, size))
        return out

    def status(self) -> int:
        s = _u32(0)
        self._ok(self.L.gqf_set_get_status(self.h, ctypes.byref(s)))
        return int(s.value)

    def close(self):
        if getattr(self, "h", None):
            self.L.gqf_set_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


OP_GET, OP_INSERT, OP_DELETE, OP_INSERT_REDUCE = 0, 1, 2, 3
SERVE_DEVICE_PTRS = 1 << 8


class Server:
    """Serving loop over one resident filter (gqf_server_* in include/gqf.h).

    submit() takes host arrays (numpy uint64, ideally in pinned memory such
    as a pinned torch tensor) or device tensors; buffers must stay alive
    until the request completes."""

    STATS = ("requests", "launches", "keys", "p50_ms", "p99_ms", "max_ms", "staging_bytes", "peak_staging_bytes")

    def __init__(self, qf: "QF", staging_bytes: int = 0):
        self.L = load()
        self.qf = qf
        h = _vp()
        if self.L.gqf_server_create(qf.h, staging_bytes, ctypes.byref(h)) != 0:
            raise RuntimeError("gqf_server_create failed: " + last_error())
        self.h = h

    @staticmethod
    def _buf(x):
        if x is None:
            return 0, False
        if isinstance(x, np.ndarray):
            return x.ctypes.data, False
        if hasattr(x, "data_ptr"):
            return x.data_ptr(), bool(getattr(x, "is_cuda", False))
        return int(x), False

    def submit(self, op: int, keys, counts=None, n: int | None = None, flags: int = 0) -> int:
        kp, kdev = self._buf(keys)
        cp, cdev = self._buf(counts)
        if counts is not None and cdev != kdev:
            raise ValueError("keys and counts must both be host or both be device buffers")
        n = (keys.size if isinstance(keys, np.ndarray) else keys.numel()) if n is None else n
        t = self.L.gqf_server_submit(self.h, op, kp, n, cp, flags | (SERVE_DEVICE_PTRS if kdev else 0))
        if t < 0:
            raise RuntimeError("gqf_server_submit failed: " + last_error())
        return int(t)

    def poll(self, ticket: int) -> int:
        return int(self.L.gqf_server_poll(self.h, ticket))

    def wait(self, ticket: int) -> float:
        lat = ctypes.c_double(0)
        if self.L.gqf_server_wait(self.h, ticket, ctypes.byref(lat)) != 0:
            raise RuntimeError("request failed: " + last_error())
        return lat.value

    def drain(self):
        if self.L.gqf_server_drain(self.h) != 0:
            raise RuntimeError("server error: " + last_error())

    def stats(self) -> dict:
        out = np.zeros(len(self.STATS), dtype=np.float64)
        self.L.gqf_server_stats(self.h, out.ctypes.data, out.size)
        return {k: float(v) for k, v in zip(self.STATS, out)}

    def reset_stats(self):
        self.L.gqf_server_reset_stats(self.h)

    def close(self):
        if getattr(self, "h", None):
            self.L.gqf_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def kmers_extract(reads, k: int, out, stream=None):
    """out[read * nk + pos] = canonical k-mer (uint64; all ones = skipped window)."""
    nreads, read_len = reads.shape
    if load().gqf_kmers_extract(_ptr(reads), nreads, read_len, k, _ptr(out), _stream_ptr(stream)) != 0:
        raise RuntimeError(last_error())


def launch_count() -> int:
    return int(load().gqf_launch_count())


def exported_symbols_from_header(header: str) -> list[str]:
    """Function names declared in include/gqf.h (for the ABI check)."""
    import re

    text = open(header).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^[A-Za-z_][\w\s\*]*?\b([a-z_][a-z0-9_]*)\s*\(", text, flags=re.M)
    return sorted(set(n for n in names if n not in {"if", "while", "for", "sizeof", "defined"}))
