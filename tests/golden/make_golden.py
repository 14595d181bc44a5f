"""Regenerate the golden fixtures from the reference itself.

Runs the reference GQF host path compiled from its own sources
(oracle/_ref/libgqf_ref.so, built by ``oracle/ref/Makefile`` on an x86 host
that has the reference tree) on seeded synthetic inputs and records its
outputs: packed filter dumps (or their SHA-256 for the larger ones), counts,
false-positive sets and point-API return codes.

    python tests/golden/make_golden.py

The CPU tests pin oracle/gqf_oracle.c against these files, and the GPU tests
pin the CUDA path against the oracle.  Inputs are splitmix64 streams and the
integer-only skew generator in oracle/__init__.py, so every host regenerates
the same keys.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def uniform_case(nbits: int, arrays: dict, meta: dict, keep_dump: bool):
    """Config-1 shape at any size: fill to 90% with splitmix64 seed 1, get the
    present keys and 2^nbits absent keys (seed 2), delete the first half."""
    n = int(0.9 * (1 << nbits))
    present = oracle.splitmix64(1, n)
    absent = oracle.splitmix64(2, 1 << nbits)
    f = oracle.RefFilter(nbits)
    f.bulk_insert(present.copy())
    d_ins = f.dump()
    c_present = f.bulk_get(present)
    c_absent = f.bulk_get(absent)
    f.bulk_delete(present[: n // 2].copy())
    d_del = f.dump()
    c_after = f.bulk_get(present)
    f.close()
    tag = f"uniform{nbits}"
    m = {
        "nbits": nbits,
        "n": n,
        "dump_insert_sha256": sha(d_ins),
        "dump_delete_sha256": sha(d_del),
        "counts_present_sha256": sha(c_present),
        "counts_absent_sha256": sha(c_absent),
        "counts_after_delete_sha256": sha(c_after),
        "false_positives": int((c_absent > 0).sum()),
        "present_count_hist": {str(int(k)): int(v) for k, v in zip(*np.unique(c_present, return_counts=True))},
        "after_delete_count_hist": {str(int(k)): int(v) for k, v in zip(*np.unique(c_after, return_counts=True))},
    }
    arrays[f"{tag}_fp_index"] = np.nonzero(c_absent)[0].astype(np.uint32)
    if keep_dump:
        arrays[f"{tag}_dump_insert"] = d_ins
        arrays[f"{tag}_dump_delete"] = d_del
    meta[tag] = m


def skew_case(nbits: int, arrays: dict, meta: dict):
    """Counter encodings: a skewed multiset through bulk_insert_reduce, more of
    it through bulk_insert (in-place counter increments), then deletes."""
    n = 2 << nbits
    k1 = oracle.skewed_keys(5, n, nbits - 2)
    k2 = oracle.skewed_keys(9, n // 4, nbits - 2)
    f = oracle.RefFilter(nbits)
    f.bulk_insert_reduce(k1.copy())
    d1 = f.dump()
    f.bulk_insert(k2.copy())
    d2 = f.dump()
    f.bulk_delete(k1[: n // 3].copy())
    d3 = f.dump()
    probe = np.concatenate([np.unique(k1), oracle.splitmix64(77, 1 << 10)])
    c = f.bulk_get(probe)
    f.close()
    tag = f"skew{nbits}"
    arrays[f"{tag}_dump_reduce"] = d1
    arrays[f"{tag}_dump_insert"] = d2
    arrays[f"{tag}_dump_delete"] = d3
    arrays[f"{tag}_counts"] = c
    meta[tag] = {"nbits": nbits, "n": n, "max_count": int(c.max())}


def point_case(nbits: int, arrays: dict, meta: dict):
    """qf_insert_not_exists / qf_query (the point API's bodies) on a filter
    that also holds counters from qf_insert."""
    f = oracle.RefFilter(nbits)
    mask = (1 << (nbits + 8)) - 1
    hs = (oracle.splitmix64(21, 600) & np.uint64(mask)).astype(np.uint64)
    dup = hs[:100]
    for h in dup:
        f.insert_hash(int(h), 3)
    rets = []
    for h in np.concatenate([hs, hs[:300]]):
        r, v = f.insert_not_exists_hash(int(h))
        rets.append(r * 256 + v)
    q = np.array([f.query_hash(int(h)) for h in np.concatenate([hs, oracle.splitmix64(22, 200) & np.uint64(mask)])],
                 dtype=np.uint64)
    tag = f"point{nbits}"
    arrays[f"{tag}_rets"] = np.array(rets, dtype=np.uint32)
    arrays[f"{tag}_query"] = q
    arrays[f"{tag}_dump"] = f.dump()
    meta[tag] = {"nbits": nbits}
    f.close()


def main():
    lib = oracle.build_ref()
    if lib is None:
        raise SystemExit("oracle/_ref could not be built here (needs x86-64 and the reference tree)")
    arrays: dict = {}
    meta: dict = {"generator": "tests/golden/make_golden.py", "source": "oracle/_ref (reference src/gqf.cu host path)"}
    for nb in (10, 12, 14):
        uniform_case(nb, arrays, meta, keep_dump=True)
    for nb in (16, 20):
        uniform_case(nb, arrays, meta, keep_dump=False)
    skew_case(12, arrays, meta)
    point_case(10, arrays, meta)
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **arrays)
    with open(os.path.join(HERE, "golden.json"), "w") as fh:
        json.dump(meta, fh, indent=1, sort_keys=True)
    print("wrote", os.path.join(HERE, "golden.npz"), os.path.getsize(os.path.join(HERE, "golden.npz")), "bytes")


if __name__ == "__main__":
    main()
