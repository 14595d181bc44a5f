"""Single bulk workloads on one filter, for profiling a kernel in isolation.

    python -m cqf_gb300.cases --nbits 27 --load 0.8 --extra 1 --op insert

fills a 2^nbits-slot filter with splitmix64 keys (seed 1) in batches of
--batch keys up to --load of its slots, then runs --extra more batches of
--op (insert: fresh keys; delete / get: keys inserted by the fill) and
prints one line of CUDA-event times.  --op zipf and --op kmers instead run
--extra counted inserts on an empty filter: 2^28 Zipf(1.5) draws over 2^24
keys through bulk_insert_reduce, or the canonical 31-mers of 2^20
synthetic 150-base reads through the device k-mer counter (the skewed
counting workloads; --load and --batch do not apply).

Each bulk insert or delete launches, per parity of regions, the
short-window and the full-window rebuild, so the k-th rebuild launch of the
extra batches is number 4 * (fill calls) + k; the fill makes
ceil(load * 2^nbits / batch) calls.
"""
from __future__ import annotations

import argparse
import json
import math

import torch

from . import QF
from .synth import splitmix64_dev


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--nbits", type=int, default=27)
    ap.add_argument("--load", type=float, default=0.8, help="fill fraction of the slots")
    ap.add_argument("--batch", type=int, default=1 << 24, help="keys per bulk call")
    ap.add_argument("--extra", type=int, default=1, help="bulk calls after the fill")
    ap.add_argument("--op", choices=["insert", "delete", "get", "zipf", "kmers"], default="insert")
    a = ap.parse_args(argv)
    if a.op in ("zipf", "kmers"):
        return skewed(a)
    n_fill = int(a.load * (1 << a.nbits))
    n_extra = a.extra * a.batch
    keys = splitmix64_dev(1, n_fill + (n_extra if a.op == "insert" else 0))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    out = {"nbits": a.nbits, "load": a.load, "batch": a.batch, "op": a.op,
           "fill_calls": math.ceil(n_fill / a.batch)}
    with QF(a.nbits) as qf:
        e0.record()
        for s in range(0, n_fill, a.batch):
            qf.bulk_insert(keys[s:min(s + a.batch, n_fill)])
        e1.record()
        torch.cuda.synchronize()
        out["fill_ms"] = round(e0.elapsed_time(e1), 3)
        res = torch.empty(a.batch, dtype=torch.int64, device="cuda")
        e0.record()
        for i in range(a.extra):
            if a.op == "insert":
                qf.bulk_insert(keys[n_fill + i * a.batch:n_fill + (i + 1) * a.batch])
            else:
                s = (i * a.batch) % max(1, n_fill - a.batch)
                chunk = keys[s:s + a.batch]
                if a.op == "delete":
                    qf.bulk_delete(chunk)
                else:
                    qf.bulk_get(chunk, res)
        e1.record()
        torch.cuda.synchronize()
        out["extra_ms"] = round(e0.elapsed_time(e1), 3)
        out["status"] = qf.status()
        out["counters"] = qf.counters()
    print(json.dumps(out))
    return 0


def skewed(a) -> int:
    from .synth import dna_reads_dev, zipf_keys_dev

    if a.op == "zipf":
        data = zipf_keys_dev(3, 1 << 28, 1 << 24)
    else:
        data = dna_reads_dev(4, 1 << 20, 150, 1 << 24, 0.01)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    out = {"nbits": a.nbits, "op": a.op, "calls": a.extra, "ms": []}
    with QF(a.nbits) as qf:
        for _ in range(a.extra):
            qf.reset()
            e0.record()
            if a.op == "zipf":
                qf.bulk_insert_reduce(data)
            else:
                qf.bulk_insert_kmers(data, 31)
            e1.record()
            torch.cuda.synchronize()
            out["ms"].append(round(e0.elapsed_time(e1), 3))
        out["status"] = qf.status()
        out["counters"] = qf.counters()
    print(json.dumps(out))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
