"""bench.py's reference arm on CPU: `--impl reference` times the reference's
CPU implementation of the path (the oracle port where the reference's own
host code cannot run) and prints one JSON line with every key of the bench
contract, the `impl`, `cpu_baseline` and zero-copy `e2e` objects of that arm
included.  Run on a 2^14-slot filter so that it takes seconds."""
import json
import os
import subprocess
import sys

import pytest

pytest.importorskip("torch")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

KEYS = {"metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
        "scaling", "vs_baseline", "dtype", "data", "config"}


def test_reference_arm_prints_one_contract_line():
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--nbits", "14", "--steps", "2",
                          "--warmup", "3"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1, out.stdout
    d = json.loads(lines[0])
    assert KEYS <= set(d), KEYS - set(d)
    assert d["impl"] == "reference"
    assert d["n_gpus"] == 1 and d["steps"] == 2 and d["warmup"] == 3
    assert d["value"] > 0 and d["higher_is_better"] is True
    assert d["config"]["nbits"] == 14 and "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}


def test_parity_block_of_the_oracle_step():
    """The parity block bench.py adds to its line: two sides that ran the same
    step agree on every hash; a side whose filter differs by one byte is
    reported unequal for that item only."""
    import numpy as np

    sys.path.insert(0, ROOT)
    import bench
    import oracle

    oracle.build()
    wl = bench.Workload(14, 12, 12)
    keys = oracle.splitmix64(1, wl.n_insert)
    absent = oracle.splitmix64(2, wl.n_get)
    a = bench.cpu_step(wl, keys, absent, 2, oracle, "port", parity=True)["parity"]
    b = bench.cpu_step(wl, keys, absent, 1, oracle, "port", parity=True)["parity"]
    assert set(bench.PARITY_KEYS) <= set(a)
    p = bench.parity_block(14, {"oracle": a, "again": b, "absent": None})
    assert p["compared"] == ["again", "oracle"]
    assert p["dump_insert_equal"] and p["counts_present_equal"] and p["fp_set_equal"] and p["dump_delete_equal"]
    o = oracle.Oracle(14)
    o.bulk_insert(keys)
    d = o.dump()
    d[-1] ^= 1
    c = dict(b, dump_insert=bench.sha256_of(d))
    p = bench.parity_block(14, {"oracle": a, "changed": c})
    assert not p["dump_insert_equal"] and p["dump_delete_equal"] and p["fp_set_equal"]
    assert bench.sha256_of(np.arange(4, dtype=np.uint64)) == bench.sha256_of(np.arange(4, dtype=np.int64))
