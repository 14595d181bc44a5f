#!/usr/bin/env python3
"""Benchmark of the GQF bulk hot path at 2^28 slots and 90% load.

Workload (one "step", the reference's large bulk configuration): an empty
2^28-slot filter is filled to 90% load with 241,591,910 uniform uint64 keys
(splitmix64, seed 1) in bulk_insert batches of 2^24 keys; then bulk_get of
2^26 present keys and 2^26 absent keys (splitmix64, seed 2); then bulk_delete
of the 2^26 present keys.  Metric: key operations per second over the whole
step (inserts + gets + deletes), in Mkeys/s; per-operation rates are reported
beside it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
  python bench.py --case insert|delete|get|zipf|kmers [--nbits B] [--load F] [--extra E]

--impl ours (default) prints one JSON line with the device-resident value,
the end-to-end value through the C ABI from pinned host buffers (copies in
the timed region), the roofline of the dominant kernel, a CPU baseline, SM
clocks sampled during the timed region and the number of library kernel
launches.  --impl reference times the reference's CPU implementation of the
same path (the oracle restatement, multi-threaded over regions the way the
reference's launch is) on the host cores.

--case runs one workload on one filter for profiling a kernel in isolation
(no JSON contract line): it fills a 2^nbits-slot filter with splitmix64 keys
(seed 1) in batches of --case-batch keys up to --load of its slots, then runs
--extra more batches of the op (insert: fresh keys; delete / get: keys the
fill inserted) and prints one line of CUDA-event times.  zipf and kmers
instead run --extra counted inserts on an empty filter: 2^28 Zipf(1.5) draws
over 2^24 keys through bulk_insert_reduce, or the canonical 31-mers of 2^20
synthetic 150-base reads through the device k-mer counter (--load and
--case-batch do not apply).  Each bulk insert or delete launches, per parity
of regions, the short-window and the full-window rebuild, so the k-th rebuild
launch of the extra batches is number 4 * (fill calls) + k; the fill makes
ceil(load * 2^nbits / case-batch) calls.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "bulk insert/get Mkeys/s at 2^28 slots 90% load vs ref CUDA; serving p99 ms"
UNIT = "Mkeys/s"
L2_BYTES = 129 * 2**20  # GB300 L2
# Algorithmic bytes, counted on the reference's packed format (81-byte
# blocks: 1-byte offset, occupieds, runends, 64 one-byte slots).  A get moves
# its key, its count and one block; a bulk insert or delete reads and writes
# every block its batch touches once, plus its keys through the partition.
BYTES_GET = 97.0          # 8 key in + 8 count out + one 81-byte block
BLOCK_BYTES = 81.0
PART_BYTES_PER_KEY = 16.0  # key read + partitioned key written
REBUILD_KEY_BYTES = 8.0    # partitioned key read back


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--nbits", type=int, default=28)
    ap.add_argument("--batch-log", type=int, default=24)
    ap.add_argument("--get-log", type=int, default=26)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-ref-cuda", action="store_true")
    ap.add_argument("--cpu-threads", type=int, default=0)
    ap.add_argument("--no-skew", action="store_true", help="skip the skewed-counting workloads")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving-loop workload")
    ap.add_argument("--no-batched", action="store_true", help="skip the many-filter workload")
    ap.add_argument("--serve-nbits", type=int, default=30)
    ap.add_argument("--serve-load", type=float, default=0.7,
                    help="Poisson offered load as a fraction of the measured saturated throughput")
    ap.add_argument("--case", choices=["insert", "delete", "get", "zipf", "kmers"], default=None,
                    help="profile one op on one filter instead of the benchmark")
    ap.add_argument("--load", type=float, default=0.8, help="--case: fill fraction of the slots")
    ap.add_argument("--case-batch", type=int, default=1 << 24, help="--case: keys per bulk call")
    ap.add_argument("--extra", type=int, default=1, help="--case: bulk calls after the fill")
    return ap.parse_args()


class Workload:
    def __init__(self, nbits, batch_log, get_log):
        self.nbits = nbits
        self.nslots = 1 << nbits
        self.n_insert = int(0.9 * self.nslots)
        self.batch = 1 << batch_log
        self.n_get = min(1 << get_log, self.n_insert)
        self.batches = [(i, min(self.batch, self.n_insert - i)) for i in range(0, self.n_insert, self.batch)]
        self.xnslots = self.nslots + int(10 * np.sqrt(self.nslots))
        self.nblocks = (self.xnslots + 63) // 64

    @property
    def key_ops(self):
        return self.n_insert + 2 * self.n_get + self.n_get

    def touched_blocks(self, b):
        return self.nblocks * (1.0 - np.exp(-b / self.nblocks))

    def l2_note(self):
        keys, filt = 8 * (self.n_insert + self.n_get), 96 * self.nblocks
        size = lambda b: f"{b / 1e9:.2g} GB" if b >= 1e9 else f"{b / 1e6:.3g} MB"
        what = f"inputs ({size(keys)} of keys, {size(filt)} filter)"
        if keys + filt > L2_BYTES:
            return what + " exceed the 129 MB L2; no extra flush"
        return what + " fit the 129 MB L2"

    def describe(self):
        return {
            "workload": f"config 2: nbits={self.nbits} ({self.nslots} slots), fill 90% ({self.n_insert} keys) "
                        f"in {len(self.batches)} bulk_insert batches of 2^{int(np.log2(self.batch))}, "
                        f"bulk_get {self.n_get} present + {self.n_get} absent, bulk_delete {self.n_get} present",
            "nbits": self.nbits,
            "keys_inserted": self.n_insert,
            "insert_batch": self.batch,
            "gets_present": self.n_get,
            "gets_absent": self.n_get,
            "deletes": self.n_get,
            "key_ops_per_step": self.key_ops,
            "keys": "splitmix64 seed 1 (present), seed 2 (absent)",
            "l2": self.l2_note(),
        }


def splitmix_dev(seed, n, torch):
    """splitmix64 stream on the device (torch int64 arithmetic wraps)."""
    out = torch.empty(n, dtype=torch.int64, device="cuda")
    chunk = 1 << 26
    g = np.int64(np.uint64(0x9E3779B97F4A7C15).view(np.int64))
    m1 = np.int64(np.uint64(0xBF58476D1CE4E5B9).view(np.int64))
    m2 = np.int64(np.uint64(0x94D049BB133111EB).view(np.int64))
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        x = torch.arange(s + 1, e + 1, dtype=torch.int64, device="cuda") * g + seed
        x = (x ^ ((x >> 30) & ((1 << 34) - 1))) * m1
        x = (x ^ ((x >> 27) & ((1 << 37) - 1))) * m2
        out[s:e] = x ^ ((x >> 31) & ((1 << 33) - 1))
    return out


class ClockSampler:
    """nvidia-smi samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, mx, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
                power.append(float(p[3]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {
            "sm_mhz": statistics.median(sm) if sm else None,
            "sm_max_mhz": max(mx) if mx else None,
            "reasons": sorted(reasons),
            "samples": len(sm),
            "power_w_max": max(power) if power else None,
        }


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def sha256_of(a) -> str:
    """SHA-256 of an array's bytes (a numpy array, or a torch tensor copied
    to the host)."""
    if hasattr(a, "cpu"):
        a = a.cpu().numpy()
    return hashlib.sha256(np.ascontiguousarray(a).view(np.uint8).data).hexdigest()


PARITY_KEYS = ("dump_insert", "counts_present", "counts_absent", "dump_delete")


def parity_block(nbits, sides):
    """Word-for-word agreement of the sides that ran the same step: the
    packed filter after the inserts and after the deletes, and the count
    arrays of the present and absent gets (equal absent counts = the same
    false-positive set with the same counts)."""
    sides = {k: v for k, v in sides.items() if isinstance(v, dict) and "dump_insert" in v}
    out = {"nbits": nbits, "compared": sorted(sides)}
    names = {"dump_insert": "dump_insert_equal", "counts_present": "counts_present_equal",
             "counts_absent": "fp_set_equal", "dump_delete": "dump_delete_equal"}
    for k in PARITY_KEYS:
        vals = {s: d[k] for s, d in sides.items() if k in d}
        out[names[k]] = len(vals) >= 2 and len(set(vals.values())) == 1
    out["false_positives_absent"] = {s: d.get("false_positives") for s, d in sides.items()}
    out["sha256"] = {s: {k: d[k] for k in PARITY_KEYS if k in d} for s, d in sides.items()}
    return out


def profile_traffic():
    """DRAM bytes per unit of work (probe, key or block) of each kernel from
    the committed ncu summaries (profiles/ncu_traffic.txt)."""
    out = {}
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_traffic.txt")) as fh:
            for ln in fh:
                p = ln.split()
                if len(p) >= 3 and not ln.startswith("#"):
                    out[p[0]] = (float(p[1]), p[2])
    except Exception:
        pass
    return out


# ------------------------------------------------------ replicas (N > 1)

def max_over_ranks(x: float, dist=None, device="cuda") -> float:
    """The slowest rank's time (or any per-rank figure's maximum); x itself
    when running alone.  Works with NCCL (device tensors) and gloo (CPU)."""
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank: float, world: int, seconds: float) -> float:
    """Whole-job Mkeys/s: every rank processed units_per_rank in at most
    `seconds` (the slowest rank's time)."""
    return units_per_rank * world / seconds / 1e6


# --------------------------------------------------------------- GPU arm

def run_gpu(args, wl, rank, world):
    import torch

    import cqf_gb300
    from cqf_gb300 import build

    build.build()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    keys = splitmix_dev(1, wl.n_insert, torch)
    absent = splitmix_dev(2, wl.n_get, torch)
    present = keys[: wl.n_get]
    out = torch.empty(wl.n_get, dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()

    qf = cqf_gb300.QF(wl.nbits)

    def step():
        qf.reset()
        for s, n in wl.batches:
            qf.bulk_insert(keys[s:s + n], n=n)
        e_ins.record()
        qf.bulk_get(present, out)
        qf.bulk_get(absent, out)
        e_get.record()
        for s in range(0, wl.n_get, wl.batch):
            n = min(wl.batch, wl.n_get - s)
            qf.bulk_delete(present[s:s + n], n=n)

    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e_ins, e_get = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    # correctness of one whole step, outside the timed region: the packed
    # filter after the inserts and after the deletes and both count arrays,
    # hashed for the word-for-word comparison with the reference's CUDA build
    # and the oracle
    qf.reset()
    for s, n in wl.batches:
        qf.bulk_insert(keys[s:s + n], n=n)
    ours_par = {"dump_insert": sha256_of(qf.export())}
    qf.bulk_get(present, out)
    ok_present = bool((out > 0).all().item())
    ours_par["counts_present"] = sha256_of(out)
    qf.bulk_get(absent, out)
    fp = int((out > 0).sum().item())
    ours_par["counts_absent"] = sha256_of(out)
    ours_par["false_positives"] = fp
    for s in range(0, wl.n_get, wl.batch):
        n = min(wl.batch, wl.n_get - s)
        qf.bulk_delete(present[s:s + n], n=n)
    ours_par["dump_delete"] = sha256_of(qf.export())
    ours_par["status"] = qf.status()
    torch.cuda.synchronize()

    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    time.sleep(0.4)
    qf.profile(True)
    launches0 = cqf_gb300.launch_count()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    per = {"insert": 0.0, "get": 0.0, "delete": 0.0}
    e0.record()
    for _ in range(args.steps):
        s0 = torch.cuda.Event(enable_timing=True)
        s0.record()
        step()
        s1 = torch.cuda.Event(enable_timing=True)
        s1.record()
        torch.cuda.synchronize()
        per["insert"] += s0.elapsed_time(e_ins)
        per["get"] += e_ins.elapsed_time(e_get)
        per["delete"] += e_get.elapsed_time(s1)
    e1.record()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ms = e0.elapsed_time(e1) / args.steps
    launches = cqf_gb300.launch_count() - launches0
    prof = qf.profile_read()
    qf.profile(False)
    clk = clocks.stop()
    status = qf.status()
    ms = max_over_ranks(ms, dist)
    value = job_rate(wl.key_ops, world, ms * 1e-3)
    ops = {k: {"ms": v / args.steps} for k, v in per.items()}
    ops["insert"]["mkeys_s"] = wl.n_insert / (ops["insert"]["ms"] * 1e3)
    ops["get"]["mkeys_s"] = 2 * wl.n_get / (ops["get"]["ms"] * 1e3)
    ops["delete"]["mkeys_s"] = wl.n_get / (ops["delete"]["ms"] * 1e3)

    # roofline per kernel phase, algorithmic bytes per launch / event time
    peak, peak_kind = measured_peak()
    t_ins_blocks = sum(wl.touched_blocks(n) for _, n in wl.batches)
    t_del_blocks = sum(wl.touched_blocks(min(wl.batch, wl.n_get - s)) for s in range(0, wl.n_get, wl.batch))
    phases = {
        "rebuild_insert": (prof["insert"], 2 * BLOCK_BYTES * t_ins_blocks + REBUILD_KEY_BYTES * wl.n_insert),
        "rebuild_delete": (prof["delete"], 2 * BLOCK_BYTES * t_del_blocks + REBUILD_KEY_BYTES * wl.n_get),
        "probe_get": (prof["get"], BYTES_GET * 2 * wl.n_get),
        "partition": (prof["partition"], PART_BYTES_PER_KEY * (wl.n_insert + wl.n_get)),
    }
    kernels = {}
    for name, (p, bytes_per_step) in phases.items():
        if p["calls"] == 0 or p["ms"] <= 0:
            continue
        t_step = p["ms"] / args.steps
        kernels[name] = {
            "ms_per_step": t_step,
            "calls_per_step": p["calls"] // args.steps,
            "algorithmic_gb_per_step": bytes_per_step / 1e9,
            "achieved_gbs": bytes_per_step / (t_step * 1e-3) / 1e9,
        }
    dom = max(kernels, key=lambda k: kernels[k]["ms_per_step"])
    d = kernels[dom]
    # units of the ncu traffic figures per bulk call: keys probed, regions
    # staged by the rebuild (both parities; every region holds keys here)
    nregions = wl.nslots >> qf.region_log()
    units_per_launch = {
        "probe_get": wl.n_get,
        "rebuild_insert": nregions,
        "rebuild_delete": nregions,
        "partition": (wl.n_insert + wl.n_get) / max(1, kernels.get("partition", {}).get("calls_per_step", 1)),
    }
    tr = profile_traffic()
    for k, kd in kernels.items():
        if k in tr:
            kd["dram_bytes_per_launch"] = tr[k][0] * units_per_launch[k]
    traffic = {"bytes_per_launch": kernels[dom]["dram_bytes_per_launch"]} if "dram_bytes_per_launch" in kernels[dom] else None
    roofline = {
        "bound": "hbm",
        "kernel": dom,
        "achieved": round(d["achieved_gbs"], 1),
        "peak": peak,
        "unit": "GB/s",
        "frac": round(d["achieved_gbs"] / peak, 4),
        "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback 6.8 TB/s",
        "traffic": traffic.get("bytes_per_launch") if traffic else None,
        "algorithmic_bytes_per_launch": d["algorithmic_gb_per_step"] * 1e9 / max(1, d["calls_per_step"]),
    }

    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(args, wl, qf, keys, absent, torch, dist, world)

    cpu = None
    cpu_par = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = run_cpu_sample(wl, keys, absent, args)
        cpu_par = cpu.pop("parity", None)

    ref_cuda = None
    if rank == 0 and world == 1 and not args.no_ref_cuda:
        qf.close()
        ref_cuda = run_ref_cuda(wl, keys, absent, ops, value, torch)
    parity = parity_block(wl.nbits, {"ours": ours_par, "oracle": cpu_par,
                                     "ref_cuda": (ref_cuda or {}).pop("parity", None)})

    workloads = {}
    if not args.no_skew and args.nbits == 28:
        qf.close()
        del keys, absent, present, out
        torch.cuda.empty_cache()
        workloads["skewed_counting"] = run_skew(args, torch, cqf_gb300)
    if not args.no_batched and rank == 0 and world == 1:
        qf.close()
        torch.cuda.empty_cache()
        workloads["many_filters"] = run_batched(args, torch, cqf_gb300)
    if not args.no_serve and rank == 0 and world == 1:
        qf.close()
        torch.cuda.empty_cache()
        workloads["serving"] = run_serving(args, torch, cqf_gb300)

    line = {
        "metric": METRIC,
        "value": round(value, 2),
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u64",
        "data": "synthetic (splitmix64 keys, generated on the device before timing)",
        "config": wl.describe() | {"parallelism": "replicas" if world > 1 else "single GPU"},
        "impl": "ours",
        "ops": {k: {kk: round(vv, 3) for kk, vv in v.items()} for k, v in ops.items()},
        "kernels": {k: {kk: round(vv, 4) if isinstance(vv, float) else vv for kk, vv in v.items()}
                    for k, v in kernels.items()},
        "roofline": roofline,
        "e2e": e2e,
        "cpu_baseline": cpu,
        "ref_cuda": ref_cuda,
        "workloads": workloads,
        "clocks": clk,
        "gpu_launches": int(launches),
        "gpu_launches_per_step": int(launches // args.steps),
        "check": {"present_all_found": ok_present, "false_positives_absent": fp, "status": status},
        "parity": parity,
    }
    qf.close()
    if dist:
        dist.destroy_process_group()
    return line


def run_e2e(args, wl, qf, keys_dev, absent_dev, torch, dist=None, world=1):
    """The same step through the C ABI from pinned host buffers: every input
    is copied host->device and every get result device->host inside the timed
    region, each step.  Insert batches go up through two rotating device
    buffers on one stream; the get and delete inputs go up on a second stream
    into buffers of their own, chunk by chunk between the insert batches (the
    step's inputs are known when it starts, and the inserts leave the copy
    engines mostly idle);
    get results come down on a third stream, chunk by chunk, as the gets
    finish; the bulk calls run on a fourth."""
    hk = torch.empty(wl.n_insert, dtype=torch.int64, pin_memory=True)
    ha = torch.empty(wl.n_get, dtype=torch.int64, pin_memory=True)
    hk.copy_(keys_dev.cpu())
    ha.copy_(absent_dev.cpu())
    hres = torch.empty(2 * wl.n_get, dtype=torch.int64, pin_memory=True)
    comp, copy, pre, down = (torch.cuda.Stream() for _ in range(4))
    B = wl.batch
    bufs = [torch.empty(B, dtype=torch.int64, device="cuda") for _ in range(2)]
    getbuf = torch.empty(2 * wl.n_get, dtype=torch.int64, device="cuda")
    delbuf = torch.empty(wl.n_get, dtype=torch.int64, device="cuda")
    resbuf = torch.empty(2 * wl.n_get, dtype=torch.int64, device="cuda")
    copied = [torch.cuda.Event() for _ in range(2)]
    done = [torch.cuda.Event() for _ in range(2)]  # bufs[b] consumed
    gets_in, dels_in = torch.cuda.Event(), torch.cuda.Event()
    gets_done, dels_done, drained = torch.cuda.Event(), torch.cuda.Event(), torch.cuda.Event()
    for e in done + [gets_done, dels_done]:
        e.record(comp)
    drained.record(down)
    qf.set_stream(comp)
    get_chunks = [(s, min(B, 2 * wl.n_get - s)) for s in range(0, 2 * wl.n_get, B)]

    # the get and delete inputs go up in batch-sized chunks, one after each
    # insert batch's copy, so that the copy engines alternate between the two
    # and no insert waits behind the whole 1.6 GB (a step that starts on idle
    # engines would otherwise queue its first inserts behind them)
    ups = []
    for s in range(0, wl.n_get, B):
        ups.append(("get", getbuf[s:s + min(B, wl.n_get - s)], hk[s:s + min(B, wl.n_get - s)]))
    for s in range(0, wl.n_get, B):
        n = min(B, wl.n_get - s)
        ups.append(("get", getbuf[wl.n_get + s:wl.n_get + s + n], ha[s:s + n]))
    for s in range(0, wl.n_get, B):
        ups.append(("del", delbuf[s:s + min(B, wl.n_get - s)], hk[s:s + min(B, wl.n_get - s)]))
    first_del = next(j for j, u in enumerate(ups) if u[0] == "del")

    def upload(j):
        # each buffer is refilled once the previous step's calls are done with it
        if j == 0:
            pre.wait_event(gets_done)
        if j == first_del:
            pre.wait_event(dels_done)
        with torch.cuda.stream(pre):
            ups[j][1].copy_(ups[j][2], non_blocking=True)
            if j == first_del - 1:
                gets_in.record(pre)
            if j == len(ups) - 1:
                dels_in.record(pre)

    def step():
        with torch.cuda.stream(comp):
            qf.reset()
        j = 0
        for i, (s, n) in enumerate(wl.batches):  # inserts through the rotating buffers
            b = i & 1
            copy.wait_event(done[b])
            with torch.cuda.stream(copy):
                bufs[b][:n].copy_(hk[s:s + n], non_blocking=True)
                copied[b].record(copy)
            comp.wait_event(copied[b])
            qf.bulk_insert_async(bufs[b], n, stream=comp)
            done[b].record(comp)
            if i >= 1 and j < len(ups):
                upload(j)
                j += 1
        while j < len(ups):
            upload(j)
            j += 1
        comp.wait_event(gets_in)
        comp.wait_event(drained)  # the previous step's results are down
        for s, n in get_chunks:
            qf.bulk_get_async(getbuf[s:s + n], resbuf[s:s + n], n, stream=comp)
            ev = torch.cuda.Event()
            ev.record(comp)
            down.wait_event(ev)
            with torch.cuda.stream(down):
                hres[s:s + n].copy_(resbuf[s:s + n], non_blocking=True)
        drained.record(down)
        gets_done.record(comp)
        comp.wait_event(dels_in)
        for s in range(0, wl.n_get, B):
            n = min(B, wl.n_get - s)
            qf.bulk_delete_async(delbuf[s:s + n], n, stream=comp)
        dels_done.record(comp)

    # the first passes over fresh pinned buffers run slower: warm up at
    # least three full steps
    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize()
    dt = max_over_ranks((time.perf_counter() - t0) / args.steps, dist)
    qf.set_stream(None)
    found = bool((hres[: wl.n_get] > 0).all().item())
    h2d = 8 * (wl.n_insert + 2 * wl.n_get + wl.n_get)
    return {
        "value": round(job_rate(wl.key_ops, world, dt), 2),
        "unit": UNIT,
        "ms_per_step": round(dt * 1e3, 3),
        "h2d_bytes_per_step": h2d,
        "d2h_bytes_per_step": 8 * 2 * wl.n_get,
        "path": "C ABI (gqf_bulk_*_async) from pinned host buffers: insert batches up through two rotating "
                "device buffers, the get and delete inputs up on a second stream during the inserts, get "
                "results down on a third stream as each chunk finishes, bulk calls on a fourth",
        "present_all_found": found,
    }


def run_ref_cuda(wl, keys, absent, ours_ops, ours_value, torch):
    """The reference's own CUDA build (its kernels compiled from its sources,
    driven by baseline/refgpu.py) on the same step, timed per call by wall
    clock around a synchronised call (the reference synchronises inside each
    bulk call).  Keys are copied to a scratch buffer before each call, outside
    the timing, because the reference overwrites them."""
    from baseline import refgpu

    if not refgpu.available():
        return {"unavailable": "reference cubin not built (needs the reference tree on an x86 host)"}
    r = refgpu.RefGPU(wl.nbits)
    scratch = torch.empty(wl.batch, dtype=torch.int64, device="cuda")
    out = torch.empty(wl.n_get, dtype=torch.int64, device="cuda")
    t = {"insert": 0.0, "get": 0.0, "delete": 0.0}
    par = {}  # hashes of its filter and counts, taken between the timed calls
    try:
        for s0, n in wl.batches:
            scratch[:n].copy_(keys[s0:s0 + n])
            torch.cuda.synchronize()
            a = time.perf_counter()
            r.bulk_insert(scratch, n)
            torch.cuda.synchronize()
            t["insert"] += time.perf_counter() - a
        par["dump_insert"] = sha256_of(r.dump())
        for name, probe in (("counts_present", keys[: wl.n_get]), ("counts_absent", absent)):
            torch.cuda.synchronize()
            a = time.perf_counter()
            r.bulk_get(probe, out)
            torch.cuda.synchronize()
            t["get"] += time.perf_counter() - a
            par[name] = sha256_of(out)
            if name == "counts_present":
                found = bool((out > 0).all().item())
            else:
                par["false_positives"] = int((out > 0).sum().item())
        for s0 in range(0, wl.n_get, wl.batch):
            n = min(wl.batch, wl.n_get - s0)
            scratch[:n].copy_(keys[s0:s0 + n])
            torch.cuda.synchronize()
            a = time.perf_counter()
            r.bulk_delete(scratch, n)
            torch.cuda.synchronize()
            t["delete"] += time.perf_counter() - a
        par["dump_delete"] = sha256_of(r.dump())
    finally:
        r.close()
    total = sum(t.values())
    rates = {"insert_mkeys_s": wl.n_insert / t["insert"] / 1e6,
             "get_mkeys_s": 2 * wl.n_get / t["get"] / 1e6,
             "delete_mkeys_s": wl.n_get / t["delete"] / 1e6}
    return {
        "value": round(wl.key_ops / total / 1e6, 3),
        "unit": UNIT,
        "seconds": round(total, 3),
        "ops": {k: round(v, 3) for k, v in rates.items()},
        "speedup": {
            "step": round(ours_value / (wl.key_ops / total / 1e6), 2),
            "insert": round(ours_ops["insert"]["mkeys_s"] / rates["insert_mkeys_s"], 2),
            "get": round(ours_ops["get"]["mkeys_s"] / rates["get_mkeys_s"], 2),
            "delete": round(ours_ops["delete"]["mkeys_s"] / rates["delete_mkeys_s"], 2),
        },
        "present_all_found": found,
        "parity": par,
        "what": "reference src/gqf.cu kernels compiled for sm_103a from its sources; host orchestration "
                "restated (baseline/refgpu.py), thrust::sort replaced by torch.sort",
    }


# ------------------------------------------------- skewed counting (config 3)

def _exact_check(qf, keys, mask, torch):
    """bulk_get of every distinct key (mod 2^(nbits+8)) equals its exact
    multiplicity in keys; returns (ok, distinct)."""
    u, c = torch.unique(keys & mask, return_counts=True)
    out = torch.empty_like(u)
    qf.bulk_get(u, out)
    torch.cuda.synchronize()
    return bool(torch.equal(out, c.to(torch.int64))), int(u.numel())


def _time_reps(fn, reps, torch):
    ts = []
    for _ in range(reps):
        torch.cuda.synchronize()
        a = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        ts.append(time.perf_counter() - a)
    return min(ts), statistics.median(ts)


def run_skew(args, torch, cqf_gb300):
    """Config 3 at full size on a fresh 2^28-slot filter per run:
    (i) 2^28 Zipf(1.5) draws over 2^24 splitmix64 keys (seed 3) through
    bulk_insert_reduce; (ii) canonical 31-mers of 2^20 150-bp reads (seed 4,
    1% substitutions, genome of 2^24 bases) through gqf_bulk_insert_kmers.
    Timed end to end on the device (events) per call, after warm-up; the
    reference's CUDA reduce path (baseline/refgpu.py) on the same multisets."""
    from cqf_gb300 import synth

    nbits = 28
    mask = (1 << (nbits + 8)) - 1
    res = {}
    keys = synth.zipf_keys_dev(3, 1 << 28, 1 << 24)
    reads = synth.dna_reads_dev(4, 1 << 20, 150, 1 << 24, 0.01)
    kmers = torch.empty(reads.shape[0] * 120, dtype=torch.int64, device="cuda")
    cqf_gb300.kmers_extract(reads, 31, kmers)
    kmers = kmers[kmers != -1]
    torch.cuda.synchronize()
    reps = max(2, min(args.steps, 5))
    with cqf_gb300.QF(nbits) as qf:
        for name, run, n, units in (
            ("zipf_reduce", lambda: qf.bulk_insert_reduce(keys), keys.numel(), "draws"),
            ("kmers_31", lambda: qf.bulk_insert_kmers(reads, 31), kmers.numel(), "k-mers"),
        ):
            def once():
                qf.reset()
                run()
            for _ in range(2):
                once()
            tmin, tmed = _time_reps(once, reps, torch)
            qf.reset()
            run()
            ok, distinct = _exact_check(qf, keys if name == "zipf_reduce" else kmers, mask, torch)
            res[name] = {"mkeys_s": round(n / tmed / 1e6, 1), "mkeys_s_best": round(n / tmin / 1e6, 1),
                         "ms": round(tmed * 1e3, 3), "keys": n, "units": units, "distinct": distinct,
                         "exact_counts_equal": ok, "status": qf.status()}
    if not args.no_ref_cuda:
        from baseline import refgpu

        if refgpu.available():
            scratch = torch.empty(keys.numel(), dtype=torch.int64, device="cuda")
            for name, src in (("zipf_reduce", keys), ("kmers_31", kmers)):
                r = refgpu.RefGPU(nbits)
                try:
                    n = src.numel()
                    scratch[:n].copy_(src)
                    torch.cuda.synchronize()
                    a = time.perf_counter()
                    r.bulk_insert_reduce(scratch, n)
                    torch.cuda.synchronize()
                    dt = time.perf_counter() - a
                finally:
                    r.close()
                res[name]["ref_cuda_mkeys_s"] = round(n / dt / 1e6, 1)
                res[name]["speedup_vs_ref_cuda"] = round(res[name]["mkeys_s"] / (n / dt / 1e6), 2)
            res["ref_cuda_what"] = ("reference kernels (hash_all, set_buffers_*, insert_from_buffers_thrust) "
                                    "with torch.sort + unique_consecutive for thrust sort + reduce_by_key; "
                                    "the reference's k-mer step is host code, so its arm starts from the "
                                    "extracted k-mers")
            del scratch
    del keys, reads, kmers
    torch.cuda.empty_cache()
    return res


# ------------------------------------------------ many-filter launch (config 4)

def batched_shapes(nfilters=4096, seed=7):
    """Config 4's filters from splitmix64 seed 7: nbits = 10 + (x >> 32) % 11
    (uniform in [10, 20]), load = 0.5 + 0.4 u (u a 53-bit uniform of the
    second stream); filter f gets floor(load * 2^nbits) keys."""
    from cqf_gb300 import synth

    x = synth.splitmix64(seed, nfilters)
    u = _u53(synth.splitmix64(seed + 1000, nfilters))
    nbits = (10 + (x >> np.uint64(32)) % np.uint64(11)).astype(np.int32)
    loads = 0.5 + 0.4 * u
    sizes = np.floor(loads * (2.0 ** nbits)).astype(np.int64)
    offsets = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    return nbits, sizes, offsets


def run_batched(args, torch, cqf_gb300):
    """Config 4: 4096 filters filled to their loads in one batch (uniform
    splitmix64 keys, seed 8) and queried with as many present and absent
    keys (seed 9).  One step = reset + insert + get present + get absent,
    captured once as a CUDA graph and replayed; the region size and the
    key-by-key threshold come from the set's autotuner.  The reference arm
    runs qf_malloc_device + bulk_insert + bulk_get (present, absent) per
    filter, one filter after another, as its API requires."""
    from cqf_gb300 import synth

    nbits, sizes, offsets = batched_shapes()
    total = int(offsets[-1])
    keys = synth.splitmix64_dev(8, total)
    absent = synth.splitmix64_dev(9, total)
    od = torch.from_numpy(offsets).cuda()
    cp = torch.empty(total, dtype=torch.int64, device="cuda")
    ca = torch.empty(total, dtype=torch.int64, device="cuda")
    fs = cqf_gb300.FilterSet(nbits, total)
    tune_ms = fs.tune(keys, od)
    cfg = fs.config()
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        fs.reset(stream=s)
        fs.insert(keys, od, stream=s)
        fs.get(keys, od, cp, stream=s)
        fs.get(absent, od, ca, stream=s)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        fs.reset(stream=s)
        fs.insert(keys, od, stream=s)
        fs.get(keys, od, cp, stream=s)
        fs.get(absent, od, ca, stream=s)
    for _ in range(3):
        g.replay()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = max(3, args.steps)
    e0.record()
    for _ in range(reps):
        g.replay()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    found = bool((cp > 0).all().item())
    fp = int((ca > 0).sum().item())
    status = fs.status()
    fs.close()
    ops = 3 * total
    res = {
        "filters": int(nbits.size), "nbits_range": [int(nbits.min()), int(nbits.max())],
        "keys_inserted": total, "key_ops_per_step": ops,
        "ms_per_step": round(ms, 3), "mkeys_s": round(ops / ms / 1e3, 1),
        "graph": "reset + insert + 2 gets captured once, replayed",
        "autotuned": cfg | {"tune_insert_ms": round(tune_ms, 3)},
        "present_all_found": found, "false_positives": fp, "status": status,
    }
    if not args.no_ref_cuda:
        from baseline import refgpu

        if refgpu.available():
            out = torch.empty(int(sizes.max()), dtype=torch.int64, device="cuda")
            scratch = torch.empty(int(sizes.max()), dtype=torch.int64, device="cuda")
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            ok = True
            sample = range(0, nbits.size, 16)  # every 16th filter: the same size law
            for f in sample:
                a, n = int(offsets[f]), int(sizes[f])
                r = refgpu.RefGPU(int(nbits[f]))
                scratch[:n].copy_(keys[a:a + n])
                r.bulk_insert(scratch, n)
                r.bulk_get(keys[a:a + n], out, n)
                if f % 256 == 0:
                    ok &= bool((out[:n] > 0).all().item())
                r.bulk_get(absent[a:a + n], out, n)
                r.close()
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            sops = 3 * int(sum(int(sizes[f]) for f in sample))
            rate = sops / dt / 1e6
            res["ref_cuda"] = {"sample_seconds": round(dt, 3), "sample_filters": len(sample), "mkeys_s": round(rate, 1),
                               "seconds_all_filters_est": round(ops / rate / 1e6, 1),
                               "present_found_sampled": ok,
                               "what": "per filter: device buffers + bulk_insert + bulk_get x2 of the reference's "
                                       "kernels (baseline/refgpu.py), synchronised as its API is; every 16th "
                                       "filter timed, rate over the sample's key operations"}
            res["speedup_vs_ref_cuda"] = round((ops / ms / 1e3) / rate, 1)
            # the same sample with the reference's filters allocated beforehand
            # and its keys staged: only its bulk calls timed
            filters = [refgpu.RefGPU(int(nbits[f])) for f in sample]
            stage = [keys[int(offsets[f]):int(offsets[f]) + int(sizes[f])].clone() for f in sample]
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for r, f, kf in zip(filters, sample, stage):
                a, n = int(offsets[f]), int(sizes[f])
                r.bulk_insert(kf, n)
                r.bulk_get(keys[a:a + n], out, n)
                r.bulk_get(absent[a:a + n], out, n)
            torch.cuda.synchronize()
            dt2 = time.perf_counter() - t0
            for r in filters:
                r.close()
            del filters, stage
            rate2 = sops / dt2 / 1e6
            res["ref_cuda_preallocated"] = {
                "sample_seconds": round(dt2, 3), "mkeys_s": round(rate2, 1),
                "what": "the same filters and calls with the reference's filters allocated and its keys copied "
                        "before the timed loop: bulk_insert + bulk_get x2 per filter only"}
            res["speedup_vs_ref_cuda_preallocated"] = round((ops / ms / 1e3) / rate2, 1)
    del keys, absent, cp, ca
    torch.cuda.empty_cache()
    return res


# ------------------------------------------------------ serving loop (config 5)

def _u53(x):
    return (x >> np.uint64(11)).astype(np.float64) * (1.0 / (1 << 53))


class ServeStream:
    """The request stream of the serving workload, from splitmix64 seed 11:
    per request u0 -> exponential inter-arrival (unit mean, scaled by the
    rate later), u1 -> op (50% get, 40% insert, 10% delete), u2 -> size
    2^(10 + 14 u2) keys (log-uniform in [2^10, 2^24]).  Inserts take fresh
    keys of one splitmix64 stream (seed 12) in order, deletes remove the
    oldest inserted keys, gets ask for the n keys of that stream around the
    insert cursor: up to n/2 already inserted (present unless deleted) and
    the rest not yet inserted (absent when the get runs).  The stream ends
    when inserted minus deleted keys reach 90% of the slots."""

    def __init__(self, nbits):
        from cqf_gb300 import synth

        self.nslots = 1 << nbits
        target = int(0.9 * self.nslots)
        reqs, ins, dele, i = [], 0, 0, 0
        chunk = 4096
        while ins - dele < target:
            u = _u53(synth.splitmix64(11, 3 * (i + chunk)))[3 * i:].reshape(-1, 3)
            for u0, u1, u2 in u:
                n = int(2 ** (10 + 14 * u2))
                gap = -np.log(max(u0, 1e-300))
                if u1 < 0.5:
                    reqs.append(("get", n, gap, (ins, dele)))
                elif u1 < 0.9:
                    n = min(n, target - (ins - dele))
                    reqs.append(("insert", n, gap, ins))
                    ins += n
                else:
                    n = min(n, ins - dele)
                    if n == 0:
                        continue
                    reqs.append(("delete", n, gap, dele))
                    dele += n
                if ins - dele >= target:
                    break
            i += chunk
        self.reqs = reqs
        self.n_insert = ins
        self.total_keys = sum(r[1] for r in reqs)
        self.mean_size = self.total_keys / len(reqs)


def run_serving(args, torch, cqf_gb300):
    """Config 5: one resident 2^30-slot filter served through gqf_server_*
    from pinned host buffers.  (1) saturated: the whole stream submitted at
    once -> sustained Mkeys/s; (2) Poisson arrivals at --serve-load of that
    rate, submitted in real time -> p50/p99 latency (submission to results
    on the host).  The reference arm runs the same stream one request at a
    time (copy in, call, copy out), in real time at the same arrival times,
    FIFO: its latencies are observed the same way."""
    import queue

    from cqf_gb300 import synth

    nbits = args.serve_nbits
    st = ServeStream(nbits)
    npool = st.n_insert + (1 << 24)
    pool = torch.empty(npool, dtype=torch.int64, pin_memory=True)
    for a in range(0, npool, 1 << 26):
        b = min(npool, a + (1 << 26))
        pool[a:b].copy_(synth._splitmix_range_dev(12, a, b, "cuda"))
    out_cap = 1 << 28
    outbuf = torch.empty(out_cap, dtype=torch.int64, pin_memory=True)
    outbuf.copy_(torch.zeros(out_cap, dtype=torch.int64, device="cuda"))  # first device writes, untimed
    torch.cuda.synchronize()

    def payload(r):
        """(keys, present range within them) of a request."""
        kind, n, _, arg = r
        if kind != "get":
            return pool[arg:arg + n], None
        ins, dele = arg
        s0 = max(0, ins - n // 2)
        return pool[s0:s0 + n], (max(dele, s0) - s0, ins - s0)

    def run(realtime_rate=None, nreq=None):
        reqs = st.reqs if nreq is None else st.reqs[:nreq]
        qf = cqf_gb300.QF(nbits)
        srv = cqf_gb300.Server(qf)
        ops = {"get": cqf_gb300.OP_GET, "insert": cqf_gb300.OP_INSERT, "delete": cqf_gb300.OP_DELETE}
        q = queue.Queue()
        checks = {"ok": True, "checked": 0}
        lat = []
        prog = {"done": -1}

        def waiter():
            while True:
                item = q.get()
                if item is None:
                    return
                seq, t, out, pr = item
                lat.append(srv.wait(t))
                if out is not None:  # the inserted, undeleted keys are found
                    a, b = pr
                    b = min(b, a + 4096)
                    checks["ok"] &= bool((out[a:b] > 0).all())
                    checks["checked"] += 1
                prog["done"] = seq

        th = threading.Thread(target=waiter)
        th.start()
        users = []  # (seq, start, end) of output slices still to be checked
        oat = 0
        t0 = time.perf_counter()
        sched = 0.0
        lag = 0.0
        for seq, r in enumerate(reqs):
            kind, n = r[0], r[1]
            if realtime_rate:
                sched += r[2] / realtime_rate
                now = time.perf_counter() - t0
                if sched > now:
                    time.sleep(sched - now)
                lag = max(lag, time.perf_counter() - t0 - sched)
            keys, pr = payload(r)
            out = None
            if kind == "get":
                if oat + n > out_cap:
                    oat = 0
                a, b = oat, oat + n
                oat = b
                # reuse an output slice only after its previous request was checked
                while any(sq > prog["done"] and u0 < b and a < u1 for sq, u0, u1 in users):
                    time.sleep(50e-6)
                users = [u for u in users if u[0] > prog["done"]] + [(seq, a, b)]
                out = outbuf[a:b].numpy()
            t = srv.submit(ops[kind], keys, out)
            q.put((seq, t, out, pr))
        q.put(None)
        th.join()
        srv.drain()
        dt = time.perf_counter() - t0
        stats = srv.stats()
        srv.close()
        qf.close()
        lat_sorted = np.sort(np.array(lat))
        return {"seconds": dt, "mkeys_s": sum(r[1] for r in reqs) / dt / 1e6,
                "p50_ms": float(np.percentile(lat_sorted, 50)), "p99_ms": float(np.percentile(lat_sorted, 99)),
                "max_ms": float(lat_sorted[-1]), "launches": int(stats["launches"]),
                "peak_staging_gb": stats["peak_staging_bytes"] / 1e9, "staging_gb": stats["staging_bytes"] / 1e9,
                "submit_lag_max_ms": lag * 1e3, "present_found": checks["ok"],
                "gets_checked": checks["checked"]}

    run(None, 64)  # warm-up on a fresh filter and server, untimed
    sat = run(None)
    rate = args.serve_load * sat["mkeys_s"] * 1e6 / st.mean_size  # requests per second
    pois = run(rate)
    rnd = lambda d: {k: round(v, 3) if isinstance(v, float) else v for k, v in d.items()}
    res = {
        "requests": len(st.reqs),
        "keys": st.total_keys,
        "mix": {k: sum(1 for r in st.reqs if r[0] == k) for k in ("get", "insert", "delete")},
        "nbits": nbits,
        "saturated": rnd(sat),
        "poisson": rnd(pois) | {"rate_req_s": round(rate, 1), "offered_mkeys_s": round(rate * st.mean_size / 1e6, 1)},
        "what": "gqf_server from pinned host buffers; latency = submission to results on the host",
    }
    if not args.no_ref_cuda:
        try:
            res["ref_cuda"] = run_serving_ref(st, nbits, pool, rate, torch)
        except Exception as e:  # the baseline leg must not cost the line
            res["ref_cuda"] = {"error": f"{type(e).__name__}: {e}"}
        if "poisson_p99_ms" in res["ref_cuda"]:
            res["p99_ref_cuda_over_ours"] = round(res["ref_cuda"]["poisson_p99_ms"] / max(1e-9, pois["p99_ms"]), 2)
    del pool, outbuf
    return res


def run_serving_ref(st, nbits, pool, rate, torch):
    """The reference's CUDA build as a server: one request at a time (copy
    in, bulk call, copy out).  First back to back on one filter (its service
    times: busy seconds and sustained rate), then on a fresh filter in real
    time at the same Poisson arrival times as our arm, each request served
    when it has arrived and the previous one is done (FIFO): its latencies
    are observed on the host clock, arrival to results."""
    from baseline import refgpu

    if not refgpu.available():
        return {"unavailable": "reference cubin not built"}
    dbuf = torch.empty(1 << 24, dtype=torch.int64, device="cuda")
    dout = torch.empty(1 << 24, dtype=torch.int64, device="cuda")
    hout = torch.empty(1 << 24, dtype=torch.int64, pin_memory=True)
    dout.zero_()
    hout.copy_(dout)  # first device writes to the pinned buffer, untimed (as for our arm)

    def serve(r, kind, n, arg):
        s0 = arg if kind != "get" else max(0, arg[0] - n // 2)
        dbuf[:n].copy_(pool[s0:s0 + n], non_blocking=True)
        if kind == "get":
            r.bulk_get(dbuf, dout, n)
            hout[:n].copy_(dout[:n], non_blocking=True)
        else:
            (r.bulk_insert if kind == "insert" else r.bulk_delete)(dbuf, n)
        torch.cuda.synchronize()

    service = []
    r = refgpu.RefGPU(nbits)
    try:
        for kind, n, _, arg in st.reqs:
            torch.cuda.synchronize()
            a = time.perf_counter()
            serve(r, kind, n, arg)
            service.append(time.perf_counter() - a)
    finally:
        r.close()
    arrivals = np.cumsum([q[2] for q in st.reqs]) / rate
    lat = []
    r = refgpu.RefGPU(nbits)
    try:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for (kind, n, _, arg), arr in zip(st.reqs, arrivals):
            wait = arr - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(wait)
            serve(r, kind, n, arg)
            lat.append(time.perf_counter() - t0 - arr)
        span = time.perf_counter() - t0
    finally:
        r.close()
    lat = np.array(lat) * 1e3
    busy = sum(service)
    return {"busy_seconds": round(busy, 3), "mkeys_s": round(st.total_keys / busy / 1e6, 1),
            "poisson_p50_ms": round(float(np.percentile(lat, 50)), 3),
            "poisson_p99_ms": round(float(np.percentile(lat, 99)), 3),
            "poisson_seconds": round(span, 3),
            "what": "reference CUDA build, one request at a time (copy in, bulk call, copy out): back to back "
                    "for its service rate, then in real time at the same Poisson arrival times, FIFO, "
                    "latencies observed from arrival to results"}


# --------------------------------------------------------------- CPU arms

def cpu_threads(args):
    return args.cpu_threads or os.cpu_count() or 1


def run_cpu_sample(wl, keys_dev, absent_dev, args):
    """The oracle (the reference's algorithm restated in C) on the host cores,
    on the full step's inputs once: a bounded sample of about 5-30 s."""
    import oracle

    oracle.build()
    keys = keys_dev.cpu().numpy().view(np.uint64)
    absent = absent_dev.cpu().numpy().view(np.uint64)
    return cpu_step(wl, keys, absent, cpu_threads(args), oracle, kind="port", parity=True)


def cpu_step(wl, keys, absent, threads, oracle, kind, parity=False):
    """One full step on the oracle; with parity, also the hashes of its
    filter after the inserts and the deletes and of its count arrays, taken
    outside the timed spans."""
    o = oracle.Oracle(wl.nbits, threads=threads)
    par = {}
    t0 = time.perf_counter()
    for s, n in wl.batches:
        o.bulk_insert(keys[s:s + n])
    t1 = time.perf_counter()
    if parity:
        par["dump_insert"] = sha256_of(o.dump())
    t1b = time.perf_counter()
    c1 = o.bulk_get(keys[: wl.n_get])
    c2 = o.bulk_get(absent)
    t2 = time.perf_counter()
    for s in range(0, wl.n_get, wl.batch):
        o.bulk_delete(keys[s:min(wl.n_get, s + wl.batch)])
    t3 = time.perf_counter()
    if parity:
        par["counts_present"] = sha256_of(c1.view(np.int64))
        par["counts_absent"] = sha256_of(c2.view(np.int64))
        par["false_positives"] = int((c2 > 0).sum())
        par["dump_delete"] = sha256_of(o.dump())
    o.close()
    t_ins, t_get, t_del = t1 - t0, t2 - t1b, t3 - t2
    dt = t_ins + t_get + t_del
    assert (c1 > 0).all()
    res = {
        "value": round(wl.key_ops / dt / 1e6, 3),
        "unit": UNIT,
        "cores": threads,
        "kind": kind,
        "sample": f"the full step once ({wl.key_ops} key ops), {threads} threads: regions of one parity "
                  f"in parallel, as the reference's even/odd launch; hash + sort single-threaded",
        "seconds": round(dt, 3),
        "ops": {"insert_mkeys_s": round(wl.n_insert / t_ins / 1e6, 3),
                "get_mkeys_s": round(2 * wl.n_get / t_get / 1e6, 3),
                "delete_mkeys_s": round(wl.n_get / t_del / 1e6, 3)},
    }
    if parity:
        res["parity"] = par
    return res


def run_reference(args, wl, rank, world):
    """--impl reference: the reference's CPU implementation of the path (the
    oracle port on this host; the reference's own host code is x86-only) on
    all host cores, each step one full step of the workload."""
    if rank != 0:
        return None
    import oracle

    oracle.build()
    keys = oracle.splitmix64(1, wl.n_insert)
    absent = oracle.splitmix64(2, wl.n_get)
    threads = cpu_threads(args)
    for _ in range(args.warmup):
        cpu_step(wl, keys, absent, threads, oracle, "port")
    vals, secs = [], []
    for _ in range(args.steps):
        r = cpu_step(wl, keys, absent, threads, oracle, "port")
        vals.append(r["value"])
        secs.append(r["seconds"])
    dt = sum(secs) / len(secs)
    v = wl.key_ops / dt / 1e6
    return {
        "metric": METRIC,
        "value": round(v, 3),
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(dt * 1e3, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u64",
        "data": "synthetic (splitmix64 keys)",
        "config": wl.describe() | {"parallelism": "replicas" if world > 1 else "single GPU"},
        "impl": "reference",
        "cpu_baseline": {"value": round(v, 3), "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"each step is the full workload ({wl.key_ops} key ops) on {threads} threads"},
        "e2e": {"value": round(v, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


# ------------------------------------------------- single-kernel profiling

def run_case(a):
    """--case: one fill and a few bulk calls on one filter (see the module
    docstring); prints one JSON line of CUDA-event times."""
    import math

    import torch

    import cqf_gb300
    from cqf_gb300 import build, synth

    build.build()
    if a.case in ("zipf", "kmers"):
        if a.case == "zipf":
            data = synth.zipf_keys_dev(3, 1 << 28, 1 << 24)
        else:
            data = synth.dna_reads_dev(4, 1 << 20, 150, 1 << 24, 0.01)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        out = {"nbits": a.nbits, "op": a.case, "calls": a.extra, "ms": []}
        with cqf_gb300.QF(a.nbits) as qf:
            for _ in range(a.extra):
                qf.reset()
                e0.record()
                if a.case == "zipf":
                    qf.bulk_insert_reduce(data)
                else:
                    qf.bulk_insert_kmers(data, 31)
                e1.record()
                torch.cuda.synchronize()
                out["ms"].append(round(e0.elapsed_time(e1), 3))
            out["status"] = qf.status()
            out["counters"] = qf.counters()
        return out
    B = a.case_batch
    n_fill = int(a.load * (1 << a.nbits))
    n_extra = a.extra * B
    keys = synth.splitmix64_dev(1, n_fill + (n_extra if a.case == "insert" else 0))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    out = {"nbits": a.nbits, "load": a.load, "batch": B, "op": a.case, "fill_calls": math.ceil(n_fill / B)}
    with cqf_gb300.QF(a.nbits) as qf:
        e0.record()
        for s in range(0, n_fill, B):
            qf.bulk_insert(keys[s:min(s + B, n_fill)])
        e1.record()
        torch.cuda.synchronize()
        out["fill_ms"] = round(e0.elapsed_time(e1), 3)
        res = torch.empty(B, dtype=torch.int64, device="cuda")
        e0.record()
        for i in range(a.extra):
            if a.case == "insert":
                qf.bulk_insert(keys[n_fill + i * B:n_fill + (i + 1) * B])
            else:
                s = (i * B) % max(1, n_fill - B)
                chunk = keys[s:s + B]
                if a.case == "delete":
                    qf.bulk_delete(chunk)
                else:
                    qf.bulk_get(chunk, res)
        e1.record()
        torch.cuda.synchronize()
        out["extra_ms"] = round(e0.elapsed_time(e1), 3)
        out["status"] = qf.status()
        out["counters"] = qf.counters()
    return out


def main():
    args = parse()
    if args.case:
        print(json.dumps(run_case(args)), flush=True)
        return
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    wl = Workload(args.nbits, args.batch_log, args.get_log)
    if args.impl == "reference":
        line = run_reference(args, wl, rank, world)
    else:
        line = run_gpu(args, wl, rank, world)
    if rank == 0 and line is not None:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
