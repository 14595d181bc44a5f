"""Seeded synthetic inputs for the GQF workloads (host numpy or device torch).

Both variants of each generator return identical values: they use only
integer arithmetic and IEEE float64 comparisons.

* splitmix64(seed, n): out[i] = mix(seed + (i + 1) * 0x9E3779B97F4A7C15),
  the uniform keys of the bulk workloads.
* zipf_keys(seed, n, nkeys, s): n draws from a Zipf(s) law over nkeys
  distinct splitmix64 keys (rank r has weight r^-s); ranks come from an
  inverse-CDF lookup of 53-bit uniforms.
* dna_reads(seed, nreads, read_len, genome_len, err): fixed-length ASCII
  reads sampled from a random genome, half of them reverse-complemented, each
  base substituted with probability err.
"""
from __future__ import annotations

import numpy as np

GOLDEN = 0x9E3779B97F4A7C15
_M1 = 0xBF58476D1CE4E5B9
_M2 = 0x94D049BB133111EB


def _i64(v: int) -> int:
    return int(np.uint64(v).view(np.int64))


def splitmix64(seed: int, n: int) -> np.ndarray:
    x = np.uint64(seed) + np.arange(1, n + 1, dtype=np.uint64) * np.uint64(GOLDEN)
    z = (x ^ (x >> np.uint64(30))) * np.uint64(_M1)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(_M2)
    return z ^ (z >> np.uint64(31))


def splitmix64_dev(seed: int, n: int, device="cuda"):
    """splitmix64 on the device as int64 (the same bits as the numpy uint64)."""
    import torch

    out = torch.empty(n, dtype=torch.int64, device=device)
    chunk = 1 << 26
    for a in range(0, n, chunk):
        b = min(n, a + chunk)
        out[a:b] = _splitmix_range_dev(seed, a, b, device)
    return out


def zipf_cdf(nkeys: int, s: float = 1.5) -> np.ndarray:
    w = np.arange(1, nkeys + 1, dtype=np.float64) ** (-s)
    c = np.cumsum(w)
    return c / c[-1]


def _u53(x: np.ndarray) -> np.ndarray:
    return (x >> np.uint64(11)).astype(np.float64) * (1.0 / (1 << 53))


def zipf_keys(seed: int, n: int, nkeys: int, s: float = 1.5) -> np.ndarray:
    cdf = zipf_cdf(nkeys, s)
    pool = splitmix64(seed, nkeys)
    r = np.searchsorted(cdf, _u53(splitmix64(seed + 1, n)), side="right")
    return pool[np.minimum(r, nkeys - 1)]


def zipf_keys_dev(seed: int, n: int, nkeys: int, s: float = 1.5, device="cuda"):
    import torch

    cdf = torch.from_numpy(zipf_cdf(nkeys, s)).to(device)
    pool = splitmix64_dev(seed, nkeys, device)
    out = torch.empty(n, dtype=torch.int64, device=device)
    chunk = 1 << 26
    for a in range(0, n, chunk):
        b = min(n, a + chunk)
        x = _splitmix_range_dev(seed + 1, a, b, device)
        u = ((x >> 11) & ((1 << 53) - 1)).to(torch.float64) * (1.0 / (1 << 53))
        r = torch.searchsorted(cdf, u, right=True).clamp_(max=nkeys - 1)
        out[a:b] = pool[r]
    return out


def _splitmix_range_dev(seed: int, a: int, b: int, device):
    import torch

    g, m1, m2 = _i64(GOLDEN), _i64(_M1), _i64(_M2)
    x = torch.arange(a + 1, b + 1, dtype=torch.int64, device=device) * g + _i64(seed)
    x = (x ^ ((x >> 30) & ((1 << 34) - 1))) * m1
    x = (x ^ ((x >> 27) & ((1 << 37) - 1))) * m2
    return x ^ ((x >> 31) & ((1 << 33) - 1))


_ACGT = np.frombuffer(b"ACGT", dtype=np.uint8)


def dna_reads(seed: int, nreads: int, read_len: int = 150, genome_len: int = 1 << 24,
              err: float = 0.01) -> np.ndarray:
    """uint8 [nreads, read_len] of 'A' 'C' 'G' 'T'."""
    words = splitmix64(seed, (genome_len + 31) // 32)
    i = np.arange(genome_len, dtype=np.uint64)
    genome = ((words[(i >> np.uint64(5)).astype(np.int64)] >> ((i & np.uint64(31)) * np.uint64(2)))
              & np.uint64(3)).astype(np.int64)
    span = genome_len - read_len + 1
    pos = (((splitmix64(seed + 1, nreads) >> np.uint64(32)) * np.uint64(span)) >> np.uint64(32)).astype(np.int64)
    rev = (splitmix64(seed + 2, nreads) >> np.uint64(63)).astype(bool)
    b = genome[pos[:, None] + np.arange(read_len)[None, :]]
    b[rev] = 3 - b[rev][:, ::-1]
    e = splitmix64(seed + 3, nreads * read_len).reshape(nreads, read_len)
    thr = np.uint64(int(err * (1 << 32)))
    hit = (e >> np.uint64(32)) < thr
    alt = (b + 1 + ((e & np.uint64(0xFFFF)) % np.uint64(3)).astype(np.int64)) & 3
    b = np.where(hit, alt, b)
    return _ACGT[b]


def dna_reads_dev(seed: int, nreads: int, read_len: int = 150, genome_len: int = 1 << 24,
                  err: float = 0.01, device="cuda"):
    import torch

    words = splitmix64_dev(seed, (genome_len + 31) // 32, device)
    i = torch.arange(genome_len, dtype=torch.int64, device=device)
    genome = (words[i >> 5] >> ((i & 31) * 2)) & 3
    span = genome_len - read_len + 1
    pos = ((((splitmix64_dev(seed + 1, nreads, device) >> 32) & 0xFFFFFFFF) * span) >> 32)
    rev = ((splitmix64_dev(seed + 2, nreads, device) >> 63) & 1).bool()
    acgt = torch.tensor(list(b"ACGT"), dtype=torch.uint8, device=device)
    out = torch.empty((nreads, read_len), dtype=torch.uint8, device=device)
    thr = int(err * (1 << 32))
    ar = torch.arange(read_len, device=device)
    chunk = max(1, (1 << 24) // read_len)
    for a in range(0, nreads, chunk):
        bb = min(nreads, a + chunk)
        b = genome[pos[a:bb, None] + ar[None, :]]
        rv = rev[a:bb]
        b = torch.where(rv[:, None], 3 - b.flip(1), b)
        e = _splitmix_range_dev(seed + 3, a * read_len, bb * read_len, device).view(bb - a, read_len)
        hit = ((e >> 32) & 0xFFFFFFFF) < thr
        alt = (b + 1 + (e & 0xFFFF) % 3) & 3
        out[a:bb] = acgt[torch.where(hit, alt, b)]
    return out
