"""The oracle's canonical k-mers against the definition, string by string,
and the synthetic read / Zipf generators (host and device variants agree)."""
import numpy as np
import pytest

import oracle
from cqf_gb300 import synth

_COMP = {"A": "T", "C": "G", "G": "C", "T": "A"}
_CODE = {"A": 0, "C": 1, "G": 2, "T": 3}


def _pack(s: str) -> int:
    v = 0
    for ch in s:
        v = (v << 2) | _CODE[ch]
    return v


def _canonical(s: str) -> int:
    s = s.upper()
    if any(ch not in _CODE for ch in s):
        return (1 << 64) - 1
    rc = "".join(_COMP[ch] for ch in reversed(s))
    return min(_pack(s), _pack(rc))


@pytest.mark.parametrize("k", [1, 5, 21, 31, 32])
def test_canonical_kmers_match_definition(k):
    rng = np.random.default_rng(k)
    reads = np.frombuffer(b"ACGTacgtN", dtype=np.uint8)[rng.integers(0, 9, size=(6, 45))]
    reads[0] = np.frombuffer(b"ACGT" * 11 + b"A", dtype=np.uint8)  # no skipped window
    got = oracle.canonical_kmers(reads, k)
    want = [_canonical(bytes(r[p:p + k]).decode()) for r in reads for p in range(45 - k + 1)]
    assert got.tolist() == want


def test_exact_counts_mod_key_bits():
    keys = np.array([5, 5, 7, 5 + (1 << 18), 9], dtype=np.uint64)  # nbits 10: keys mod 2^18
    got = oracle.exact_counts(keys, 10, np.array([5, 7, 9, 11], dtype=np.uint64))
    assert got.tolist() == [3, 1, 1, 0]


def test_generators_host_and_device_agree():
    torch = pytest.importorskip("torch")
    a = synth.splitmix64(11, 5000)
    b = synth.splitmix64_dev(11, 5000, "cpu").numpy().view(np.uint64)
    assert np.array_equal(a, b)
    assert np.array_equal(synth.splitmix64(1, 1000), oracle.splitmix64(1, 1000))
    z = synth.zipf_keys(3, 1 << 15, 1 << 10)
    zd = synth.zipf_keys_dev(3, 1 << 15, 1 << 10, device="cpu").numpy().view(np.uint64)
    assert np.array_equal(z, zd)
    # rank 1 dominates a Zipf(1.5) law: about 1 / zeta(1.5) of the draws
    top = np.unique(z, return_counts=True)[1].max() / z.size
    assert 0.35 < top < 0.42
    r = synth.dna_reads(4, 300, 150, 1 << 14)
    rd = synth.dna_reads_dev(4, 300, 150, 1 << 14, device="cpu").numpy()
    assert np.array_equal(r, rd)
    assert set(np.unique(r).tolist()) <= set(b"ACGT")
    del torch
