"""Properties of the reference's counter encoding (src/gqf.cu:1216-1273) that
the rebuild's run merge relies on, checked on the oracle's encoder (pinned
to the reference by the golden vectors in test_oracle.py).

* A run whose slots strictly increase holds only counts of one: every
  counter of two or more repeats its remainder ([r, r], [0, 0, 0]) or steps
  down after it ([r, 0, r], [r, d, ..., r] with d < r, and for remainder 0
  a trailing [..., 0, 0]).  The merge takes a single key into such a run
  without the counter decoder.
* One more count lengthens a counter by at most one slot, and no counter
  takes more than 12 slots: the bound on a merged run's length.
"""
import numpy as np

import oracle


def _run(rems, counts):
    out = []
    for r, c in zip(rems, counts):
        out += oracle.encode_counter(int(r), int(c))
    return out


def test_a_strictly_increasing_run_holds_only_single_counts():
    rng = np.random.default_rng(5)
    special = [0, 1, 2, 3, 127, 253, 254, 255]
    for _ in range(4000):
        m = int(rng.integers(1, 7))
        pool = special if rng.random() < 0.3 else range(256)
        rems = sorted(rng.choice(list(pool), size=min(m, len(pool)), replace=False).tolist())
        counts = [1 if rng.random() < 0.7 else int(rng.choice([2, 3, 4, 5, 254, 255, 256, 258, 1000, 65536]))
                  for _ in rems]
        run = _run(rems, counts)
        increasing = all(a < b for a, b in zip(run, run[1:]))
        assert increasing == all(c == 1 for c in counts), (rems, counts, run)


def test_one_more_count_adds_at_most_one_slot():
    for r in (0, 1, 2, 3, 127, 253, 254, 255):
        prev = len(oracle.encode_counter(r, 1))
        for c in range(2, 70000):
            n = len(oracle.encode_counter(r, c))
            assert n - prev in (0, 1), (r, c)
            prev = n


def test_no_counter_takes_more_than_twelve_slots():
    edges = [2**64 - 1, 2**63, 2**32, 2**32 - 1]
    for base in (254, 255):
        for k in range(1, 9):
            for d in (-2, -1, 0, 1, 2):
                edges.append(base**k + 3 + d)
                edges.append(base**k + 4 + d)
    for r in range(256):
        for c in edges:
            if 0 < c < 2**64:
                n = len(oracle.encode_counter(r, c))
                assert 1 <= n <= 12, (r, c, n)
        # lengths never shrink as counts grow
        lens = [len(oracle.encode_counter(r, c)) for c in sorted(x for x in edges if 0 < x < 2**64)]
        assert lens == sorted(lens), r
