"""Filter sets (gqf_set_*): many filters of uneven sizes in one launch per
phase.  Every filter of a set must hold exactly what a single filter of the
same size holds after the same keys (byte-exact exports, equal counts), under
every region size and key-by-key setting, and a captured CUDA graph of the
operations must replay to the same result."""
import numpy as np
import pytest

import oracle
from cqf_gb300 import synth
from tests.gpu_util import dev, first_diff, gpu_get, host

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gq():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import cqf_gb300
    from cqf_gb300 import build

    build.build()
    cqf_gb300.load()
    return cqf_gb300


def _workload(seed, nfilters, lo, hi, load_lo=0.5, load_hi=0.9):
    rng = np.random.default_rng(seed)
    nbits = rng.integers(lo, hi + 1, size=nfilters)
    loads = rng.uniform(load_lo, load_hi, size=nfilters)
    sizes = (loads * (1 << nbits)).astype(np.int64)
    sizes[rng.integers(0, nfilters)] = 0  # one empty filter
    offsets = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint64)
    keys = synth.splitmix64(seed + 100, int(offsets[-1]))
    absent = synth.splitmix64(seed + 200, int(offsets[-1]))
    return nbits, offsets, keys, absent


@pytest.mark.parametrize("log_region,sparse", [(11, 0xFFFFFFFF), (11, 0), (12, 1 << 20), (13, 0xFFFFFFFF)])
def test_set_matches_single_filters(gq, log_region, sparse):
    nbits, offsets, keys, absent = _workload(7, 24, 8, 15)
    with gq.FilterSet(nbits, keys.size) as fs:
        fs.config(log_region=log_region, sparse_max=sparse)
        kd, od = dev(keys), dev(offsets)
        # insert in two halves of every filter, then delete a third
        half = [(int(offsets[f]), int(offsets[f] + (offsets[f + 1] - offsets[f]) // 2)) for f in range(len(nbits))]
        first = np.concatenate([keys[a:b] for a, b in half])
        foff = np.concatenate([[0], np.cumsum([b - a for a, b in half])]).astype(np.uint64)
        second = np.concatenate([keys[b:int(offsets[f + 1])] for f, (a, b) in enumerate(half)])
        soff = np.concatenate([[0], np.cumsum([int(offsets[f + 1]) - b for f, (a, b) in enumerate(half)])]).astype(np.uint64)
        fs.insert(dev(first), dev(foff))
        fs.insert(dev(second), dev(soff))
        dl = [keys[int(offsets[f]):int(offsets[f]) + int(offsets[f + 1] - offsets[f]) // 3] for f in range(len(nbits))]
        doff = np.concatenate([[0], np.cumsum([d.size for d in dl])]).astype(np.uint64)
        fs.delete(dev(np.concatenate(dl)), dev(doff))
        import torch

        cp = torch.zeros(keys.size, dtype=torch.int64, device="cuda")
        ca = torch.zeros(keys.size, dtype=torch.int64, device="cuda")
        fs.get(kd, od, cp)
        fs.get(dev(absent), od, ca)
        torch.cuda.synchronize()
        cp, ca = host(cp), host(ca)
        assert fs.status() & ~gq.STATUS_DEFERRED == 0
        for f, nb in enumerate(nbits):
            a, b = int(offsets[f]), int(offsets[f + 1])
            with gq.QF(int(nb)) as qf:
                qf.bulk_insert(dev(keys[a:b]))
                if dl[f].size:
                    qf.bulk_delete(dev(dl[f]))
                want = qf.export()
                got = fs.export(f)
                assert np.array_equal(want, got), (f, int(nb), first_diff(want, got))
                assert np.array_equal(cp[a:b], gpu_get(qf, keys[a:b]))
                assert np.array_equal(ca[a:b], gpu_get(qf, absent[a:b]))


def test_set_matches_oracle(gq):
    nbits, offsets, keys, _ = _workload(3, 6, 10, 13)
    with gq.FilterSet(nbits, keys.size) as fs:
        fs.insert(dev(keys), dev(offsets))
        for f, nb in enumerate(nbits):
            o = oracle.Oracle(int(nb))
            o.bulk_insert(keys[int(offsets[f]):int(offsets[f + 1])])
            a, b = o.dump(), fs.export(f)
            assert np.array_equal(a, b), (f, first_diff(a, b))


def test_set_graph_replay(gq):
    """The operations only enqueue work: captured once into a CUDA graph,
    each replay rebuilds the same filters."""
    import torch

    nbits, offsets, keys, absent = _workload(11, 40, 9, 14)
    kd, od, ad = dev(keys), dev(offsets), dev(absent)
    both = torch.cat([kd, ad])
    boff = dev(np.concatenate([offsets, offsets[1:] + offsets[-1]]))
    out = torch.zeros(2 * keys.size, dtype=torch.int64, device="cuda")
    with gq.FilterSet(np.concatenate([nbits, nbits]), 2 * keys.size) as fs, \
            gq.FilterSet(nbits, keys.size) as eager:
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):  # one eager call of each kind configures the kernels
            fs.reset(stream=s)
            fs.insert(torch.cat([kd, kd]), boff, stream=s)
            fs.get(both, boff, out, stream=s)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            fs.reset(stream=s)
            fs.insert(torch.cat([kd, kd]), boff, stream=s)
            fs.get(both, boff, out, stream=s)
        eager.insert(kd, od)
        want = eager.export(0)
        for rep in range(3):
            out.zero_()
            g.replay()
            torch.cuda.synchronize()
            for f in range(len(nbits)):
                assert np.array_equal(fs.export(f), eager.export(f)), (rep, f)
        o = host(out)
        ref = torch.zeros(keys.size, dtype=torch.int64, device="cuda")
        eager.get(kd, od, ref)
        torch.cuda.synchronize()
        assert np.array_equal(o[: keys.size], host(ref))
        assert want is not None


def test_set_tune_picks_a_config_and_leaves_set_empty(gq):
    nbits, offsets, keys, _ = _workload(5, 16, 10, 16)
    with gq.FilterSet(nbits, keys.size) as fs:
        ms = fs.tune(dev(keys), dev(offsets))
        cfg = fs.config()
        assert ms > 0 and cfg["log_region"] in (11, 12, 13)
        with gq.QF(int(nbits[0])) as qf:
            assert np.array_equal(fs.export(0), qf.export())  # empty after tuning


def test_set_rejects_bad_input(gq):
    with pytest.raises(RuntimeError):
        gq.FilterSet([5], 10)
    with gq.FilterSet([10, 12], 100) as fs:
        with pytest.raises(RuntimeError):
            fs.insert(dev(np.zeros(200, dtype=np.uint64)), dev(np.array([0, 100, 200], dtype=np.uint64)))
