"""The serving loop (gqf_server_*): every request's result is the same alone
and in the mix.  A mixed stream submitted at once (so that the server
coalesces and overlaps it) is compared request by request with the same
requests run one at a time through the plain bulk calls, and the final
filters are compared byte for byte."""
import threading

import numpy as np
import pytest

import oracle
from cqf_gb300 import synth
from tests.gpu_util import dev, first_diff, gpu_get, host

pytestmark = pytest.mark.gpu

GET, INSERT, DELETE, REDUCE = 0, 1, 2, 3


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


def _stream(seed, nbits, nreq, lo=4, hi=16):
    """Mixed requests: 50% gets (half present, half absent), 40% inserts (some
    counted), 10% deletes of inserted keys; log-uniform sizes."""
    rng = np.random.default_rng(seed)
    ins = synth.splitmix64(seed + 1, 1 << (nbits - 1))
    absent = synth.splitmix64(seed + 2, 1 << hi)
    reqs, used, dcur = [], 0, 0
    for _ in range(nreq):
        n = int(2 ** rng.uniform(lo, hi))
        u = rng.random()
        if u < 0.5:
            pres = ins[: max(1, used)]
            k = np.concatenate([pres[rng.integers(0, pres.size, n // 2)], absent[: n - n // 2]])
            reqs.append((GET, k))
        elif u < 0.9:
            n = min(n, ins.size - used)
            if n == 0:
                continue
            k = ins[used:used + n]
            used += n
            op = REDUCE if rng.random() < 0.3 else INSERT
            if op == REDUCE:
                k = np.concatenate([k, k[: n // 3]])
            reqs.append((op, k))
        else:
            n = min(n, used - dcur)
            if n == 0:
                continue
            reqs.append((DELETE, ins[dcur:dcur + n]))
            dcur += n
    return reqs


def _sequential(gq, nbits, reqs):
    out = []
    with gq.QF(nbits) as qf:
        for op, k in reqs:
            if op == GET:
                out.append(gpu_get(qf, k))
            elif op == INSERT:
                qf.bulk_insert(dev(k))
            elif op == REDUCE:
                qf.bulk_insert_reduce(dev(k))
            else:
                qf.bulk_delete(dev(k))
        return out, qf.export()


@pytest.mark.parametrize("staging", [0, 1 << 20])
def test_mix_equals_one_by_one(gq, staging):
    nbits = 20
    reqs = _stream(7, nbits, 120)
    want, want_dump = _sequential(gq, nbits, reqs)
    with gq.QF(nbits) as qf:
        with gq.Server(qf, staging) as srv:
            keys = [np.ascontiguousarray(k) for _, k in reqs]
            outs = [np.zeros(k.size, dtype=np.uint64) if op == GET else None for (op, _), k in zip(reqs, keys)]
            tickets = [srv.submit(op, k, o) for (op, _), k, o in zip(reqs, keys, outs)]
            lats = [srv.wait(t) for t in tickets]
            st = srv.stats()
        got_dump = qf.export()
    got = [o for o in outs if o is not None]
    assert len(got) == len(want)
    for i, (a, b) in enumerate(zip(got, want)):
        assert np.array_equal(a, b), i
    assert np.array_equal(got_dump, want_dump), first_diff(got_dump, want_dump)
    assert st["requests"] == len(reqs) and min(lats) >= 0
    assert st["launches"] < len(reqs)  # consecutive requests of one kind were coalesced
    assert st["peak_staging_bytes"] <= st["staging_bytes"]


def test_device_buffers_and_split_requests(gq):
    import torch

    nbits = 22
    keys = synth.splitmix64(3, 1 << 20)
    with gq.QF(nbits) as qf:
        with gq.Server(qf, 1 << 20) as srv:  # 1 MiB ring: a 2^20-key request is cut in parts
            kd = dev(keys)
            t1 = srv.submit(INSERT, kd)
            out = torch.zeros(keys.size, dtype=torch.int64, device="cuda")
            t2 = srv.submit(GET, kd, out)
            srv.wait(t1)
            srv.wait(t2)
            srv.drain()
        o = oracle.Oracle(nbits)
        o.bulk_insert(keys)
        # keys equal modulo 2^(nbits+8) share a counter: compare with the oracle
        assert np.array_equal(host(out), o.bulk_get(keys))
        a, b = o.dump(), qf.export()
        assert np.array_equal(a, b), first_diff(a, b)


def test_concurrent_submitters(gq):
    nbits = 20
    parts = [synth.splitmix64(10 + i, 30000) for i in range(6)]
    with gq.QF(nbits) as qf:
        with gq.Server(qf, 4 << 20) as srv:
            def client(k):
                for c in np.array_split(k, 7):
                    srv.wait(srv.submit(INSERT, np.ascontiguousarray(c)))
            th = [threading.Thread(target=client, args=(p,)) for p in parts]
            for t in th:
                t.start()
            for t in th:
                t.join()
            srv.drain()
        got = qf.export()
    o = oracle.Oracle(nbits)
    o.bulk_insert(np.concatenate(parts))
    assert np.array_equal(got, o.dump())


def test_bad_requests(gq):
    with gq.QF(10) as qf:
        with gq.Server(qf, 1 << 20) as srv:
            with pytest.raises(RuntimeError):
                srv.submit(9, np.zeros(4, dtype=np.uint64))
            with pytest.raises(RuntimeError):
                srv.submit(GET, np.zeros(4, dtype=np.uint64), None)
            t = srv.submit(INSERT, np.zeros(0, dtype=np.uint64))
            assert srv.poll(t) == 1
            assert srv.poll(12345) == -1
