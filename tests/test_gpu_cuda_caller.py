"""A CUDA program that calls the device point API from its own kernels,
compiled and linked the way the reference's callers are (-rdc=true against
the relocatable device library, tests/cuda_caller.cu), builds the same
filter as the oracle's bulk insert of the same keys, word for word, and its
point_query counts match the oracle's counts."""
import os
import subprocess

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def caller(tmp_path_factory):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from cqf_gb300 import build

    build.build()
    nvcc = build.nvcc()
    exe = str(tmp_path_factory.mktemp("caller") / "cuda_caller")
    lib = os.path.dirname(build.SO_PATH)
    cmd = [nvcc, "-rdc=true", *build.ARCH, "-std=c++17", "-O2", os.path.join(ROOT, "tests", "cuda_caller.cu"),
           "-I", os.path.join(ROOT, "include"), "-L", lib, "-lgqf_gb300_device", "-lgqf_gb300",
           "-Xlinker", "-rpath=" + lib, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


@pytest.mark.parametrize("nbits", [12, 16])
def test_cuda_caller_point_inserts_match_oracle(caller, tmp_path, nbits):
    n = int(0.85 * (1 << nbits))
    keys = np.unique(oracle.splitmix64(21, n))  # distinct keys: every insert is new
    kin, dump_out, counts_out = (str(tmp_path / x) for x in ("keys.bin", "dump.bin", "counts.bin"))
    keys.astype(np.uint64).tofile(kin)
    r = subprocess.run([caller, str(nbits), kin, dump_out, counts_out], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    o = oracle.Oracle(nbits)
    o.bulk_insert(keys)
    dump = np.fromfile(dump_out, dtype=np.uint8)
    assert np.array_equal(dump, o.dump())
    counts = np.fromfile(counts_out, dtype=np.uint64)
    assert np.array_equal(counts, o.bulk_get(keys))

