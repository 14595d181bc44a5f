"""Small helpers shared by the GPU tests (device buffers via torch)."""
import hashlib

import numpy as np


def dev(a):
    import torch

    a = np.ascontiguousarray(a, dtype=np.uint64)
    return torch.from_numpy(a.view(np.int64)).cuda()


def host(t) -> np.ndarray:
    return t.cpu().numpy().view(np.uint64)


def zeros_dev(n, dtype=None):
    import torch

    return torch.zeros(int(n), dtype=dtype or torch.int64, device="cuda")


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def gpu_get(qf, keys: np.ndarray) -> np.ndarray:
    import torch

    k = dev(keys)
    out = zeros_dev(len(keys))
    qf.bulk_get(k, out)
    torch.cuda.synchronize()
    return host(out)


def first_diff(a: np.ndarray, b: np.ndarray):
    """Human-readable location of the first differing byte of two dumps."""
    d = np.nonzero(np.asarray(a) != np.asarray(b))[0]
    if d.size == 0:
        return None
    i = int(d[0])
    if i < 120:
        return f"metadata byte {i}: {a[i]} vs {b[i]} ({d.size} bytes differ)"
    blk, off = divmod(i - 120, 81)
    field = "offset" if off == 0 else "occupieds" if off < 9 else "runends" if off < 17 else f"slot {off - 17}"
    return f"block {blk} {field}: {a[i]} vs {b[i]} ({d.size} bytes differ)"
