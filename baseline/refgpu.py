"""The reference's own CUDA build, driven on a GPU -- BENCH/TEST INFRASTRUCTURE.

baseline.build() compiles the reference's device code (src/gqf.cu +
src/hashutil.cu, unmodified) into baseline/_ref/gqf_ref_sm103a.cubin on the
host that has the reference tree, and records the byte layout of its structs
(baseline/_ref/refgpu_layout.json).  The reference's host code is x86-only, so
this module restates its host orchestration and launches its kernels through
the CUDA driver API:

  bulk_insert  (src/gqf.cu:3184-3232): device sync (its num_locks readback,
               :3193-3201), hash_all, sort, set_buffers_binary,
               set_buffer_lens, insert_from_buffers_hashed even then odd
  bulk_delete  (src/gqf.cu:3316-3363): the same with delete_from_buffers_hashed
  bulk_get     (src/gqf.cu:3397-3400): bulk_get_kernel, 512 threads per CTA
  bulk_insert_reduce (src/gqf.cu:3238-3313): hash_all, sort, reduce_by_key,
               set_buffers_binary / set_buffer_lens on the distinct hashes,
               then insert_from_buffers_thrust (:2806) even then odd -- the
               counted insert the reference function stops short of (it
               returns after set_buffer_lens without launching an insert)

thrust::sort is replaced by torch.sort (a device radix sort as well).  Like
the reference, insert and delete overwrite the key buffer with sorted hashes.
Device memory comes from torch; the filter is the reference's own packed
81-byte blocks.  Never imported by the product.
"""
from __future__ import annotations

import ctypes
import json
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN = os.path.join(HERE, "_ref", "gqf_ref_sm103a.cubin")  # baseline/_ref
LAYOUT = os.path.join(HERE, "_ref", "refgpu_layout.json")

KERNELS = {
    "hash_all": "_Z8hash_allP15quotient_filterPmS1_mh",
    "set_buffers_binary": "_Z18set_buffers_binaryP15quotient_filtermPmh",
    "set_buffer_lens": "_Z15set_buffer_lensP15quotient_filtermPm",
    "insert_hashed": "_Z26insert_from_buffers_hashedP15quotient_filterm",
    "delete_hashed": "_Z26delete_from_buffers_hashedP15quotient_filterm",
    "bulk_get": "_Z15bulk_get_kernelP15quotient_filterPmmS1_h",
    "insert_thrust": "_Z26insert_from_buffers_thrustP15quotient_filtermPmS1_",
}
CU_LIMIT_STACK_SIZE = 0x00


def available() -> bool:
    return os.path.exists(CUBIN) and os.path.exists(LAYOUT)


class _Driver:
    def __init__(self):
        self.cu = ctypes.CDLL("libcuda.so.1")
        self.cu.cuModuleLoad.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_char_p]
        self.cu.cuModuleGetFunction.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p, ctypes.c_char_p]
        self.cu.cuLaunchKernel.argtypes = [ctypes.c_void_p] + [ctypes.c_uint] * 6 + [
            ctypes.c_uint, ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p]
        self.cu.cuModuleUnload.argtypes = [ctypes.c_void_p]
        self.cu.cuCtxSetLimit.argtypes = [ctypes.c_int, ctypes.c_size_t]

    def check(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"{what}: CUDA driver error {rc}")


_MODULE = {}  # the driver library, the loaded cubin and its kernels, once per process


def _driver():
    if "driver" not in _MODULE:
        _MODULE["driver"] = _Driver()
    return _MODULE["driver"]


def _module(d):
    if "mod" not in _MODULE:
        # per-thread stack of this process's context: the counted insert's
        # frames (1120 bytes, all static) fit with a wide margin
        d.check(d.cu.cuCtxSetLimit(CU_LIMIT_STACK_SIZE, 8192), "cuCtxSetLimit")
        mod = ctypes.c_void_p()
        d.check(d.cu.cuModuleLoad(ctypes.byref(mod), CUBIN.encode()), "cuModuleLoad")
        fn = {}
        for k, name in KERNELS.items():
            f = ctypes.c_void_p()
            d.check(d.cu.cuModuleGetFunction(ctypes.byref(f), mod, name.encode()), name)
            fn[k] = f
        _MODULE["mod"], _MODULE["fn"] = mod, fn
    return _MODULE["fn"]


class RefGPU:
    """One filter of the reference's CUDA build (2^nbits slots).  The cubin
    is loaded once per process and kept; a filter costs only its device
    buffers, as a qf_malloc_device does."""

    def __init__(self, nbits: int):
        import torch

        if not available():
            raise FileNotFoundError(CUBIN)
        self.torch = torch
        torch.cuda.init()
        torch.zeros(1, device="cuda")  # primary context current on this thread
        self.d = _driver()
        with open(LAYOUT) as fh:
            self.lay = json.load(fh)
        self.fn = _module(self.d)
        # qf_init sizing (src/gqf.cu:1939-1996) for qf_malloc_device's parameters
        self.nbits = nbits
        self.nslots = 1 << nbits
        self.xnslots = self.nslots + int(10 * math.sqrt(self.nslots))
        self.nblocks = (self.xnslots + 63) // 64
        self.num_locks = self.xnslots // 8192 + 2
        L = self.lay
        dev = lambda nbytes: torch.zeros((max(1, nbytes) + 7) // 8, dtype=torch.int64, device="cuda")
        self.blocks = dev(self.nblocks * L["sizeof_qfblock"])
        meta = np.zeros(15, dtype=np.uint64)
        meta[0] = 1018874902021329732  # MAGIC_NUMBER
        meta[1] = 1                    # QF_HASH_INVERTIBLE, reserved 0
        meta[2] = self.nblocks * L["sizeof_qfblock"]
        meta[4], meta[5], meta[6] = self.nslots, self.xnslots, nbits + 8
        meta[8], meta[9] = 8, 8        # key_remainder_bits, bits_per_slot
        meta[10], meta[11] = self.nslots << 8, self.nblocks
        self.meta = torch.from_numpy(meta.view(np.int64)).cuda()
        self.locks = dev(2)
        self.buffers = dev(2 * self.num_locks * 8)
        self.buffer_sizes = dev(2 * self.num_locks * 8)
        rt = np.zeros(L["sizeof_qfruntime"] // 8, dtype=np.uint64)
        rt[L["qfruntime_num_locks"] // 8] = self.num_locks
        rt[L["qfruntime_locks"] // 8] = self.locks.data_ptr()
        rt[L["qfruntime_buffers"] // 8] = self.buffers.data_ptr()
        rt[L["qfruntime_buffer_sizes"] // 8] = self.buffer_sizes.data_ptr()
        self.runtime = torch.from_numpy(rt.view(np.int64)).cuda()
        q = np.zeros(L["sizeof_QF"] // 8, dtype=np.uint64)
        q[L["QF_runtimedata"] // 8] = self.runtime.data_ptr()
        q[L["QF_metadata"] // 8] = self.meta.data_ptr()
        q[L["QF_blocks"] // 8] = self.blocks.data_ptr()
        self.qf = torch.from_numpy(q.view(np.int64)).cuda()
        torch.cuda.synchronize()

    def close(self):
        """Releases the filter's buffers (after its queued work)."""
        if getattr(self, "blocks", None) is not None:
            self.torch.cuda.synchronize()
            self.blocks = self.meta = self.locks = self.buffers = self.buffer_sizes = None
            self.runtime = self.qf = None

    def _launch(self, name, grid, block, *args):
        holders = []
        for a in args:
            if isinstance(a, tuple):  # (ctype, value)
                holders.append(a[0](a[1]))
            else:
                holders.append(ctypes.c_uint64(a))
        params = (ctypes.c_void_p * len(holders))(*[ctypes.cast(ctypes.byref(h), ctypes.c_void_p) for h in holders])
        stream = self.torch.cuda.current_stream().cuda_stream
        rc = self.d.cu.cuLaunchKernel(self.fn[name], int(grid), 1, 1, int(block), 1, 1, 0,
                                      ctypes.c_void_p(stream), params, None)
        self.d.check(rc, name)

    def _prelude(self, keys, n, flags):
        # the reference reads num_locks back from the device and synchronises
        # on every bulk call (src/gqf.cu:3193-3201)
        self.torch.cuda.synchronize()
        qf = self.qf.data_ptr()
        kp = keys.data_ptr()
        self._launch("hash_all", (n - 1) // 32 + 1, 32, qf, kp, kp, n, (ctypes.c_uint8, flags))
        s, _ = self.torch.sort(keys[:n])
        keys[:n].copy_(s)
        g = (self.num_locks - 1) // 32 + 1
        self._launch("set_buffers_binary", g, 32, qf, n, kp, (ctypes.c_uint8, flags))
        self._launch("set_buffer_lens", g, 32, qf, n, kp)
        return qf, g

    def bulk_insert(self, keys, n=None, flags=0):
        """keys: device int64 tensor, overwritten with sorted hashes."""
        n = keys.numel() if n is None else n
        if n == 0:
            return
        qf, g = self._prelude(keys, n, flags)
        self._launch("insert_hashed", g, 32, qf, 0)
        self._launch("insert_hashed", g, 32, qf, 1)

    def bulk_insert_reduce(self, keys, n=None, flags=0):
        """keys: device int64 tensor, overwritten with sorted hashes."""
        n = keys.numel() if n is None else n
        if n == 0:
            return
        self.torch.cuda.synchronize()
        qf = self.qf.data_ptr()
        kp = keys.data_ptr()
        self._launch("hash_all", (n - 1) // 32 + 1, 32, qf, kp, kp, n, (ctypes.c_uint8, flags))
        s, _ = self.torch.sort(keys[:n])
        keys[:n].copy_(s)
        uk, cnt = self.torch.unique_consecutive(keys[:n], return_counts=True)  # reduce_by_key
        uk = uk.contiguous()
        cnt = cnt.to(self.torch.int64).contiguous()
        u = uk.numel()
        g = (self.num_locks - 1) // 32 + 1
        self._launch("set_buffers_binary", g, 32, qf, u, uk.data_ptr(), (ctypes.c_uint8, flags))
        self._launch("set_buffer_lens", g, 32, qf, u, uk.data_ptr())
        self._launch("insert_thrust", g, 32, qf, 0, uk.data_ptr(), cnt.data_ptr())
        self._launch("insert_thrust", g, 32, qf, 1, uk.data_ptr(), cnt.data_ptr())
        self._hold = (uk, cnt)  # alive until the launches complete

    def bulk_delete(self, keys, n=None, flags=0):
        n = keys.numel() if n is None else n
        if n == 0:
            return
        qf, g = self._prelude(keys, n, flags)
        self._launch("delete_hashed", g, 32, qf, 0)
        self._launch("delete_hashed", g, 32, qf, 1)

    def bulk_get(self, vals, returns, n=None):
        n = vals.numel() if n is None else n
        if n == 0:
            return
        self._launch("bulk_get", (n - 1) // 512 + 1, 512, self.qf.data_ptr(), vals.data_ptr(), n,
                     returns.data_ptr(), (ctypes.c_uint8, 1))

    def dump(self) -> np.ndarray:
        self.torch.cuda.synchronize()
        meta = self.meta.cpu().numpy().view(np.uint8)
        blk = self.blocks.cpu().numpy().view(np.uint8)[: self.nblocks * self.lay["sizeof_qfblock"]]
        return np.concatenate([meta, blk])
