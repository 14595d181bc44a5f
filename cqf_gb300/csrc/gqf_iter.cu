// Enumeration of a filter's (hash, count) pairs, and the kernels built on it
// (merge, intersection, inner product).
//
// The reference walks its filters with a host iterator, one counter at a
// time (qf_iterator_from_position / qfi_get_hash / qfi_next,
// src/gqf.cu:3700-3893), and builds qf_merge, qf_multi_merge, qf_intersect
// and qf_inner_product on it (:3896-4080), all on the host.  Here every
// 64-slot block is decoded by its own thread: the runs of the block's
// occupied quotients start at max(q, end of the previous run + 1), the first
// one at or after 64 b + offset(b) (exact offsets), and each run is a
// sequence of counters ending at a runend.  A count pass and a write pass
// around a scan give the pairs in increasing hash order, the iterator's
// order.
#include "gqf_kernels.cuh"
#include "gqf_probe.cuh"

namespace gqf {
namespace {

// Decodes the runs of block b's quotients, calling emit(hash, count) in
// hash order; returns the number of pairs.
template <class F>
__device__ __forceinline__ uint32_t decode_block(const Block* __restrict__ B, uint64_t nblocks, uint64_t b,
                                                 F&& emit) {
  const uint64_t occ = __ldg(&B[b].occupieds);
  if (!occ) return 0;
  const uint64_t lim = 64 * nblocks;
  auto get = [&](uint64_t i) -> uint64_t { return i < lim ? __ldg(&B[i >> 6].slots[i & 63]) : 0; };
  auto end = [&](uint64_t i) -> int { return i < lim ? (int)((__ldg(&B[i >> 6].runends) >> (i & 63)) & 1ULL) : 1; };
  uint64_t next = 64 * b + __ldg(&B[b].offset);  // first slot after the earlier quotients' runs
  uint32_t n = 0;
  for (uint64_t m = occ; m; m &= m - 1) {
    const uint64_t q = 64 * b + (uint64_t)(__ffsll((long long)m) - 1);
    uint64_t s = next > q ? next : q;
    for (;;) {
      if (s >= lim) return n;  // a corrupt table: stop at its end
      uint32_t rem;
      uint64_t cnt;
      const uint64_t e = decode_counter(get, end, s, &rem, &cnt, lim);
      emit((q << 8) | rem, cnt, n);
      n++;
      if (end(e) || e + 1 >= lim) {
        next = e + 1;
        break;
      }
      s = e + 1;
    }
  }
  return n;
}

__global__ void __launch_bounds__(256) k_enum_count(Geom g, uint32_t* __restrict__ per_block) {
  const uint64_t b = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (b >= g.nblocks) return;
  per_block[b] = decode_block(g.blocks, g.nblocks, b, [](uint64_t, uint64_t, uint32_t) {});
}

// as_keys: report keys (the inverse hash, as qfi_get_key does) instead of
// hashes.  counts32: counts as uint32 (for the counted insert), flagging any
// above 2^32 - 1 in *overflow.
__global__ void __launch_bounds__(256) k_enum_write(Geom g, const uint32_t* __restrict__ start, int as_keys,
                                                    uint64_t* __restrict__ out_h, uint64_t* __restrict__ out_c,
                                                    uint32_t* __restrict__ out_c32, uint32_t* overflow) {
  const uint64_t b = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  if (b >= g.nblocks) return;
  const uint64_t at = start[b];
  decode_block(g.blocks, g.nblocks, b, [&](uint64_t h, uint64_t c, uint32_t k) {
    out_h[at + k] = as_keys ? hash64i(h, g.mask) : h;
    if (out_c) out_c[at + k] = c;
    if (out_c32) {
      if (c > 0xFFFFFFFFull) atomicOr(overflow, 1u);
      out_c32[at + k] = (uint32_t)c;
    }
  });
}

// Probes `mem` for each pair: inner product (acc += c * count_mem), or
// intersection (the pairs found in `mem` appended to out_h / out_c32, in no
// particular order: a counted insert does not depend on it).
__global__ void __launch_bounds__(256) k_pair_probe(Geom mem, const uint64_t* __restrict__ h,
                                                    const uint64_t* __restrict__ c, uint64_t n,
                                                    unsigned long long* acc, uint64_t* __restrict__ out_h,
                                                    uint32_t* __restrict__ out_c32, unsigned long long* n_out,
                                                    uint32_t* overflow) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t nr = (n + 31) & ~31ULL;
  const unsigned lane = threadIdx.x & 31;
  unsigned long long local = 0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nr; i += stride) {
    uint64_t x = 0, m = 0, ci = 0;
    if (i < n) {
      x = h[i];
      ci = c[i];
      m = x < mem.range ? probe(mem.blocks, mem.nblocks, x) : 0;
    }
    if (acc) local += ci * m;
    if (out_h) {
      const unsigned keep = __ballot_sync(0xffffffffu, m > 0);
      unsigned long long base = 0;
      if (lane == 0 && keep) base = atomicAdd(n_out, (unsigned long long)__popc(keep));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (m > 0) {
        const unsigned long long at = base + __popc(keep & ((1u << lane) - 1u));
        out_h[at] = x;
        if (ci > 0xFFFFFFFFull) atomicOr(overflow, 1u);
        out_c32[at] = (uint32_t)ci;
      }
    }
  }
  if (acc) {
    for (int o = 16; o; o >>= 1) local += __shfl_down_sync(0xffffffffu, local, o);
    if (lane == 0 && local) atomicAdd(acc, local);
  }
}

}  // namespace

cudaError_t launch_enum_count(const Geom& g, uint32_t* per_block, cudaStream_t st) {
  k_enum_count<<<(unsigned)((g.nblocks + 255) / 256), 256, 0, st>>>(g, per_block);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_enum_write(const Geom& g, const uint32_t* start, int as_keys, uint64_t* out_h, uint64_t* out_c,
                              uint32_t* out_c32, uint32_t* overflow, cudaStream_t st) {
  k_enum_write<<<(unsigned)((g.nblocks + 255) / 256), 256, 0, st>>>(g, start, as_keys, out_h, out_c, out_c32,
                                                                     overflow);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_pair_probe(const Geom& mem, const uint64_t* h, const uint64_t* c, uint64_t n,
                              unsigned long long* acc, uint64_t* out_h, uint32_t* out_c32,
                              unsigned long long* n_out, uint32_t* overflow, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  const uint64_t want = (n + 255) / 256, cap = (uint64_t)sm_count() * 16;
  k_pair_probe<<<(unsigned)(want < cap ? want : cap), 256, 0, st>>>(mem, h, c, n, acc, out_h, out_c32, n_out,
                                                                    overflow);
  count_launch();
  return cudaGetLastError();
}

}  // namespace gqf
