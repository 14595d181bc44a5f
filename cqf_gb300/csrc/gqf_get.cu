// bulk_get: one probe per key, HBM-bound random access.
//
// Restates qf_count_key_value (src/gqf.cu:3479-3517) as called by
// bulk_get_kernel (src/gqf.cu:3386): hash the key, test the occupied bit of
// its home quotient, locate the start of its run with rank over the home
// block's occupieds and select over runends (the reference's run_end,
// src/gqf.cu:632), then walk the run's counters.
//
// On this layout the whole run-start computation needs only the home block's
// 32-byte header (occupieds, runends, exact offset) in the common case: the
// run start of quotient q is max(q, 64b + offset) when no earlier quotient of
// block b is occupied, else one past the rank-th runend at or after
// 64b + offset.  Loads go through the read-only path (ld.global.nc).
#include "gqf_kernels.cuh"

namespace gqf {
namespace {

__device__ __forceinline__ uint64_t ld_u64(const unsigned long long* p) { return __ldg(p); }

// Walks one run from `start`; returns the count for `rem` or 0.  The slots
// come through a 16-byte register window and the runends through a one-word
// register cache seeded with the home block's word, so a probe costs one
// header load and usually one slot load, whatever the L1 hit rate.
__device__ __forceinline__ uint64_t scan_run(const Block* __restrict__ B, uint64_t nblocks,
                                             uint64_t start, uint32_t rem, uint64_t home,
                                             uint64_t home_runends) {
  uint64_t cb = home;
  uint64_t cw = home_runends;
  uint64_t ci = ~0ULL;  // 16-slot chunk index held in `chunk`
  uint4 chunk = make_uint4(0, 0, 0, 0);
  auto is_end = [&](uint64_t i) -> int {
    uint64_t bi = i >> 6;
    if (bi != cb) {
      cb = bi;
      cw = bi < nblocks ? ld_u64(&B[bi].runends) : 0;
    }
    return (int)((cw >> (i & 63)) & 1ULL);
  };
  auto get = [&](uint64_t i) -> uint64_t {
    uint64_t c = i >> 4;
    if (c != ci) {
      ci = c;
      uint64_t bi = i >> 6;
      chunk = bi < nblocks ? __ldg(reinterpret_cast<const uint4*>(&B[bi].slots[(i & 63) & ~15ULL]))
                           : make_uint4(0, 0, 0, 0);
    }
    const uint32_t k = (uint32_t)(i & 15);
    const uint32_t w = k < 8 ? (k < 4 ? chunk.x : chunk.y) : (k < 12 ? chunk.z : chunk.w);
    return (w >> (8 * (k & 3))) & 0xFFu;
  };
  uint32_t cr;
  uint64_t cc, ce;
  const uint64_t lim = 64 * nblocks;
  while (start < lim) {
    ce = decode_counter(get, is_end, start, &cr, &cc, lim);
    if (cr == rem) return cc;
    if (is_end(ce)) return 0;
    start = ce + 1;
  }
  return 0;
}

__device__ __forceinline__ uint64_t probe(const Block* __restrict__ B, uint64_t nblocks, uint64_t h) {
  const uint64_t q = h >> 8;
  const uint32_t rem = (uint32_t)(h & 255);
  const uint64_t b = q >> 6;
  const int j = (int)(q & 63);
  const ulonglong2 hdr = __ldg(reinterpret_cast<const ulonglong2*>(&B[b]));
  const uint64_t occ = hdr.x;
  if (!((occ >> j) & 1ULL)) return 0;
  const uint64_t off = __ldg(&B[b].offset);
  const int rank = __popcll(occ & ((1ULL << j) - 1ULL));
  uint64_t start;
  if (rank == 0) {
    start = 64 * b + off;
    if (start < q) start = q;
  } else {
    uint64_t pos = 64 * b + off;
    uint64_t rb = pos >> 6;
    uint64_t w = (rb == b ? hdr.y : ld_u64(&B[rb].runends)) & (~0ULL << (pos & 63));
    int k = rank - 1;
    int c = __popcll(w);
    while (k >= c) {
      k -= c;
      rb++;
      if (rb >= nblocks) return 0;
      w = ld_u64(&B[rb].runends);
      c = __popcll(w);
    }
    uint64_t e = 64 * rb + (uint64_t)select64(w, k);
    start = e + 1 > q ? e + 1 : q;
  }
  return scan_run(B, nblocks, start, rem, b, hdr.y);
}

__global__ void __launch_bounds__(256) k_bulk_get(Geom g, const uint64_t* __restrict__ keys,
                                                  uint64_t n, uint64_t* __restrict__ out,
                                                  int key_is_hash) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    uint64_t k = __ldcs(keys + i);
    uint64_t h = key_is_hash ? k : hash64(k, g.mask);
    uint64_t c = (h < g.range) ? probe(g.blocks, g.nblocks, h) : 0;
    __stcs(out + i, c);
  }
}

__global__ void __launch_bounds__(256) k_bulk_get_misses(Geom g, const uint64_t* __restrict__ keys,
                                                         uint64_t n, unsigned long long* misses) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  unsigned int m = 0;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    uint64_t h = hash64(__ldcs(keys + i), g.mask);
    if (probe(g.blocks, g.nblocks, h) < 1) m++;
  }
  // warp then block reduction, one atomic per CTA
  for (int o = 16; o; o >>= 1) m += __shfl_down_sync(0xffffffffu, m, o);
  __shared__ unsigned int part[8];
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long s = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += part[w];
    if (s) atomicAdd(misses, s);
  }
}

int grid_for(uint64_t n) {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 152;
  }
  uint64_t want = (n + 255) / 256;
  uint64_t cap = (uint64_t)sms * 32;
  if (want > cap) want = cap;
  return (int)(want ? want : 1);
}

}  // namespace

cudaError_t launch_bulk_get(const Geom& g, const uint64_t* keys, uint64_t n, uint64_t* out,
                            int key_is_hash, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_bulk_get<<<grid_for(n), 256, 0, st>>>(g, keys, n, out, key_is_hash);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_bulk_get_misses(const Geom& g, const uint64_t* keys, uint64_t n,
                                   unsigned long long* misses, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  k_bulk_get_misses<<<grid_for(n), 256, 0, st>>>(g, keys, n, misses);
  count_launch();
  return cudaGetLastError();
}

}  // namespace gqf
