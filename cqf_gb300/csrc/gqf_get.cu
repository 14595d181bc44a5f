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
#include "gqf_probe.cuh"

namespace gqf {
namespace {

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
  const int sms = sm_count();
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
