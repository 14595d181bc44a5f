// Hash + partition of a key batch by region (a radix partition on the top
// quotient bits).  Replaces the reference's hash_all + thrust::sort +
// set_buffers_binary + set_buffer_lens (src/gqf.cu:2615-2750, :3206-3215):
// only the region of each hash matters for the even/odd schedule, and the
// rebuild kernel sorts each region's keys in shared memory.
//
// Pass 1 counts keys per region, pass 2 scans the counts, pass 3 scatters
// each key's region-local hash (low 8 + log_region bits, a uint32) into its
// region's bucket.  Same-region keys inside a warp share one atomic
// (match.any), which keeps skewed batches from serialising on hot regions.
#include "gqf_kernels.cuh"

namespace gqf {
namespace {

__device__ __forceinline__ bool hash_key(const Geom& g, const uint64_t* keys, uint64_t i, uint64_t n,
                                         int key_is_hash, uint32_t* status, uint64_t* h) {
  if (i >= n) return false;
  uint64_t k = keys[i];
  if (key_is_hash) {
    if (k >= g.range) {
      if (status) atomicOr(status, kStBadKey);
      return false;
    }
    *h = k;
  } else {
    *h = hash64(k, g.mask);
  }
  return true;
}

// n_dev, when given, holds the key count instead of n (a count produced on
// the device by the duplicate-merging pass).
__global__ void __launch_bounds__(256) k_part_count(Geom g, const uint64_t* __restrict__ keys,
                                                    uint64_t n, const unsigned long long* n_dev,
                                                    int key_is_hash, int shift,
                                                    uint32_t* __restrict__ region_count,
                                                    uint32_t* status) {
  if (n_dev) n = min(n, (uint64_t)*n_dev);
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t nr = (n + 31) & ~31ULL;
  const unsigned lane = threadIdx.x & 31;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nr; i += stride) {
    uint64_t h = 0;
    bool ok = hash_key(g, keys, i, n, key_is_hash, status, &h);
    uint32_t r = ok ? (uint32_t)(h >> shift) : 0xFFFFFFFFu;
    unsigned peers = __match_any_sync(0xffffffffu, r);
    if (ok && lane == (unsigned)(__ffs(peers) - 1)) atomicAdd(&region_count[r], (uint32_t)__popc(peers));
  }
}

// Exclusive scan of the nregions counts (also resetting the cursors), in
// chunks of kScanChunk regions: one CTA per chunk sums it, then one CTA per
// chunk adds the sums of the chunks before it and scans its own.  Loads and
// stores are coalesced: thread t of a CTA owns counts 4t..4t+3 of the chunk.
constexpr int kScanThreads = 1024;
constexpr int kScanChunk = 4 * kScanThreads;

__device__ __forceinline__ uint32_t block_sum_excl(uint32_t v, uint32_t* warp_sum, uint32_t* total) {
  const unsigned lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= (unsigned)o) x += t;
  }
  if (lane == 31) warp_sum[wid] = x;
  __syncthreads();
  if (wid == 0) {
    uint32_t w = lane < (blockDim.x >> 5) ? warp_sum[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t t = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= (unsigned)o) w += t;
    }
    warp_sum[lane] = w;
  }
  __syncthreads();
  const uint32_t r = x - v + (wid ? warp_sum[wid - 1] : 0);
  *total = warp_sum[(blockDim.x >> 5) - 1];
  __syncthreads();
  return r;
}

__device__ __forceinline__ void load4(const uint32_t* a, uint32_t n, uint32_t i, uint32_t* v) {
  for (int k = 0; k < 4; k++) v[k] = i + k < n ? a[i + k] : 0u;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_sums(const uint32_t* __restrict__ region_count,
                                                            uint32_t nregions, uint32_t* __restrict__ sums) {
  __shared__ uint32_t warp_sum[32];
  uint32_t v[4];
  load4(region_count, nregions, blockIdx.x * kScanChunk + 4 * threadIdx.x, v);
  uint32_t tot;
  block_sum_excl(v[0] + v[1] + v[2] + v[3], warp_sum, &tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_apply(const uint32_t* __restrict__ region_count,
                                                             uint32_t nregions, const uint32_t* __restrict__ sums,
                                                             uint32_t* __restrict__ region_start,
                                                             uint32_t* __restrict__ cursor) {
  __shared__ uint32_t warp_sum[32];
  uint32_t before = 0, dummy;  // sum of the chunks before this one
  for (uint32_t c = threadIdx.x; c < blockIdx.x; c += blockDim.x) before += sums[c];
  {
    uint32_t part = before;
    for (int o = 16; o; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = part;
    __syncthreads();
    before = 0;
    for (unsigned w = 0; w < (blockDim.x >> 5); w++) before += warp_sum[w];
    __syncthreads();
  }
  const uint32_t i = blockIdx.x * kScanChunk + 4 * threadIdx.x;
  uint32_t v[4];
  load4(region_count, nregions, i, v);
  uint32_t excl = before + block_sum_excl(v[0] + v[1] + v[2] + v[3], warp_sum, &dummy);
  for (int k = 0; k < 4; k++) {
    if (i + k < nregions) {
      region_start[i + k] = excl;
      cursor[i + k] = excl;
    }
    excl += v[k];
    if (i + k + 1 == nregions) region_start[nregions] = excl;
  }
}

__global__ void __launch_bounds__(256) k_part_scatter(Geom g, const uint64_t* __restrict__ keys,
                                                      uint64_t n, const unsigned long long* n_dev,
                                                      const uint32_t* __restrict__ counts,
                                                      int key_is_hash, int shift,
                                                      uint32_t* __restrict__ cursor,
                                                      uint32_t* __restrict__ out,
                                                      uint32_t* __restrict__ out_counts) {
  if (n_dev) n = min(n, (uint64_t)*n_dev);
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t nr = (n + 31) & ~31ULL;
  const unsigned lane = threadIdx.x & 31;
  const uint64_t local_mask = (1ULL << shift) - 1ULL;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nr; i += stride) {
    uint64_t h = 0;
    bool ok = hash_key(g, keys, i, n, key_is_hash, nullptr, &h);
    uint32_t r = ok ? (uint32_t)(h >> shift) : 0xFFFFFFFFu;
    unsigned peers = __match_any_sync(0xffffffffu, r);
    unsigned leader = __ffs(peers) - 1;
    uint32_t base = 0;
    if (ok && lane == leader) base = atomicAdd(&cursor[r], (uint32_t)__popc(peers));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (ok) {
      const uint32_t at = base + __popc(peers & ((1u << lane) - 1u));
      out[at] = (uint32_t)(h & local_mask);
      if (counts) out_counts[at] = counts[i];
    }
  }
}

int grid_for(uint64_t n) {
  const int sms = sm_count();
  uint64_t want = (n + 255) / 256;
  uint64_t cap = (uint64_t)sms * 16;
  if (want > cap) want = cap;
  return (int)(want ? want : 1);
}

}  // namespace

cudaError_t launch_region_scan(const Partition& p, cudaStream_t st) {
  // the chunk sums use the deferred list as scratch: the rebuild resets it
  const uint32_t chunks = (p.nregions + kScanChunk - 1) / kScanChunk;
  k_scan_sums<<<chunks, kScanThreads, 0, st>>>(p.region_count, p.nregions, p.deferred);
  k_scan_apply<<<chunks, kScanThreads, 0, st>>>(p.region_count, p.nregions, p.deferred, p.region_start, p.cursor);
  count_launch(2);
  return cudaGetLastError();
}

cudaError_t launch_partition(const Geom& g, const Partition& p, const uint64_t* keys, uint64_t n,
                             int key_is_hash, uint32_t* status, cudaStream_t st) {
  return launch_partition_counted(g, p, keys, nullptr, n, nullptr, key_is_hash, status, st);
}

cudaError_t launch_partition_counted(const Geom& g, const Partition& p, const uint64_t* keys,
                                     const uint32_t* counts, uint64_t n, const unsigned long long* n_dev,
                                     int key_is_hash, uint32_t* status, cudaStream_t st) {
  const int shift = 8 + p.log_region;
  cudaError_t e = cudaMemsetAsync(p.region_count, 0, (p.nregions + 1) * sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  if (n) {
    k_part_count<<<grid_for(n), 256, 0, st>>>(g, keys, n, n_dev, key_is_hash, shift, p.region_count, status);
    count_launch();
  }
  e = launch_region_scan(p, st);
  if (e != cudaSuccess) return e;
  if (n) {
    k_part_scatter<<<grid_for(n), 256, 0, st>>>(g, keys, n, n_dev, counts, key_is_hash, shift, p.cursor,
                                                p.keys, p.counts);
    count_launch();
  }
  return cudaGetLastError();
}

}  // namespace gqf
