// Hash + partition of a key batch by region (a radix partition on the top
// quotient bits).  Replaces the reference's hash_all + thrust::sort +
// set_buffers_binary + set_buffer_lens (src/gqf.cu:2615-2750, :3206-3215):
// only the region of each hash matters for the even/odd schedule, and the
// rebuild kernel sorts each region's keys in shared memory.
//
// Small batches (single level): pass 1 counts keys per region, pass 2 scans
// the counts, pass 3 scatters each key's region-local hash (low 8 +
// log_region bits, a uint32) into its region's bucket.  Same-region keys
// inside a warp share one atomic (match.any), which keeps skewed batches from
// serialising on hot regions.  Each key costs two global atomics.
//
// Large batches (two levels, no global atomics): the regions form about
// sqrt(nregions) super-buckets of 2^s consecutive regions.  Each tile of
// kStageTile keys histograms its super-buckets in shared memory; one scan of
// the tile histograms (bucket-major) gives every (bucket, tile) its exact
// output offset, so the tiles scatter into a staging array with shared-memory
// atomics only, in runs of consecutive entries per bucket.  Then one CTA per
// super-bucket histograms, scans and scatters its own keys to their regions,
// again in shared memory.  A staged entry packs the region's low s bits above
// the region-local hash (8 + log_region + s <= 32 bits).
#include <algorithm>

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

// With len_dev, the scanned length is nb * (the tiles of *len_dev keys, at
// most `nregions` entries) instead of nregions: a batch whose size only the
// device knows.
__device__ __forceinline__ uint32_t scan_len(uint32_t nregions, const unsigned long long* len_dev, uint32_t nb,
                                             uint32_t tile) {
  if (!len_dev) return nregions;
  const uint64_t t = ((uint64_t)*len_dev + tile - 1) / tile;
  return (uint32_t)min((uint64_t)nregions, (uint64_t)nb * t);
}

__global__ void __launch_bounds__(kScanThreads) k_scan_sums(const uint32_t* __restrict__ region_count,
                                                            uint32_t nregions, uint32_t* __restrict__ sums,
                                                            const unsigned long long* len_dev = nullptr,
                                                            uint32_t nb = 0, uint32_t tile = 1) {
  __shared__ uint32_t warp_sum[32];
  nregions = scan_len(nregions, len_dev, nb, tile);
  uint32_t v[4];
  load4(region_count, nregions, blockIdx.x * kScanChunk + 4 * threadIdx.x, v);
  uint32_t tot;
  block_sum_excl(v[0] + v[1] + v[2] + v[3], warp_sum, &tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_apply(const uint32_t* __restrict__ region_count,
                                                             uint32_t nregions, const uint32_t* __restrict__ sums,
                                                             uint32_t* __restrict__ region_start,
                                                             uint32_t* __restrict__ cursor,
                                                             const unsigned long long* len_dev = nullptr,
                                                             uint32_t nb = 0, uint32_t tile = 1) {
  __shared__ uint32_t warp_sum[32];
  nregions = scan_len(nregions, len_dev, nb, tile);
  if ((uint64_t)blockIdx.x * kScanChunk > nregions) return;  // past the (device) length
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
      if (cursor) cursor[i + k] = excl;
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

// ------------------------------------------------- two-level partition

constexpr int kStageTile = 8192;       // keys per tile
constexpr int kStageThreads = 512;
constexpr int kBucketThreads = 256;
constexpr int kMaxBuckets = 4096;
constexpr uint64_t kStageMinKeys = 1ULL << 18;  // smaller batches: single level
constexpr uint32_t kStageMinRegions = 1u << 12;

struct StagePlan {
  int s;           // region bits resolved by the bucket pass
  uint32_t nb;     // super-buckets (nregions >> s)
  uint32_t ntiles;
};

int log2u(uint32_t v) {
  int l = 0;
  while ((1u << (l + 1)) <= v) l++;
  return l;
}

StagePlan stage_plan(uint64_t n, uint32_t nregions, int log_region) {
  StagePlan sp{};
  // about 1024 super-buckets: level one writes runs of a few dozen bytes per
  // bucket and tile, and level two has enough CTAs (of a few thousand keys
  // each at the usual batch sizes) to fill the GPU
  const int L = log2u(nregions);
  sp.s = std::min(std::max(2, L - 10), 24 - log_region);
  sp.nb = nregions >> sp.s;
  sp.ntiles = (uint32_t)((n + kStageTile - 1) / kStageTile);
  return sp;
}

// Tiles of a batch: ntiles for n keys, fewer when the device holds a smaller
// count (n_dev); the tile histograms are laid out for the tiles that exist.
__device__ __forceinline__ uint32_t dev_ntiles(uint64_t n, const unsigned long long* n_dev, uint32_t ntiles) {
  if (!n_dev) return ntiles;
  n = min(n, (uint64_t)*n_dev);
  return (uint32_t)min((uint64_t)ntiles, (n + kStageTile - 1) / kStageTile);
}

// A tile's keys, kStagePer per thread, all loads issued before any is used
// (latency, not bandwidth, bounds a pass that touches each key once).
constexpr int kStagePer = kStageTile / kStageThreads;
static_assert(kStageTile % kStageThreads == 0, "tiles split evenly");

__device__ __forceinline__ void load_tile(const uint64_t* __restrict__ keys, uint64_t beg, uint64_t end,
                                          uint64_t* k) {
#pragma unroll
  for (int j = 0; j < kStagePer; j++) {
    const uint64_t i = beg + threadIdx.x + (uint64_t)j * kStageThreads;
    k[j] = i < end ? __ldcs(keys + i) : 0;
  }
}

// The hash of a loaded key (as hash_key), false for keys past the end or bad.
__device__ __forceinline__ bool tile_hash(const Geom& g, uint64_t k, bool in, int key_is_hash, uint32_t* status,
                                          uint64_t* h) {
  if (!in) return false;
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

__global__ void __launch_bounds__(kStageThreads) k_stage_hist(Geom g, const uint64_t* __restrict__ keys, uint64_t n,
                                                              const unsigned long long* n_dev, int key_is_hash,
                                                              int shift, int s, uint32_t nb, uint32_t ntiles,
                                                              uint32_t* __restrict__ tiles, uint32_t* status) {
  __shared__ uint32_t hist[kMaxBuckets];
  ntiles = dev_ntiles(n, n_dev, ntiles);
  if (blockIdx.x >= ntiles) return;
  for (uint32_t b = threadIdx.x; b < nb; b += blockDim.x) hist[b] = 0;
  if (n_dev) n = min(n, (uint64_t)*n_dev);
  const uint64_t beg = (uint64_t)blockIdx.x * kStageTile, end = min(n, beg + kStageTile);
  uint64_t k[kStagePer];
  load_tile(keys, beg, end, k);
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kStagePer; j++) {
    uint64_t h;
    const bool in = beg + threadIdx.x + (uint64_t)j * kStageThreads < end;
    if (tile_hash(g, k[j], in, key_is_hash, status, &h)) atomicAdd(&hist[(uint32_t)(h >> shift) >> s], 1u);
  }
  __syncthreads();
  for (uint32_t b = threadIdx.x; b < nb; b += blockDim.x) tiles[(uint64_t)b * ntiles + blockIdx.x] = hist[b];
}

// Exclusive scan, in place, of n shared counters (n <= a few per thread);
// returns the total.  All threads of the block call it.
__device__ __forceinline__ uint32_t smem_scan(uint32_t* c, uint32_t n, uint32_t* warp_sum) {
  const uint32_t per = (n + blockDim.x - 1) / blockDim.x;
  const uint32_t a = threadIdx.x * per, z = min(n, a + per);
  uint32_t sum = 0;
  for (uint32_t i = a; i < z; i++) sum += c[i];
  uint32_t tot;
  uint32_t run = block_sum_excl(sum, warp_sum, &tot);
  for (uint32_t i = a; i < z; i++) {
    const uint32_t v = c[i];
    c[i] = run;
    run += v;
  }
  __syncthreads();
  return tot;
}

// Level one: each tile is sorted by super-bucket in shared memory, then
// written out in runs (consecutive threads, consecutive entries of one
// bucket) at the offsets the tile-histogram scan gave it.
size_t scatter_smem(uint32_t nb, bool counted) {
  return (size_t)2 * nb * 4 + (size_t)kStageTile * (4 + 2 + (counted ? 4 : 0));
}

__global__ void __launch_bounds__(kStageThreads) k_stage_scatter(Geom g, const uint64_t* __restrict__ keys,
                                                                 const uint32_t* __restrict__ counts, uint64_t n,
                                                                 const unsigned long long* n_dev, int key_is_hash,
                                                                 int shift, int s, uint32_t nb, uint32_t ntiles,
                                                                 const uint32_t* __restrict__ tiles,
                                                                 uint32_t* __restrict__ stage,
                                                                 uint32_t* __restrict__ stage_counts) {
  extern __shared__ uint32_t sm[];
  __shared__ uint32_t warp_sum[32];
  uint32_t* lcur = sm;             // nb: per-bucket cursor in the sorted tile
  uint32_t* goff = sm + nb;        // nb: output position of sorted entry e is goff[b] + e
  uint32_t* sent = sm + 2 * nb;    // kStageTile sorted entries
  uint32_t* scnt = sent + kStageTile;
  uint16_t* sbin = reinterpret_cast<uint16_t*>(scnt + (counts ? kStageTile : 0));
  ntiles = dev_ntiles(n, n_dev, ntiles);
  if (blockIdx.x >= ntiles) return;
  for (uint32_t b = threadIdx.x; b < nb; b += blockDim.x) lcur[b] = 0;
  if (n_dev) n = min(n, (uint64_t)*n_dev);
  const uint64_t beg = (uint64_t)blockIdx.x * kStageTile, end = min(n, beg + kStageTile);
  uint64_t k[kStagePer];
  load_tile(keys, beg, end, k);
  uint32_t cnt[kStagePer];
#pragma unroll
  for (int j = 0; j < kStagePer; j++) {
    const uint64_t i = beg + threadIdx.x + (uint64_t)j * kStageThreads;
    cnt[j] = (counts && i < end) ? __ldcs(counts + i) : 0u;
  }
  __syncthreads();
  const uint64_t local_mask = (1ULL << shift) - 1ULL;
  const uint32_t lo_mask = (1u << s) - 1u;
  uint32_t bkt[kStagePer], ent[kStagePer];
#pragma unroll
  for (int j = 0; j < kStagePer; j++) {
    uint64_t h;
    const uint64_t i = beg + threadIdx.x + (uint64_t)j * kStageThreads;
    bkt[j] = 0xFFFFFFFFu;
    if (!tile_hash(g, k[j], i < end, key_is_hash, nullptr, &h)) continue;
    const uint32_t r = (uint32_t)(h >> shift);
    bkt[j] = r >> s;
    ent[j] = ((r & lo_mask) << shift) | (uint32_t)(h & local_mask);
    atomicAdd(&lcur[bkt[j]], 1u);
  }
  __syncthreads();
  const uint32_t total = smem_scan(lcur, nb, warp_sum);
  for (uint32_t b = threadIdx.x; b < nb; b += blockDim.x) goff[b] = tiles[(uint64_t)b * ntiles + blockIdx.x] - lcur[b];
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kStagePer; j++) {
    if (bkt[j] == 0xFFFFFFFFu) continue;
    const uint32_t at = atomicAdd(&lcur[bkt[j]], 1u);
    sent[at] = ent[j];
    sbin[at] = (uint16_t)bkt[j];
    if (counts) scnt[at] = cnt[j];
  }
  __syncthreads();
  for (uint32_t e = threadIdx.x; e < total; e += blockDim.x) {
    const uint32_t at = goff[sbin[e]] + e;
    stage[at] = sent[e];
    if (counts) stage_counts[at] = scnt[e];
  }
}

// Level two: one CTA per super-bucket counts its 2^s regions (their counts
// and starts), then walks its entries in chunks of kBucketChunk, each sorted
// by region in shared memory and written out in runs at the regions'
// running cursors.
constexpr int kBucketChunk = 4096;
constexpr int kBucketPer = kBucketChunk / kBucketThreads;
static_assert(kBucketChunk % kBucketThreads == 0, "chunks split evenly");

size_t bucket_smem(int s, bool counted) {
  return (size_t)3 * (4u << s) + (size_t)kBucketChunk * (4 + 2 + (counted ? 4 : 0));
}

__global__ void __launch_bounds__(kBucketThreads) k_stage_bucket(Partition p, int shift, int s, uint32_t ntiles,
                                                                  uint64_t n, const unsigned long long* n_dev) {
  extern __shared__ uint32_t sm[];
  __shared__ uint32_t warp_sum[32];
  const uint32_t nb = p.nregions >> s, b = blockIdx.x;
  const uint32_t bins = 1u << s;
  uint32_t* hb = sm;                 // bins: each region's next position in p.keys
  uint32_t* lcur = sm + bins;        // bins: cursors in the sorted chunk
  uint32_t* lstart = sm + 2 * bins;  // bins: region starts in the sorted chunk
  uint32_t* sent = sm + 3 * bins;    // kBucketChunk sorted entries
  uint32_t* scnt = sent + kBucketChunk;
  uint16_t* sbin = reinterpret_cast<uint16_t*>(scnt + (p.counts ? kBucketChunk : 0));
  ntiles = dev_ntiles(n, n_dev, ntiles);
  const uint32_t bstart = ntiles ? p.tiles[(uint64_t)b * ntiles] : 0;
  const uint32_t bend = ntiles ? p.tiles[(uint64_t)(b + 1) * ntiles] : 0;  // the total after the last bucket
  for (uint32_t i = threadIdx.x; i < bins; i += blockDim.x) hb[i] = 0;
  __syncthreads();
  for (uint32_t i0 = bstart + threadIdx.x; i0 < bend; i0 += kBucketChunk) {
    uint32_t v[kBucketPer];
#pragma unroll
    for (int j = 0; j < kBucketPer; j++) {
      const uint32_t i = i0 + j * kBucketThreads;
      v[j] = i < bend ? __ldcg(p.stage + i) : 0;
    }
#pragma unroll
    for (int j = 0; j < kBucketPer; j++)
      if (i0 + j * kBucketThreads < bend) atomicAdd(&hb[v[j] >> shift], 1u);
  }
  __syncthreads();
  {
    const uint32_t per = (bins + blockDim.x - 1) / blockDim.x;
    const uint32_t a = threadIdx.x * per, z = min(bins, a + per);
    uint32_t sum = 0;
    for (uint32_t i = a; i < z; i++) sum += hb[i];
    uint32_t tot;
    uint32_t run = bstart + block_sum_excl(sum, warp_sum, &tot);
    for (uint32_t i = a; i < z; i++) {
      const uint32_t c = hb[i], r = (b << s) | i;
      p.region_count[r] = c;
      p.region_start[r] = run;
      hb[i] = run;
      run += c;
    }
  }
  if (b + 1 == nb && threadIdx.x == 0) p.region_start[p.nregions] = bend;
  const uint32_t local_mask = (uint32_t)((1ULL << shift) - 1ULL);
  for (uint32_t c0 = bstart; c0 < bend; c0 += kBucketChunk) {
    const uint32_t cn = min((uint32_t)kBucketChunk, bend - c0);
    for (uint32_t i = threadIdx.x; i < bins; i += blockDim.x) lcur[i] = 0;
    uint32_t v[kBucketPer], cc[kBucketPer];
#pragma unroll
    for (int j = 0; j < kBucketPer; j++) {
      const uint32_t e = threadIdx.x + j * kBucketThreads;
      v[j] = e < cn ? __ldcs(p.stage + c0 + e) : 0;
      cc[j] = (p.counts && e < cn) ? __ldcs(p.stage_counts + c0 + e) : 0;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kBucketPer; j++)
      if (threadIdx.x + j * kBucketThreads < cn) atomicAdd(&lcur[v[j] >> shift], 1u);
    __syncthreads();
    smem_scan(lcur, bins, warp_sum);
    for (uint32_t i = threadIdx.x; i < bins; i += blockDim.x) lstart[i] = lcur[i];
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kBucketPer; j++) {
      if (threadIdx.x + j * kBucketThreads >= cn) continue;
      const uint32_t r = v[j] >> shift;
      const uint32_t at = atomicAdd(&lcur[r], 1u);
      sent[at] = v[j] & local_mask;
      sbin[at] = (uint16_t)r;
      if (p.counts) scnt[at] = cc[j];
    }
    __syncthreads();
    for (uint32_t e = threadIdx.x; e < cn; e += blockDim.x) {
      const uint32_t r = sbin[e];
      const uint32_t at = hb[r] + (e - lstart[r]);
      p.keys[at] = sent[e];
      if (p.counts) p.counts[at] = scnt[e];
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < bins; i += blockDim.x) hb[i] += lcur[i] - lstart[i];
    __syncthreads();
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

uint64_t stage_words(uint64_t n, uint32_t nregions, int log_region) {
  if (n < kStageMinKeys || nregions < kStageMinRegions) return 0;
  const StagePlan sp = stage_plan(n, nregions, log_region);
  const uint64_t m = (uint64_t)sp.nb * sp.ntiles + 1;
  return m + (m + kScanChunk - 1) / kScanChunk + 1;  // histograms, their total, scan chunk sums
}

cudaError_t launch_partition_counted(const Geom& g, const Partition& p, const uint64_t* keys,
                                     const uint32_t* counts, uint64_t n, const unsigned long long* n_dev,
                                     int key_is_hash, uint32_t* status, cudaStream_t st) {
  const int shift = 8 + p.log_region;
  const uint64_t words = stage_words(n, p.nregions, p.log_region);
  if (words && p.stage && p.tiles && n <= p.stage_keys && words <= p.tile_words &&
      (!counts || p.stage_counts)) {
    const StagePlan sp = stage_plan(n, p.nregions, p.log_region);
    const uint64_t m = (uint64_t)sp.nb * sp.ntiles;  // histogram entries; tiles[m] gets the total
    uint32_t* sums = p.tiles + m + 1;
    k_stage_hist<<<sp.ntiles, kStageThreads, 0, st>>>(g, keys, n, n_dev, key_is_hash, shift, sp.s, sp.nb,
                                                      sp.ntiles, p.tiles, status);
    const uint32_t chunks = (uint32_t)((m + kScanChunk - 1) / kScanChunk);
    k_scan_sums<<<chunks, kScanThreads, 0, st>>>(p.tiles, (uint32_t)m, sums, n_dev, sp.nb, kStageTile);
    k_scan_apply<<<chunks, kScanThreads, 0, st>>>(p.tiles, (uint32_t)m, sums, p.tiles, nullptr, n_dev, sp.nb,
                                                  kStageTile);
    static std::atomic<bool> configured[kMaxDevices];
    once_per_device(configured, [] {
      cudaFuncSetAttribute(k_stage_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)scatter_smem(kMaxBuckets, true));
      cudaFuncSetAttribute(k_stage_bucket, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)bucket_smem(13, true));
    });
    k_stage_scatter<<<sp.ntiles, kStageThreads, scatter_smem(sp.nb, counts != nullptr), st>>>(
        g, keys, counts, n, n_dev, key_is_hash, shift, sp.s, sp.nb, sp.ntiles, p.tiles, p.stage, p.stage_counts);
    Partition q = p;
    q.counts = counts ? p.counts : nullptr;
    k_stage_bucket<<<sp.nb, kBucketThreads, bucket_smem(sp.s, counts != nullptr), st>>>(q, shift, sp.s, sp.ntiles,
                                                                                       n, n_dev);
    count_launch(5);
    return cudaGetLastError();
  }
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
