// Duplicate merging for bulk_insert_reduce (the skewed-counting path).
//
// The reference sorts the whole batch of hashes and runs reduce_by_key over
// it before a counted insert of each distinct hash (src/gqf.cu:3238-3313,
// thrust::sort + thrust::reduce_by_key, then insert() with a count,
// :1768-1874).  Only equal hashes need to meet, not a total order, so here:
//
//   tile pass    each CTA hashes a tile of 4096 keys and merges equal hashes
//                in an open-addressing table in shared memory (warp peers
//                with the same hash share one table update, match.any), then
//                appends its distinct (hash, count) pairs to one array;
//   partition    the pairs go through the usual region partition, counts
//                carried along (gqf_partition.cu);
//   region pass  a region left with more pairs than one rebuild round takes
//                (the same hot hash arriving from many tiles) is merged again
//                in shared memory and compacted in place;
//   rebuild      the counted rebuild adds each pair's count to its counter
//                (gqf_rebuild.cu, CNT).
//
// Under a Zipf(1.5) law a 4096-key tile holds a few hundred distinct hashes,
// so the batch shrinks about tenfold before it is partitioned.  A uniform
// batch passes through unchanged, at the cost of one extra pass.
#include "gqf_kernels.cuh"

namespace gqf {
namespace {

constexpr int kTileThreads = 512;
constexpr int kTileKeys = 4096;
constexpr int kTileSlots = 8192;  // table load stays <= 1/2
constexpr int kTileSmem = kTileSlots * (8 + 4);

constexpr int kRegionThreads = 512;
constexpr int kRegionSlots = 8192;
constexpr int kRegionMaxDistinct = kRegionSlots / 2;
constexpr int kRegionSmem = kRegionSlots * (4 + 4);
constexpr uint32_t kSkewLimit = 64;

__device__ __forceinline__ uint32_t table_slot(uint64_t h, int log_slots) {
  return (uint32_t)((h * 0x9E3779B97F4A7C15ULL) >> (64 - log_slots));  // Fibonacci hashing
}

// Block-wide exclusive sum (NT threads); also returns the total.
template <int NT>
__device__ int block_scan(int v, int* tmp, int* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += t;
  }
  if (lane == 31) tmp[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int w = lane < NT / 32 ? tmp[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      int t = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += t;
    }
    tmp[lane] = w;
  }
  __syncthreads();
  int r = x - v + (wid ? tmp[wid - 1] : 0);
  *total = tmp[NT / 32 - 1];
  __syncthreads();
  return r;
}

// Keys of a tile from a key array (hashed here unless key_is_hash).
struct ArraySource {
  Geom g;
  const uint64_t* keys;
  uint64_t n;
  int key_is_hash;
  uint32_t* status;
  __device__ uint64_t ntiles() const { return (n + kTileKeys - 1) / kTileKeys; }
  // Calls add(hash + 1, or 0 for none) the same number of times on every lane.
  template <class F>
  __device__ void tile(uint64_t t, F&& add) const {
    const uint64_t b = t * kTileKeys;
    for (int j = threadIdx.x; j < kTileKeys; j += kTileThreads) {
      const uint64_t i = b + j;
      unsigned long long key = 0;
      if (i < n) {
        const uint64_t k = __ldcs(keys + i);
        if (!key_is_hash) key = hash64(k, g.mask) + 1;
        else if (k < g.range) key = k + 1;
        else atomicOr(status, kStBadKey);
      }
      add(key);
    }
  }
};

// 2-bit code of a base (A C G T, either case), or -1.
__device__ __forceinline__ int base_code(uint8_t c) {
  switch (c | 0x20) {
    case 'a': return 0;
    case 'c': return 1;
    case 'g': return 2;
    case 't': return 3;
  }
  return -1;
}

// Canonical k-mers of fixed-length reads: a tile is the k-mers of
// kTileKeys / nk whole reads; each thread takes `per` consecutive k-mers and
// rolls the forward and reverse-complement words from one to the next.
struct KmerSource {
  Geom g;
  const uint8_t* reads;
  uint64_t nreads;
  uint32_t len, k, nk, reads_per_tile, per;
  __host__ __device__ uint64_t ntiles() const { return (nreads + reads_per_tile - 1) / reads_per_tile; }
  uint64_t ntiles_host() const { return ntiles(); }
  template <class F>
  __device__ void tile(uint64_t t, F&& add) const {
    const uint64_t kmask = k == 32 ? ~0ULL : (1ULL << (2 * k)) - 1ULL;
    const int hi = 2 * ((int)k - 1);
    const uint32_t items = reads_per_tile * nk;
    uint64_t fw = 0, rc = 0;
    uint32_t good = 0;  // valid bases ending at the current position
    uint64_t cur_read = ~0ULL;
    uint32_t cur_pos = 0;
    for (uint32_t step = 0; step < per; step++) {
      const uint32_t item = threadIdx.x * per + step;
      const uint64_t read = t * reads_per_tile + item / nk;
      const uint32_t pos = item % nk;
      unsigned long long key = 0;
      if (item < items && read < nreads) {
        const uint8_t* rd = reads + read * len;
        uint32_t from = pos;  // first base still to shift in
        if (read != cur_read || pos != cur_pos + 1) {
          fw = rc = 0;
          good = 0;
          from = pos;
        } else {
          from = pos + k - 1;
        }
        for (uint32_t x = from; x < pos + k; x++) {
          const int b = base_code(rd[x]);
          if (b < 0) {
            good = 0;
            fw = rc = 0;
            continue;
          }
          fw = ((fw << 2) | (uint64_t)b) & kmask;
          rc = (rc >> 2) | ((uint64_t)(3 - b) << hi);
          good++;
        }
        cur_read = read;
        cur_pos = pos;
        if (good >= k) key = hash64(fw < rc ? fw : rc, g.mask) + 1;
      }
      add(key);
    }
  }
};

template <class Src>
__global__ void __launch_bounds__(kTileThreads) k_merge_tiles(Src src, uint64_t* __restrict__ out_h,
                                                              uint32_t* __restrict__ out_c,
                                                              unsigned long long* n_out) {
  extern __shared__ __align__(16) uint8_t smem[];
  unsigned long long* tk = reinterpret_cast<unsigned long long*>(smem);  // hash + 1, 0 = empty
  uint32_t* tc = reinterpret_cast<uint32_t*>(smem + kTileSlots * 8);
  __shared__ int tmp[32];
  __shared__ unsigned long long s_base;
  constexpr int PER = kTileSlots / kTileThreads;
  const int tid = threadIdx.x, lane = tid & 31;
  const uint64_t ntiles = src.ntiles();
  auto add = [&](unsigned long long key) {  // warp-convergent
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    if (key && lane == __ffs(peers) - 1) {
      uint32_t s = table_slot(key, 13);
      for (int probe = 0; probe < kTileSlots; probe++) {  // at most half full: ends early
        unsigned long long cur = tk[s];
        if (cur == 0) {
          cur = atomicCAS(&tk[s], 0ULL, key);
          if (cur == 0) cur = key;
        }
        if (cur == key) {
          atomicAdd(&tc[s], (uint32_t)__popc(peers));
          break;
        }
        s = (s + 1) & (kTileSlots - 1);
      }
    }
  };
  for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    for (int i = tid; i < kTileSlots; i += kTileThreads) { tk[i] = 0; tc[i] = 0; }
    __syncthreads();
    src.tile(t, add);
    __syncthreads();
    // compact this thread's PER consecutive table slots
    int cnt = 0;
    for (int s = tid * PER; s < tid * PER + PER; s++) cnt += tk[s] != 0;
    int tot;
    const int ex = block_scan<kTileThreads>(cnt, tmp, &tot);
    if (tid == 0) s_base = atomicAdd(n_out, (unsigned long long)tot);
    __syncthreads();
    unsigned long long at = s_base + ex;
    for (int s = tid * PER; s < tid * PER + PER; s++) {
      const unsigned long long k = tk[s];
      if (k) {
        out_h[at] = k - 1;
        out_c[at] = tc[s];
        at++;
      }
    }
    __syncthreads();
  }
}

// Standalone extraction: out[read * nk + pos] = the canonical k-mer at pos,
// or ~0 when its window holds a byte other than ACGT (never a canonical
// k-mer: the complement of all-T is all-A).
__global__ void __launch_bounds__(256) k_kmers(const uint8_t* __restrict__ reads, uint64_t nreads,
                                               uint32_t len, uint32_t k, uint32_t nk, uint32_t per,
                                               uint64_t* __restrict__ out) {
  const uint64_t kmask = k == 32 ? ~0ULL : (1ULL << (2 * k)) - 1ULL;
  const int hi = 2 * ((int)k - 1);
  const uint32_t chunks = (nk + per - 1) / per;
  const uint64_t total = nreads * chunks;
  for (uint64_t c = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; c < total;
       c += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t read = c / chunks;
    const uint32_t p0 = (uint32_t)(c % chunks) * per;
    const uint32_t p1 = min(nk, p0 + per);
    const uint8_t* rd = reads + read * len;
    uint64_t fw = 0, rc = 0;
    uint32_t good = 0;
    for (uint32_t x = p0; x < p1 + k - 1; x++) {
      const int b = base_code(rd[x]);
      if (b < 0) {
        good = 0;
        fw = rc = 0;
      } else {
        fw = ((fw << 2) | (uint64_t)b) & kmask;
        rc = (rc >> 2) | ((uint64_t)(3 - b) << hi);
        good++;
      }
      if (x + 1 >= p0 + k) out[read * nk + (x + 1 - k)] = good >= k ? (fw < rc ? fw : rc) : ~0ULL;
    }
  }
}

// Merges, in place, the pairs of every region holding more than `limit`
// (one rebuild round).  A region with more than kRegionMaxDistinct distinct
// hashes is left as it is: the rebuild then takes it in several rounds.
__global__ void __launch_bounds__(kRegionThreads) k_merge_regions(Partition p, uint32_t limit,
                                                                  const unsigned long long* n_merged,
                                                                  uint64_t n_in) {
  // A counted insert (n_merged given) merges every region past kSkewLimit
  // pairs again: repeats of a key that arrive from many tiles (a hot key, or
  // a k-mer seen once per covering read) then reach the rebuild once.
  if (n_merged) limit = kSkewLimit;
  (void)n_in;
  extern __shared__ __align__(16) uint8_t smem[];
  uint32_t* tk = reinterpret_cast<uint32_t*>(smem);  // local hash + 1, 0 = empty
  uint32_t* tc = reinterpret_cast<uint32_t*>(smem + kRegionSlots * 4);
  __shared__ int tmp[32];
  __shared__ int s_n, s_over;
  constexpr int PER = kRegionSlots / kRegionThreads;
  const int tid = threadIdx.x, lane = tid & 31;
  for (uint32_t r = blockIdx.x; r < p.nregions; r += gridDim.x) {
    const uint32_t len = p.region_count[r];
    if (len <= limit) continue;  // uniform over the CTA
    const uint32_t beg = p.region_start[r];
    for (int i = tid; i < kRegionSlots; i += kRegionThreads) { tk[i] = 0; tc[i] = 0; }
    if (tid == 0) { s_n = 0; s_over = 0; }
    __syncthreads();
    const uint32_t lenr = (len + 31) & ~31u;
    for (uint32_t i = tid; i < lenr; i += kRegionThreads) {
      const bool ok = i < len;
      const uint32_t key = ok ? p.keys[beg + i] + 1 : 0;
      const uint32_t c = ok ? p.counts[beg + i] : 0;
      const unsigned peers = __match_any_sync(0xffffffffu, key);
      uint32_t sum = 0;  // the counts of this lane's peers
      for (int src = 0; src < 32; src++) {
        const uint32_t v = __shfl_sync(0xffffffffu, c, src);
        if ((peers >> src) & 1u) sum += v;
      }
      if (ok && lane == __ffs(peers) - 1 && !s_over) {
        uint32_t s = table_slot(key, 13);
        bool placed = false;
        for (int probe = 0; probe < kRegionSlots; probe++) {
          uint32_t cur = tk[s];
          if (cur == 0) {
            if (atomicAdd(&s_n, 1) >= kRegionMaxDistinct) {  // too many distinct: give up
              s_over = 1;
              break;
            }
            cur = atomicCAS(&tk[s], 0u, key);
            if (cur == 0) cur = key;
            else atomicSub(&s_n, 1);
          }
          if (cur == key) {
            atomicAdd(&tc[s], sum);
            placed = true;
            break;
          }
          s = (s + 1) & (kRegionSlots - 1);
        }
        if (!placed) s_over = 1;
      }
    }
    __syncthreads();
    if (s_over) {  // uniform; keep the region's pairs as they are
      __syncthreads();
      continue;
    }
    int cnt = 0;
    for (int s = tid * PER; s < tid * PER + PER; s++) cnt += tk[s] != 0;
    int tot;
    const int ex = block_scan<kRegionThreads>(cnt, tmp, &tot);
    uint32_t at = beg + (uint32_t)ex;
    for (int s = tid * PER; s < tid * PER + PER; s++) {
      if (tk[s]) {
        p.keys[at] = tk[s] - 1;
        p.counts[at] = tc[s];
        at++;
      }
    }
    if (tid == 0) p.region_count[r] = (uint32_t)tot;
    __syncthreads();
  }
}

}  // namespace

template <class Src>
cudaError_t run_merge_tiles(const Src& src, uint64_t ntiles, uint64_t* out_hashes, uint32_t* out_counts,
                            unsigned long long* n_out, cudaStream_t st) {
  static std::atomic<bool> configured[kMaxDevices];  // per source type and device
  once_per_device(configured, [] {
    cudaFuncSetAttribute(k_merge_tiles<Src>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTileSmem);
  });
  if (ntiles == 0) return cudaSuccess;
  const uint64_t cap = (uint64_t)sm_count() * 2;  // two 96 KB tables per SM
  const int grid = (int)(ntiles < cap ? ntiles : cap);
  k_merge_tiles<Src><<<grid, kTileThreads, kTileSmem, st>>>(src, out_hashes, out_counts, n_out);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_merge_tiles(const Geom& g, const uint64_t* keys, uint64_t n, int key_is_hash,
                               uint64_t* out_hashes, uint32_t* out_counts, unsigned long long* n_out,
                               uint32_t* status, cudaStream_t st) {
  ArraySource src{g, keys, n, key_is_hash, status};
  return run_merge_tiles(src, (n + kTileKeys - 1) / kTileKeys, out_hashes, out_counts, n_out, st);
}

bool kmer_shape_ok(uint64_t nreads, uint32_t read_len, uint32_t k) {
  return k >= 1 && k <= 32 && read_len >= k && read_len - k + 1 <= (uint32_t)kTileKeys &&
         nreads <= (~0ULL) / read_len;
}

cudaError_t launch_merge_kmers(const Geom& g, const uint8_t* reads, uint64_t nreads, uint32_t read_len,
                               uint32_t k, uint64_t* out_hashes, uint32_t* out_counts,
                               unsigned long long* n_out, cudaStream_t st) {
  if (!kmer_shape_ok(nreads, read_len, k)) return cudaErrorInvalidValue;
  KmerSource src{};
  src.g = g;
  src.reads = reads;
  src.nreads = nreads;
  src.len = read_len;
  src.k = k;
  src.nk = read_len - k + 1;
  src.reads_per_tile = (uint32_t)kTileKeys / src.nk;
  src.per = (src.reads_per_tile * src.nk + kTileThreads - 1) / kTileThreads;
  return run_merge_tiles(src, src.ntiles_host(), out_hashes, out_counts, n_out, st);
}

cudaError_t launch_kmers(const uint8_t* reads, uint64_t nreads, uint32_t read_len, uint32_t k, uint64_t* out,
                         cudaStream_t st) {
  if (!kmer_shape_ok(nreads, read_len, k)) return cudaErrorInvalidValue;
  if (nreads == 0) return cudaSuccess;
  const uint32_t nk = read_len - k + 1, per = 8;
  const uint64_t chunks = nreads * ((nk + per - 1) / per);
  const uint64_t want = (chunks + 255) / 256, cap = (uint64_t)sm_count() * 16;
  k_kmers<<<(int)(want < cap ? want : cap), 256, 0, st>>>(reads, nreads, read_len, k, nk, per, out);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_merge_regions(const Partition& p, cudaStream_t st, const unsigned long long* n_merged,
                                 uint64_t n_in) {
  static std::atomic<bool> configured[kMaxDevices];
  once_per_device(configured, [] {
    cudaFuncSetAttribute(k_merge_regions, cudaFuncAttributeMaxDynamicSharedMemorySize, kRegionSmem);
  });
  if (!p.counts) return cudaErrorInvalidValue;
  const uint32_t limit = p.log_region >= 13 ? 4096u : 2048u;  // keys one rebuild round takes
  const uint32_t cap = (uint32_t)sm_count() * 3;
  const uint32_t grid = p.nregions < cap ? p.nregions : cap;
  k_merge_regions<<<grid ? grid : 1, kRegionThreads, kRegionSmem, st>>>(p, limit, n_merged, n_in);
  count_launch();
  return cudaGetLastError();
}

}  // namespace gqf
