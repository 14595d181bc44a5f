// Kernel entry points of the GB300 GQF and the host-side launchers that the
// C ABI (gqf_api.cu) calls.  Every launcher enqueues on the given stream and
// returns the launch error, never synchronising.
#pragma once
#include <cuda_runtime.h>

#include <atomic>

#include "gqf_device.cuh"

namespace gqf {

// Kernels launched by this library since load (every <<<>>> counts one).
extern std::atomic<unsigned long long> g_launches;
inline void count_launch(unsigned long long n = 1) { g_launches.fetch_add(n, std::memory_order_relaxed); }

// Launch geometry and kernel attributes (the dynamic shared-memory limit set
// by cudaFuncSetAttribute) belong to one device, so every cache of them is
// kept per device, indexed by the current device.
constexpr int kMaxDevices = 64;
inline int current_device() {
  int d = 0;
  if (cudaGetDevice(&d) != cudaSuccess || d < 0 || d >= kMaxDevices) d = 0;
  return d;
}
// SMs of the current device.
inline int sm_count() {
  static std::atomic<int> sms[kMaxDevices];
  const int d = current_device();
  int v = sms[d].load(std::memory_order_relaxed);
  if (!v) {
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, d) != cudaSuccess || v <= 0) v = 152;
    sms[d].store(v, std::memory_order_relaxed);
  }
  return v;
}
// Runs set_up() once per device for the cache `flags` (one array per kernel
// or kernel variant).
template <class F>
inline void once_per_device(std::atomic<bool>* flags, F&& set_up) {
  const int d = current_device();
  if (flags[d].load(std::memory_order_acquire)) return;
  set_up();
  flags[d].store(true, std::memory_order_release);
}

// Geometry of one filter as passed by value to kernels.
struct Geom {
  Block* blocks;
  uint64_t nslots, xnslots, nblocks;
  uint64_t range;   // 2^(nbits+8)
  uint64_t mask;    // range - 1
  uint32_t nbits;
};

// Scratch the bulk path partitions keys into.  Owned by the filter, grown on
// demand by the host (gqf_api.cu).
struct Partition {
  uint32_t* keys;          // region-local hashes, grouped by region
  uint32_t* counts;        // per-key multiplicities, or nullptr (all 1)
  uint32_t* region_count;  // nregions + 1
  uint32_t* region_start;  // nregions + 1 (exclusive prefix)
  uint32_t* cursor;        // nregions
  uint32_t* deferred;      // [0] = n, then region ids
  uint32_t* retry;         // nregions + 2: [0] = n, [1] = next taken, then region ids
  unsigned long long* stats;  // [0] regions deferred, [1] keys applied serially, [2] regions retried in
                              // the full window (or nullptr)
  uint32_t nregions;
  int log_region;          // a region is 2^log_region quotients
  // Staging of the two-level partition of large batches (launch_partition*),
  // or nullptr for the single-level path: a packed entry per key, its count,
  // and the per-tile bucket histograms (stage_words(...) words).
  uint32_t* stage;
  uint32_t* stage_counts;
  uint32_t* tiles;
  uint64_t stage_keys;     // entries stage holds
  uint64_t tile_words;     // words tiles holds
};
// Words of Partition::tiles a batch of n keys needs (0: the single-level
// path runs for such batches).
uint64_t stage_words(uint64_t n, uint32_t nregions, int log_region);

enum class Op : int { kInsert = 0, kDelete = 1 };

// Where the regions of one rebuild launch live.  Region R of the launch is
// region r of the filter `q` with geometry `g`.
struct OneFilter {  // R = r
  Geom g;
  const quotient_filter* dqf;
  __device__ __forceinline__ bool locate(uint32_t R, int, Geom* gg, uint32_t* r,
                                         const quotient_filter** q) const {
    *gg = g;
    *r = R;
    *q = dqf;
    return true;
  }
};

// Many filters in one launch: their regions are numbered one after the
// other, filter f's from region_base[f]; each filter's count is rounded up to
// an even number so that parities agree (the padding regions are empty).
struct FilterSet {
  const quotient_filter* qfs;    // n descriptors in device memory
  const uint32_t* region_base;   // n + 1 entries, device memory
  uint32_t n;
  __device__ __forceinline__ bool locate(uint32_t R, int log_region, Geom* gg, uint32_t* r,
                                         const quotient_filter** q) const {
    uint32_t lo = 0, hi = n;  // the last f with region_base[f] <= R
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (region_base[mid] <= R) lo = mid;
      else hi = mid;
    }
    const quotient_filter* f = qfs + lo;
    const uint32_t rr = R - region_base[lo];
    const uint64_t nreg = f->nslots >> log_region;
    if (rr >= (nreg ? nreg : 1)) return false;
    gg->blocks = f->blocks;
    gg->nslots = f->nslots;
    gg->xnslots = f->xnslots;
    gg->nblocks = f->nblocks;
    gg->range = f->range;
    gg->mask = f->range - 1;
    gg->nbits = f->nbits;
    *r = rr;
    *q = f;
    return true;
  }
};

// What other translation units of the library may see of a filter.
struct FilterView {
  Geom g;
  quotient_filter* dqf;
  uint32_t* status;
  unsigned long long* stats;
  int log_region;
  uint32_t nregions;
  cudaStream_t stream;
  void* mu;  // std::mutex* serialising calls on the filter
  int device;  // the device holding the filter's memory
};
bool internal_view(const quotient_filter* qf, FilterView* v);
// The key-by-key threshold bulk_insert uses for a batch of n keys on qf.
uint32_t internal_sparse_max(const quotient_filter* qf, uint64_t n);
void internal_set_error(const char* msg);

// Region sizes the rebuild kernel is instantiated for.
constexpr int kMinLogRegion = 11;
constexpr int kMaxLogRegion = 13;

cudaError_t launch_bulk_get(const Geom& g, const uint64_t* keys, uint64_t n, uint64_t* out,
                            int key_is_hash, cudaStream_t st);
cudaError_t launch_bulk_get_misses(const Geom& g, const uint64_t* keys, uint64_t n,
                                   unsigned long long* misses, cudaStream_t st);

// hash -> per-region counts -> prefix -> scatter of region-local hashes.
cudaError_t launch_partition(const Geom& g, const Partition& p, const uint64_t* keys, uint64_t n,
                             int key_is_hash, uint32_t* status, cudaStream_t st);

// Exclusive scan of p.region_count into p.region_start and p.cursor (and
// region_start[nregions] = total), using p.deferred as scratch.
cudaError_t launch_region_scan(const Partition& p, cudaStream_t st);

// The same for (hash, count) pairs whose number n_dev the device holds (n
// bounds it): hashes are taken as they are, counts land in p.counts.
cudaError_t launch_partition_counted(const Geom& g, const Partition& p, const uint64_t* keys,
                                     const uint32_t* counts, uint64_t n, const unsigned long long* n_dev,
                                     int key_is_hash, uint32_t* status, cudaStream_t st);

// Duplicate merging for bulk_insert_reduce.  Tile pass: each CTA merges the
// equal hashes of a tile of keys in a shared-memory table and appends
// (hash, count) pairs at out_*[*n_out].  Region pass: regions left with more
// pairs than one rebuild round takes (with n_merged, the pair count of a tile
// pass over n_in keys, fewer when that pass found heavy duplication) are
// merged again in place, shrinking p.region_count.
cudaError_t launch_merge_tiles(const Geom& g, const uint64_t* keys, uint64_t n, int key_is_hash,
                               uint64_t* out_hashes, uint32_t* out_counts, unsigned long long* n_out,
                               uint32_t* status, cudaStream_t st);
cudaError_t launch_merge_regions(const Partition& p, cudaStream_t st, const unsigned long long* n_merged = nullptr,
                                 uint64_t n_in = 0);

// K-mers of fixed-length reads (read_len bytes each, ACGT in either case):
// the tile pass over the canonical k-mers (2-bit packed, first base in the
// high bits), hashed like keys; and a plain extraction into out[read * nk +
// pos], nk = read_len - k + 1, ~0 for windows holding another byte.
bool kmer_shape_ok(uint64_t nreads, uint32_t read_len, uint32_t k);
cudaError_t launch_merge_kmers(const Geom& g, const uint8_t* reads, uint64_t nreads, uint32_t read_len,
                               uint32_t k, uint64_t* out_hashes, uint32_t* out_counts,
                               unsigned long long* n_out, cudaStream_t st);
cudaError_t launch_kmers(const uint8_t* reads, uint64_t nreads, uint32_t read_len, uint32_t k, uint64_t* out,
                         cudaStream_t st);

// Even regions, then odd regions, then the serial fallback for regions whose
// rebuild window was exceeded.  Regions holding at most sparse_max keys are
// updated key by key instead of rebuilt (0: rebuild every region).
constexpr uint32_t kDefaultSparseMax = 32;
cudaError_t launch_rebuild(const Geom& g, const Partition& p, Op op, quotient_filter* dqf,
                           uint32_t* status, cudaStream_t st, uint32_t sparse_max = kDefaultSparseMax);
size_t rebuild_smem_bytes(int log_region);

// Enumeration (gqf_iter.cu): pairs per block, then the pairs themselves at
// start[b] (an exclusive scan of the per-block numbers) in hash order.
cudaError_t launch_enum_count(const Geom& g, uint32_t* per_block, cudaStream_t st);
cudaError_t launch_enum_write(const Geom& g, const uint32_t* start, int as_keys, uint64_t* out_h, uint64_t* out_c,
                              uint32_t* out_c32, uint32_t* overflow, cudaStream_t st);
// Probes `mem` for n (hash, count) pairs: *acc += count * count in mem, and/or
// the pairs present in mem appended at out_*[*n_out].
cudaError_t launch_pair_probe(const Geom& mem, const uint64_t* h, const uint64_t* c, uint64_t n,
                              unsigned long long* acc, uint64_t* out_h, uint32_t* out_c32,
                              unsigned long long* n_out, uint32_t* overflow, cudaStream_t st);

cudaError_t launch_export(const Geom& g, uint8_t* packed, cudaStream_t st);
cudaError_t launch_import(const Geom& g, const uint8_t* packed, cudaStream_t st);
cudaError_t launch_import_fix(quotient_filter* dqf, const uint8_t* packed, cudaStream_t st);

// Point-API batch kernels (one thread per key).
cudaError_t launch_point_insert(quotient_filter* dqf, const uint64_t* keys, uint64_t n, uint8_t flags,
                                int8_t* rets, cudaStream_t st);
cudaError_t launch_point_insert_not_exists(quotient_filter* dqf, const uint64_t* keys, uint64_t n,
                                           uint8_t flags, int8_t* rets, uint8_t* vals,
                                           cudaStream_t st);
cudaError_t launch_point_query(quotient_filter* dqf, const uint64_t* keys, uint64_t n, uint8_t flags,
                               int concurrent, uint64_t* counts, cudaStream_t st);
cudaError_t launch_point_get_misses(quotient_filter* dqf, const uint64_t* keys, uint64_t n,
                                    unsigned long long* misses, cudaStream_t st);
cudaError_t launch_point_bulk_insert(quotient_filter* dqf, uint64_t* keys, uint64_t n, cudaStream_t st);
cudaError_t launch_serial_apply(quotient_filter* dqf, const uint64_t* hashes, uint64_t n, int op,
                                cudaStream_t st);

}  // namespace gqf
