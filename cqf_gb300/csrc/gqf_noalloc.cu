// bulk_insert without any device allocation.
//
// Some callers cannot allocate device memory while they run: a serving
// process that reserves its whole device budget at start-up and forbids
// cudaMalloc afterwards, a plugin hosted by a framework that owns every
// device allocation, or a latency-critical loop that cannot afford the
// implicit device-wide synchronisation cudaMalloc/cudaFree may cause.  The
// regular bulk_insert grows per-filter partition scratch on demand; this entry
// point instead partitions the batch into one fixed array in the library's own
// device image, so it never allocates.
//
// Apart from where its scratch lives it is bulk_insert: the same partition and
// rebuild kernels, the same key-by-key threshold (gqf_set_sparse_max).  Its
// stream is the one passed in, NULL meaning the legacy default stream (as for
// the other *_async calls), not the filter's stream from gqf_set_stream.  The
// current device must be the one the filter was created on.
//
// The array (GQF_NOALLOC_SCRATCH_BYTES) is a file-scope __device__ variable:
// every GPU that loads the library holds it until the process exits.  Host
// code cannot use the variable's name as a device address, so the first call
// on each device (with that device current) looks the address up with
// cudaGetSymbolAddress and caches it; make that first call before any stream
// capture begins.  All calls share the one array and it keeps the last call's
// contents (the counters that must start at zero are cleared on every call),
// so calls that overlap on the GPU -- on different streams or filters -- race
// and must be serialised by the caller.
#include <cstdio>
#include <mutex>

#include "gqf_kernels.cuh"
#include "../../include/gqf.h"

namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[GQF_NOALLOC_SCRATCH_BYTES];

std::mutex g_setup_mu;
void* g_scratch_addr[gqf::kMaxDevices] = {nullptr};

}  // namespace

using namespace gqf;

extern "C" int gqf_bulk_insert_noalloc(QF* qf, uint64_t nvals, const uint64_t* keys, uint8_t flags,
                                       void* stream) {
  FilterView v;
  if (!internal_view(qf, &v)) return -1;
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    internal_set_error("gqf_bulk_insert_noalloc: no usable current device");
    return -1;
  }
  // The scratch address and the kernels' attributes belong to the current
  // device; the filter's memory lives on the device it was created on.
  if (dev != v.device) {
    char msg[160];
    std::snprintf(msg, sizeof msg,
                  "gqf_bulk_insert_noalloc: the current device is %d but the filter lives on device %d; "
                  "make that device current first", dev, v.device);
    internal_set_error(msg);
    return -1;
  }
  void* base = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_addr[dev]) {
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p) {
        char msg[160];
        std::snprintf(msg, sizeof msg, "gqf_bulk_insert_noalloc: cudaGetSymbolAddress failed: %s",
                      cudaGetErrorString(e));
        internal_set_error(msg);
        return -1;
      }
      g_scratch_addr[dev] = p;
    }
    base = g_scratch_addr[dev];
  }

  std::lock_guard<std::mutex> lk(*static_cast<std::mutex*>(v.mu));
  internal_view(qf, &v);  // geometry as of now, under the filter's lock
  // five per-region tables (counts, starts, cursors, deferred and retry
  // lists), then keys
  const uint64_t words = (uint64_t)v.nregions + 2;
  const uint64_t table_bytes = (20 * words + 255) & ~255ULL;
  const uint64_t max_keys = table_bytes < GQF_NOALLOC_SCRATCH_BYTES
                                ? (GQF_NOALLOC_SCRATCH_BYTES - table_bytes) / sizeof(uint32_t)
                                : 0;
  if (nvals > max_keys) {
    char msg[200];
    std::snprintf(msg, sizeof msg,
                  "gqf_bulk_insert_noalloc: a batch of %llu keys exceeds the %llu keys that fit the "
                  "%u-byte scratch for this filter; split the batch",
                  (unsigned long long)nvals, (unsigned long long)max_keys,
                  (unsigned)GQF_NOALLOC_SCRATCH_BYTES);
    internal_set_error(msg);
    return -1;
  }
  if (nvals == 0) return 0;
  if (!keys) {
    internal_set_error("gqf_bulk_insert_noalloc: null keys");
    return -1;
  }
  uint32_t* w = static_cast<uint32_t*>(base);
  Partition p{};
  p.region_count = w;
  p.region_start = w + words;
  p.cursor = w + 2 * words;
  p.deferred = w + 3 * words;
  p.retry = w + 4 * words;
  p.keys = reinterpret_cast<uint32_t*>(static_cast<unsigned char*>(base) + table_bytes);
  p.counts = nullptr;
  p.stats = v.stats;
  p.nregions = v.nregions;
  p.log_region = v.log_region;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int key_is_hash = (flags & QF_KEY_IS_HASH) ? 1 : 0;
  cudaError_t e = launch_partition(v.g, p, keys, nvals, key_is_hash, v.status, st);
  if (e == cudaSuccess)
    e = launch_rebuild(v.g, p, Op::kInsert, v.dqf, v.status, st, internal_sparse_max(qf, nvals));
  if (e != cudaSuccess) {
    char msg[160];
    std::snprintf(msg, sizeof msg, "gqf_bulk_insert_noalloc: %s", cudaGetErrorString(e));
    internal_set_error(msg);
    return -1;
  }
  return 0;
}
