// Host side of the C ABI declared in include/gqf.h.
//
// Replaces the reference's host orchestration (src/gqf.cu:2123-2269 and
// :3184-3419).  Differences that matter for performance:
//   * no per-call device->host readback of num_locks and no
//     cudaDeviceSynchronize (the reference does both on every bulk call,
//     src/gqf.cu:3193-3201); geometry lives in a host mirror;
//   * no per-call device allocation (thrust temporaries, managed memory):
//     partition scratch is owned by the filter and grown stream-ordered;
//   * the filter is built on the device (memset), not on the host and copied.
#include <atomic>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include "gqf_kernels.cuh"
#include "../../include/gqf.h"

using namespace gqf;

namespace gqf {
std::atomic<unsigned long long> g_launches{0};
}

namespace {

thread_local std::string g_err;

void set_err(const std::string& s) { g_err = s; }

bool ck(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return true;
  set_err(std::string(what) + ": " + cudaGetErrorString(e));
  return false;
}

struct HostFilter {
  QF* dqf = nullptr;        // device descriptor: the handle users hold
  quotient_filter h{};      // host mirror of the descriptor
  Geom g{};
  cudaStream_t stream = 0;  // legacy default stream, like the reference
  int device = 0;           // the device the filter's memory lives on
  int log_region = 12;
  bool auto_region = true;
  uint32_t sparse_max = GQF_SPARSE_AUTO;  // regions with <= this many keys go key by key
  uint8_t* aux = nullptr;   // status word + miss counter
  Partition part{};
  uint64_t key_cap = 0;
  uint32_t region_cap = 0;
  bool counts_alloc = false;
  uint64_t* merge_h = nullptr;  // bulk_insert_reduce: merged (hash, count) pairs
  uint32_t* merge_c = nullptr;
  uint64_t merge_cap = 0;
  uint8_t* packed = nullptr;  // export / import staging
  // phase timers (CUDA events on the launching stream), off by default
  bool prof = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending[GQF_PROF_PHASES];
  std::vector<cudaEvent_t> spare;
  double prof_ms[GQF_PROF_PHASES] = {0};
  uint64_t prof_calls[GQF_PROF_PHASES] = {0};
  uint64_t prof_keys[GQF_PROF_PHASES] = {0};
  std::mutex mu;
};

cudaEvent_t take_event(HostFilter* f) {
  if (!f->spare.empty()) {
    cudaEvent_t e = f->spare.back();
    f->spare.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

// Brackets one phase of work on stream st with a pair of events.
struct PhaseTimer {
  HostFilter* f;
  int phase;
  cudaStream_t st;
  cudaEvent_t e0 = nullptr;
  PhaseTimer(HostFilter* f_, int ph, cudaStream_t s, uint64_t keys) : f(f_), phase(ph), st(s) {
    if (!f->prof) return;
    e0 = take_event(f);
    cudaEventRecord(e0, st);
    f->prof_calls[phase]++;
    f->prof_keys[phase] += keys;
  }
  ~PhaseTimer() {
    if (!e0) return;
    cudaEvent_t e1 = take_event(f);
    cudaEventRecord(e1, st);
    f->pending[phase].push_back({e0, e1});
  }
};

std::mutex g_mu;
std::unordered_map<const QF*, HostFilter*> g_filters;

HostFilter* lookup(const QF* qf) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_filters.find(qf);
  if (it == g_filters.end()) {
    set_err("unknown QF handle");
    return nullptr;
  }
  return it->second;
}

int auto_log_region(int nbits) {
  // 2^12-quotient regions fit four or five rebuild CTAs per SM and measured
  // fastest on large tables; small tables use 2^11 for more regions per phase.
  return nbits >= 21 ? 12 : 11;
}

uint32_t* status_ptr(HostFilter* f) { return reinterpret_cast<uint32_t*>(f->aux); }
unsigned long long* misses_ptr(HostFilter* f) { return reinterpret_cast<unsigned long long*>(f->aux + 64); }
unsigned long long* stats_ptr(HostFilter* f) { return reinterpret_cast<unsigned long long*>(f->aux + 128); }
unsigned long long* merged_ptr(HostFilter* f) { return reinterpret_cast<unsigned long long*>(f->aux + 192); }

uint32_t nregions_for(const HostFilter* f, int log_region) {
  uint64_t n = f->h.nslots >> log_region;
  return (uint32_t)(n ? n : 1);
}

// Key-by-key threshold in use.  The automatic one weighs the key-by-key
// kernel, whose time follows its busiest region (about k sequential
// single-key updates of ~25 us each, one thread per region), against a
// rebuild of every region (~75 ns per region on a GB300): a region of k keys
// goes key by key while 2 k * 25 us stays under half of nregions * 75 ns.
uint32_t sparse_max_of(const HostFilter* f) {
  if (f->sparse_max != GQF_SPARSE_AUTO) return f->sparse_max;
  const uint32_t t = nregions_for(f, f->log_region) / 1400;
  return t < 16 ? 16 : t > 256 ? 256 : t;
}

// The threshold for a batch of n keys.  Under the automatic choice a batch
// averaging more than half the threshold per region leaves few regions to
// the key-by-key kernel, whose time is still set by its busiest region, so
// such batches rebuild every touched region.
uint32_t sparse_max_for(const HostFilter* f, uint64_t n) {
  const uint32_t t = sparse_max_of(f);
  if (f->sparse_max != GQF_SPARSE_AUTO) return t;
  const uint64_t per_region = n / nregions_for(f, f->log_region);
  return 2 * per_region <= t ? t : 0;
}

// Grow partition scratch (stream-ordered, so work already queued keeps its
// buffers until it completes).
bool ensure_partition(HostFilter* f, uint64_t nkeys, bool with_counts, cudaStream_t st) {
  const uint32_t nr = nregions_for(f, f->log_region);
  if (nkeys > 0xFFFFFFF0ULL) {
    set_err("batch larger than 2^32 keys");
    return false;
  }
  if (nkeys > f->key_cap || (with_counts && !f->counts_alloc)) {
    const uint64_t cap = nkeys > f->key_cap ? nkeys + nkeys / 8 + 1024 : f->key_cap;
    const bool had_counts = f->counts_alloc;
    if (f->part.keys) cudaFreeAsync(f->part.keys, st);
    if (f->part.counts) cudaFreeAsync(f->part.counts, st);
    // until both allocations succeed the filter holds no key scratch, so a
    // failed growth is retried by the next call instead of reused
    f->part.keys = nullptr;
    f->part.counts = nullptr;
    f->key_cap = 0;
    f->counts_alloc = false;
    if (!ck(cudaMallocAsync((void**)&f->part.keys, cap * sizeof(uint32_t), st), "cudaMallocAsync keys"))
      return false;
    if (with_counts || had_counts) {
      if (!ck(cudaMallocAsync((void**)&f->part.counts, cap * sizeof(uint32_t), st), "cudaMallocAsync counts"))
        return false;
      f->counts_alloc = true;
    }
    f->key_cap = cap;
  }
  if (nr + 2 > f->region_cap) {
    uint32_t cap = nr + 2;
    if (f->part.region_count) cudaFreeAsync(f->part.region_count, st);
    f->part.region_count = f->part.region_start = f->part.cursor = f->part.deferred = f->part.retry = nullptr;
    f->region_cap = 0;
    uint32_t* base = nullptr;
    // region_count | region_start | cursor | deferred | retry, one allocation
    if (!ck(cudaMallocAsync((void**)&base, 5ULL * cap * sizeof(uint32_t), st), "cudaMallocAsync regions"))
      return false;
    f->part.region_count = base;
    f->part.region_start = base + cap;
    f->part.cursor = base + 2ULL * cap;
    f->part.deferred = base + 3ULL * cap;
    f->part.retry = base + 4ULL * cap;
    f->region_cap = cap;
  }
  // staging of the two-level partition (large batches); without it those
  // batches take the single-level path
  if (const uint64_t words = stage_words(nkeys, nr, f->log_region)) {
    Partition& p = f->part;
    if (nkeys > p.stage_keys || (with_counts && !p.stage_counts)) {
      const uint64_t cap = nkeys > p.stage_keys ? nkeys + nkeys / 8 + 1024 : p.stage_keys;
      const bool had_counts = p.stage_counts != nullptr;
      if (p.stage) cudaFreeAsync(p.stage, st);
      if (p.stage_counts) cudaFreeAsync(p.stage_counts, st);
      p.stage = p.stage_counts = nullptr;
      p.stage_keys = 0;
      if (cudaMallocAsync((void**)&p.stage, cap * sizeof(uint32_t), st) != cudaSuccess) {
        p.stage = nullptr;
      } else if ((with_counts || had_counts) &&
                 cudaMallocAsync((void**)&p.stage_counts, cap * sizeof(uint32_t), st) != cudaSuccess) {
        p.stage_counts = nullptr;
        cudaFreeAsync(p.stage, st);
        p.stage = nullptr;
      } else {
        p.stage_keys = cap;
      }
    }
    if (words > p.tile_words) {
      if (p.tiles) cudaFreeAsync(p.tiles, st);
      p.tiles = nullptr;
      p.tile_words = 0;
      const uint64_t cap = words + words / 8 + 64;
      if (cudaMallocAsync((void**)&p.tiles, cap * sizeof(uint32_t), st) == cudaSuccess) p.tile_words = cap;
      else p.tiles = nullptr;
    }
    cudaGetLastError();  // a failed staging allocation is not an error: the single level runs
  }
  f->part.nregions = nr;
  f->part.log_region = f->log_region;
  f->part.stats = stats_ptr(f);
  return true;
}

bool ensure_merge(HostFilter* f, uint64_t nkeys, cudaStream_t st) {
  if (nkeys <= f->merge_cap) return true;
  const uint64_t cap = nkeys + nkeys / 8 + 1024;
  if (f->merge_h) cudaFreeAsync(f->merge_h, st);
  if (f->merge_c) cudaFreeAsync(f->merge_c, st);
  f->merge_h = nullptr;
  f->merge_c = nullptr;
  f->merge_cap = 0;
  if (!ck(cudaMallocAsync((void**)&f->merge_h, cap * sizeof(uint64_t), st), "cudaMallocAsync merge") ||
      !ck(cudaMallocAsync((void**)&f->merge_c, cap * sizeof(uint32_t), st), "cudaMallocAsync merge"))
    return false;
  f->merge_cap = cap;
  return true;
}

// bulk_insert_reduce: equal hashes are merged into (hash, count) pairs first
// (gqf_reduce.cu), then partitioned and rebuilt with counts.  With reads,
// the keys are the reads' canonical k-mers instead of keys[].
int do_bulk_reduce(HostFilter* f, uint64_t n, const uint64_t* keys, uint8_t flags, cudaStream_t st,
                   const uint8_t* reads = nullptr, uint64_t nreads = 0, uint32_t read_len = 0,
                   uint32_t k = 0) {
  std::lock_guard<std::mutex> lk(f->mu);
  if (reads) {
    if (!kmer_shape_ok(nreads, read_len, k)) {
      set_err("k-mers: need 1 <= k <= 32 and k <= read_len <= k + 4095");
      return -1;
    }
    n = nreads * (read_len - k + 1);
  } else if (!keys && n) {
    set_err("null keys");
    return -1;
  }
  if (n == 0) return 0;
  if (!ensure_partition(f, n, true, st) || !ensure_merge(f, n, st)) return -1;
  Partition p = f->part;
  const int key_is_hash = (flags & QF_KEY_IS_HASH) ? 1 : 0;
  {
    PhaseTimer t(f, GQF_PROF_PARTITION, st, n);
    if (!ck(cudaMemsetAsync(merged_ptr(f), 0, sizeof(unsigned long long), st), "memset") ||
        !ck(reads ? launch_merge_kmers(f->g, reads, nreads, read_len, k, f->merge_h, f->merge_c,
                                       merged_ptr(f), st)
                  : launch_merge_tiles(f->g, keys, n, key_is_hash, f->merge_h, f->merge_c, merged_ptr(f),
                                       status_ptr(f), st), "merge_tiles") ||
        !ck(launch_partition_counted(f->g, p, f->merge_h, f->merge_c, n, merged_ptr(f), 1, status_ptr(f), st),
            "partition") ||
        !ck(launch_merge_regions(p, st, merged_ptr(f), n), "merge_regions"))
      return -1;
  }
  {
    PhaseTimer t(f, GQF_PROF_INSERT, st, n);
    if (!ck(launch_rebuild(f->g, p, Op::kInsert, f->dqf, status_ptr(f), st, sparse_max_for(f, n)), "rebuild"))
      return -1;
  }
  return 0;
}

int do_bulk(HostFilter* f, uint64_t n, const uint64_t* keys, uint8_t flags, Op op, cudaStream_t st) {
  std::lock_guard<std::mutex> lk(f->mu);
  if (n == 0) return 0;
  if (!keys) {
    set_err("null keys");
    return -1;
  }
  if (!ensure_partition(f, n, false, st)) return -1;
  Partition p = f->part;
  p.counts = nullptr;
  const int key_is_hash = (flags & QF_KEY_IS_HASH) ? 1 : 0;
  {
    PhaseTimer t(f, GQF_PROF_PARTITION, st, n);
    if (!ck(launch_partition(f->g, p, keys, n, key_is_hash, status_ptr(f), st), "partition")) return -1;
  }
  {
    PhaseTimer t(f, op == Op::kDelete ? GQF_PROF_DELETE : GQF_PROF_INSERT, st, n);
    if (!ck(launch_rebuild(f->g, p, op, f->dqf, status_ptr(f), st, sparse_max_for(f, n)), "rebuild")) return -1;
  }
  return 0;
}

}  // namespace

namespace gqf {
// Read-only view of a filter for entry points defined in other translation
// units of this library.
bool internal_view(const QF* qf, FilterView* v) {
  HostFilter* f = lookup(qf);
  if (!f) return false;
  v->g = f->g;
  v->dqf = f->dqf;
  v->status = status_ptr(f);
  v->stats = stats_ptr(f);
  v->log_region = f->log_region;
  v->nregions = nregions_for(f, f->log_region);
  v->stream = f->stream;
  v->mu = &f->mu;
  v->device = f->device;
  return true;
}

uint32_t internal_sparse_max(const QF* qf, uint64_t n) {
  HostFilter* f = lookup(qf);
  return f ? sparse_max_for(f, n) : kDefaultSparseMax;
}

void internal_set_error(const char* msg) { set_err(msg); }
}  // namespace gqf

extern "C" {

const char* gqf_last_error(void) { return g_err.c_str(); }
const char* gqf_version(void) { return "gqf_gb300 0.1 (sm_103a)"; }

}  // extern "C"

namespace {
// Sizes the table of a 2^nbits-slot filter into h (qf_init, src/gqf.cu:
// 1939-1996, for qf_malloc_device's parameters) and allocates its zeroed
// blocks and locks; on failure nothing stays allocated.
bool alloc_table(quotient_filter& h, int nbits) {
  h.nslots = 1ULL << nbits;
  // qf_init (src/gqf.cu:1950-1951): xnslots = nslots + 10 sqrt(nslots)
  h.xnslots = h.nslots + (uint64_t)(10 * std::sqrt((double)h.nslots));
  h.nblocks = (h.xnslots + 63) / 64;
  h.range = h.nslots << 8;
  h.nbits = (uint32_t)nbits;
  h.key_bits = (uint32_t)nbits + 8;
  h.nlocks = h.xnslots / kLockRegion + 2;  // num_locks, src/gqf.cu:1996
  h.blocks = nullptr;
  h.locks = nullptr;
  const bool ok = ck(cudaMalloc((void**)&h.blocks, h.nblocks * sizeof(Block)), "cudaMalloc blocks") &&
                  ck(cudaMemset(h.blocks, 0, h.nblocks * sizeof(Block)), "cudaMemset blocks") &&
                  ck(cudaMalloc((void**)&h.locks, h.nlocks * kLockStride * sizeof(uint32_t)), "cudaMalloc locks") &&
                  ck(cudaMemset(h.locks, 0, h.nlocks * kLockStride * sizeof(uint32_t)), "cudaMemset locks");
  if (!ok) {
    if (h.blocks) cudaFree(h.blocks);
    if (h.locks) cudaFree(h.locks);
    h.blocks = nullptr;
    h.locks = nullptr;
  }
  return ok;
}

void set_geometry(HostFilter* f) {
  const quotient_filter& h = f->h;
  f->g.blocks = h.blocks;
  f->g.nslots = h.nslots;
  f->g.xnslots = h.xnslots;
  f->g.nblocks = h.nblocks;
  f->g.range = h.range;
  f->g.mask = h.range - 1;
  f->g.nbits = h.nbits;
}
}  // namespace

extern "C" {

void qf_malloc_device(QF** qf, int nbits, bool bulk_config) {
  (void)bulk_config;
  if (!qf) return;
  *qf = nullptr;
  if (nbits < 6 || nbits > 36) {
    set_err("nbits must be in [6, 36]");
    return;
  }
  HostFilter* f = new HostFilter();
  quotient_filter& h = f->h;
  h.lock_spin_limit = 1u << 20;
  f->device = current_device();
  bool ok = alloc_table(h, nbits) &&
            ck(cudaMalloc((void**)&f->aux, 256), "cudaMalloc aux") &&
            ck(cudaMemset(f->aux, 0, 256), "cudaMemset aux");
  if (ok) {
    h.status = status_ptr(f);
    ok = ck(cudaMalloc((void**)&f->dqf, sizeof(quotient_filter)), "cudaMalloc descriptor") &&
         ck(cudaMemcpy(f->dqf, &h, sizeof(quotient_filter), cudaMemcpyHostToDevice), "cudaMemcpy descriptor");
  }
  if (!ok) {
    if (h.blocks) cudaFree(h.blocks);
    if (h.locks) cudaFree(h.locks);
    if (f->aux) cudaFree(f->aux);
    if (f->dqf) cudaFree(f->dqf);
    delete f;
    return;
  }
  set_geometry(f);
  f->log_region = auto_log_region(nbits);
  {
    std::lock_guard<std::mutex> lk(g_mu);
    g_filters[f->dqf] = f;
  }
  *qf = f->dqf;
}

void qf_destroy_device(QF* qf) {
  HostFilter* f = lookup(qf);
  if (!f) return;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    g_filters.erase(qf);
  }
  cudaStreamSynchronize(f->stream);
  cudaDeviceSynchronize();
  for (auto& v : f->pending)
    for (auto& pr : v) { cudaEventDestroy(pr.first); cudaEventDestroy(pr.second); }
  for (cudaEvent_t e : f->spare) cudaEventDestroy(e);
  if (f->part.keys) cudaFree(f->part.keys);
  if (f->part.counts) cudaFree(f->part.counts);
  if (f->merge_h) cudaFree(f->merge_h);
  if (f->merge_c) cudaFree(f->merge_c);
  if (f->part.region_count) cudaFree(f->part.region_count);
  if (f->part.stage) cudaFree(f->part.stage);
  if (f->part.stage_counts) cudaFree(f->part.stage_counts);
  if (f->part.tiles) cudaFree(f->part.tiles);
  if (f->packed) cudaFree(f->packed);
  cudaFree(f->h.blocks);
  cudaFree(f->h.locks);
  cudaFree(f->aux);
  cudaFree(f->dqf);
  delete f;
}

void bulk_insert(QF* qf, uint64_t nvals, uint64_t* keys, uint8_t flags) {
  if (HostFilter* f = lookup(qf)) do_bulk(f, nvals, keys, flags, Op::kInsert, f->stream);
}

// Equal hashes are merged in shared-memory tables instead of the reference's
// sort + reduce_by_key (src/gqf.cu:3261-3279); the counted rebuild then adds
// each distinct hash once with its multiplicity.
void bulk_insert_reduce(QF* qf, uint64_t nvals, uint64_t* keys, uint8_t flags) {
  if (HostFilter* f = lookup(qf)) do_bulk_reduce(f, nvals, keys, flags, f->stream);
}

void bulk_delete(QF* qf, uint64_t nvals, uint64_t* keys, uint8_t flags) {
  if (HostFilter* f = lookup(qf)) do_bulk(f, nvals, keys, flags, Op::kDelete, f->stream);
}

void bulk_get(QF* qf, uint64_t nvals, uint64_t* vals, uint64_t* returns) {
  HostFilter* f = lookup(qf);
  if (!f) return;
  std::lock_guard<std::mutex> lk(f->mu);
  PhaseTimer t(f, GQF_PROF_GET, f->stream, nvals);
  ck(launch_bulk_get(f->g, vals, nvals, returns, 0, f->stream), "bulk_get");
}

uint64_t bulk_get_misses_wrapper(QF* qf, uint64_t* vals, uint64_t nvals) {
  HostFilter* f = lookup(qf);
  if (!f) return 0;
  std::lock_guard<std::mutex> lk(f->mu);
  unsigned long long m = 0;
  if (ck(cudaMemsetAsync(misses_ptr(f), 0, 8, f->stream), "memset") &&
      ck(launch_bulk_get_misses(f->g, vals, nvals, misses_ptr(f), f->stream), "bulk_get_misses") &&
      ck(cudaMemcpyAsync(&m, misses_ptr(f), 8, cudaMemcpyDeviceToHost, f->stream), "memcpy") &&
      ck(cudaStreamSynchronize(f->stream), "sync"))
    return m;
  return 0;
}

uint64_t point_get_wrapper(QF* qf, uint64_t* hashes, uint64_t nitems) {
  HostFilter* f = lookup(qf);
  if (!f) return 0;
  std::lock_guard<std::mutex> lk(f->mu);
  unsigned long long m = 0;
  if (ck(cudaMemsetAsync(misses_ptr(f), 0, 8, f->stream), "memset") &&
      ck(launch_point_get_misses(f->dqf, hashes, nitems, misses_ptr(f), f->stream), "point_get") &&
      ck(cudaMemcpyAsync(&m, misses_ptr(f), 8, cudaMemcpyDeviceToHost, f->stream), "memcpy") &&
      ck(cudaStreamSynchronize(f->stream), "sync"))
    return m;
  return 0;
}

int gqf_point_bulk_insert(QF* qf, uint64_t* keys, uint64_t nitems) {
  HostFilter* f = lookup(qf);
  if (!f) return -1;
  return ck(launch_point_bulk_insert(f->dqf, keys, nitems, f->stream), "point_bulk_insert") ? 0 : -1;
}

int gqf_point_insert_batch(QF* qf, const uint64_t* keys, uint64_t n, uint8_t flags, int8_t* rets) {
  HostFilter* f = lookup(qf);
  if (!f) return -1;
  return ck(launch_point_insert(f->dqf, keys, n, flags, rets, f->stream), "point_insert") ? 0 : -1;
}

int gqf_point_insert_not_exists_batch(QF* qf, const uint64_t* keys, uint64_t n, uint8_t flags,
                                      int8_t* rets, uint8_t* vals) {
  HostFilter* f = lookup(qf);
  if (!f) return -1;
  return ck(launch_point_insert_not_exists(f->dqf, keys, n, flags, rets, vals, f->stream),
            "point_insert_not_exists") ? 0 : -1;
}

int gqf_point_query_batch(QF* qf, const uint64_t* keys, uint64_t n, uint8_t flags, int concurrent,
                          uint64_t* counts) {
  HostFilter* f = lookup(qf);
  if (!f) return -1;
  return ck(launch_point_query(f->dqf, keys, n, flags, concurrent, counts, f->stream), "point_query") ? 0 : -1;
}

int gqf_bulk_insert_async(QF* qf, uint64_t nvals, const uint64_t* keys, uint8_t flags, void* stream) {
  HostFilter* f = lookup(qf);
  return f ? do_bulk(f, nvals, keys, flags, Op::kInsert, (cudaStream_t)stream) : -1;
}

int gqf_bulk_insert_reduce_async(QF* qf, uint64_t nvals, const uint64_t* keys, uint8_t flags,
                                 void* stream) {
  HostFilter* f = lookup(qf);
  return f ? do_bulk_reduce(f, nvals, keys, flags, (cudaStream_t)stream) : -1;
}

int gqf_bulk_insert_kmers(QF* qf, const uint8_t* reads, uint64_t nreads, uint32_t read_len, uint32_t k,
                          void* stream) {
  HostFilter* f = lookup(qf);
  if (!f) return -1;
  if (!reads && nreads) {
    set_err("null reads");
    return -1;
  }
  return do_bulk_reduce(f, 0, nullptr, 0, (cudaStream_t)stream, reads, nreads, read_len, k);
}

int gqf_kmers_extract(const uint8_t* reads, uint64_t nreads, uint32_t read_len, uint32_t k, uint64_t* out,
                      void* stream) {
  if (!kmer_shape_ok(nreads, read_len, k)) {
    set_err("k-mers: need 1 <= k <= 32 and k <= read_len <= k + 4095");
    return -1;
  }
  if (nreads && (!reads || !out)) {
    set_err("null reads or output");
    return -1;
  }
  return ck(launch_kmers(reads, nreads, read_len, k, out, (cudaStream_t)stream), "kmers") ? 0 : -1;
}

int gqf_bulk_delete_async(QF* qf, uint64_t nvals, const uint64_t* keys, uint8_t flags, void* stream) {
  HostFilter* f = lookup(qf);
  return f ? do_bulk(f, nvals, keys, flags, Op::kDelete, (cudaStream_t)stream) : -1;
}

int gqf_bulk_get_async(QF* qf, uint64_t nvals, const uint64_t* vals, uint64_t* returns, uint8_t flags,
                       void* stream) {
  HostFilter* f = lookup(qf);
  if (!f) return -1;
  std::lock_guard<std::mutex> lk(f->mu);
  PhaseTimer t(f, GQF_PROF_GET, (cudaStream_t)stream, nvals);
  return ck(launch_bulk_get(f->g, vals, nvals, returns, (flags & QF_KEY_IS_HASH) ? 1 : 0,
                            (cudaStream_t)stream), "bulk_get") ? 0 : -1;
}

int gqf_set_stream(QF* qf, void* stream) {
  HostFilter* f = lookup(qf);
  if (!f) return -1;
  f->stream = (cudaStream_t)stream;
  return 0;
}

int gqf_set_region_log(QF* qf, int log_region) {
  HostFilter* f = lookup(qf);
  if (!f) return -1;
  std::lock_guard<std::mutex> lk(f->mu);
  if (log_region == 0) {
    f->auto_region = true;
    f->log_region = auto_log_region((int)f->h.nbits);
    return 0;
  }
  if (log_region < kMinLogRegion || log_region > kMaxLogRegion) {
    set_err("log_region must be 11, 12 or 13");
    return -1;
  }
  f->auto_region = false;
  f->log_region = log_region;
  return 0;
}

int gqf_set_sparse_max(QF* qf, uint32_t max_keys) {
  HostFilter* f = lookup(qf);
  if (!f) return -1;
  std::lock_guard<std::mutex> lk(f->mu);
  f->sparse_max = max_keys;
  return 0;
}

int64_t gqf_get_sparse_max(QF* qf) {
  HostFilter* f = lookup(qf);
  return f ? (int64_t)sparse_max_of(f) : -1;
}

int gqf_get_region_log(QF* qf) {
  HostFilter* f = lookup(qf);
  return f ? f->log_region : -1;
}

uint64_t gqf_nslots(QF* qf) { HostFilter* f = lookup(qf); return f ? f->h.nslots : 0; }
uint64_t gqf_xnslots(QF* qf) { HostFilter* f = lookup(qf); return f ? f->h.xnslots : 0; }
uint64_t gqf_nblocks(QF* qf) { HostFilter* f = lookup(qf); return f ? f->h.nblocks : 0; }
uint64_t gqf_device_bytes(QF* qf) {
  HostFilter* f = lookup(qf);
  return f ? f->h.nblocks * sizeof(Block) : 0;
}

int gqf_get_status(QF* qf, uint32_t* status) {
  HostFilter* f = lookup(qf);
  if (!f || !status) return -1;
  uint32_t s = 0;
  if (!ck(cudaMemcpyAsync(&s, status_ptr(f), 4, cudaMemcpyDeviceToHost, f->stream), "memcpy status") ||
      !ck(cudaStreamSynchronize(f->stream), "sync"))
    return -1;
  *status = s;
  return 0;
}

int gqf_clear_status(QF* qf) {
  HostFilter* f = lookup(qf);
  if (!f) return -1;
  return ck(cudaMemsetAsync(status_ptr(f), 0, 4, f->stream), "memset status") &&
         ck(cudaMemsetAsync(stats_ptr(f), 0, 24, f->stream), "memset counters") ? 0 : -1;
}

int gqf_get_counters(QF* qf, uint64_t* counters, int n) {
  HostFilter* f = lookup(qf);
  if (!f || !counters || n < 0) return -1;
  unsigned long long c[3] = {0, 0, 0};
  if (!ck(cudaMemcpyAsync(c, stats_ptr(f), 24, cudaMemcpyDeviceToHost, f->stream), "memcpy counters") ||
      !ck(cudaStreamSynchronize(f->stream), "sync"))
    return -1;
  for (int i = 0; i < n && i < 3; i++) counters[i] = c[i];
  return 0;
}

int gqf_set_lock_wait(QF* qf, uint32_t max_spins) {
  HostFilter* f = lookup(qf);
  if (!f) return -1;
  if (max_spins == 0) {
    set_err("gqf_set_lock_wait: at least one attempt");
    return -1;
  }
  std::lock_guard<std::mutex> lk(f->mu);
  f->h.lock_spin_limit = max_spins;
  return ck(cudaMemcpy(reinterpret_cast<uint8_t*>(f->dqf) + offsetof(quotient_filter, lock_spin_limit),
                       &f->h.lock_spin_limit, sizeof(uint32_t), cudaMemcpyHostToDevice),
            "cudaMemcpy")
             ? 0
             : -1;
}

int gqf_debug_hold_lock(QF* qf, uint64_t lock_index, int held) {
  HostFilter* f = lookup(qf);
  if (!f) return -1;
  if (lock_index >= f->h.nlocks) {
    set_err("gqf_debug_hold_lock: no such lock");
    return -1;
  }
  const uint32_t v = held ? 1u : 0u;
  return ck(cudaMemcpy(f->h.locks + lock_index * kLockStride, &v, sizeof v, cudaMemcpyHostToDevice), "cudaMemcpy")
             ? 0
             : -1;
}

int gqf_reset(QF* qf) {
  HostFilter* f = lookup(qf);
  if (!f) return -1;
  return ck(cudaMemsetAsync(f->h.blocks, 0, f->h.nblocks * sizeof(Block), f->stream), "memset blocks") ? 0 : -1;
}

uint64_t gqf_export_size(QF* qf) {
  HostFilter* f = lookup(qf);
  return f ? 120 + f->h.nblocks * 81 : 0;
}

namespace {
// qfmetadata (include/gqf_int.cuh:96-113) as qf_init fills it for
// qf_malloc_device's parameters (src/gqf.cu:1978-1994); the element counters
// stay 0, as in the reference, which never updates them on the device.
void fill_metadata(const HostFilter* f, uint8_t* out) {
  uint64_t w[15] = {0};
  w[0] = 1018874902021329732ULL;            // MAGIC_NUMBER
  w[1] = (uint64_t)QF_HASH_INVERTIBLE;      // hash_mode (int) | reserved (0)
  w[2] = f->h.nblocks * 81;                 // total_size_in_bytes
  w[3] = 0;                                 // seed | padding
  w[4] = f->h.nslots;
  w[5] = f->h.xnslots;
  w[6] = f->h.key_bits;
  w[7] = 0;                                 // value_bits
  w[8] = 8;                                 // key_remainder_bits
  w[9] = 8;                                 // bits_per_slot
  w[10] = f->h.range;
  w[11] = f->h.nblocks;
  std::memcpy(out, w, 120);
}

bool ensure_packed(HostFilter* f) {
  if (f->packed) return true;
  return ck(cudaMalloc((void**)&f->packed, f->h.nblocks * 81), "cudaMalloc packed");
}
}  // namespace

int gqf_export(QF* qf, void* host_buf, uint64_t len) {
  HostFilter* f = lookup(qf);
  if (!f) return -1;
  std::lock_guard<std::mutex> lk(f->mu);
  uint64_t need = 120 + f->h.nblocks * 81;
  if (!host_buf || len < need) {
    set_err("export buffer too small");
    return -1;
  }
  if (!ensure_packed(f)) return -1;
  uint8_t* out = static_cast<uint8_t*>(host_buf);
  fill_metadata(f, out);
  if (!ck(launch_export(f->g, f->packed, f->stream), "export") ||
      !ck(cudaMemcpyAsync(out + 120, f->packed, f->h.nblocks * 81, cudaMemcpyDeviceToHost, f->stream), "memcpy") ||
      !ck(cudaStreamSynchronize(f->stream), "sync"))
    return -1;
  return 0;
}

int gqf_import(QF* qf, const void* host_buf, uint64_t len) {
  HostFilter* f = lookup(qf);
  if (!f) return -1;
  std::lock_guard<std::mutex> lk(f->mu);
  uint64_t need = 120 + f->h.nblocks * 81;
  if (!host_buf || len != need) {
    set_err("import image size does not match this filter");
    return -1;
  }
  uint8_t meta[120];
  fill_metadata(f, meta);
  const uint8_t* in = static_cast<const uint8_t*>(host_buf);
  // nslots, xnslots, key_bits, nblocks must agree
  if (std::memcmp(in + 32, meta + 32, 24) != 0 || std::memcmp(in + 88, meta + 88, 8) != 0) {
    set_err("import image geometry does not match this filter");
    return -1;
  }
  if (!ensure_packed(f)) return -1;
  if (!ck(cudaMemcpyAsync(f->packed, in + 120, f->h.nblocks * 81, cudaMemcpyHostToDevice, f->stream), "memcpy") ||
      !ck(launch_import(f->g, f->packed, f->stream), "import") ||
      !ck(launch_import_fix(f->dqf, f->packed, f->stream), "import_fix") ||
      !ck(cudaStreamSynchronize(f->stream), "sync"))
    return -1;
  return 0;
}

uint64_t gqf_serialize(QF* qf, const char* path) {
  HostFilter* f = lookup(qf);
  if (!f || !path) return 0;
  std::vector<uint8_t> img(120 + f->h.nblocks * 81);
  if (gqf_export(qf, img.data(), img.size()) != 0) return 0;
  FILE* fh = std::fopen(path, "wb");
  if (!fh) {
    set_err(std::string("gqf_serialize: cannot open ") + path);
    return 0;
  }
  const size_t w = std::fwrite(img.data(), 1, img.size(), fh);
  const bool good = std::fclose(fh) == 0 && w == img.size();
  if (!good) set_err(std::string("gqf_serialize: short write to ") + path);
  return good ? (uint64_t)w : 0;
}

uint64_t gqf_deserialize(QF** out, const char* path) {
  if (!out || !path) return 0;
  *out = nullptr;
  FILE* fh = std::fopen(path, "rb");
  if (!fh) {
    set_err(std::string("gqf_deserialize: cannot open ") + path);
    return 0;
  }
  uint64_t meta[15] = {0};
  if (std::fread(meta, 1, 120, fh) != 120 || meta[0] != 1018874902021329732ULL || meta[9] != 8 ||
      meta[4] == 0 || (meta[4] & (meta[4] - 1)) != 0) {
    std::fclose(fh);
    set_err("gqf_deserialize: not a filter image with 8-bit slots");
    return 0;
  }
  int nbits = 0;
  while ((1ULL << nbits) < meta[4]) nbits++;
  std::vector<uint8_t> img(120 + 81 * meta[11]);
  std::memcpy(img.data(), meta, 120);
  const size_t r = std::fread(img.data() + 120, 1, img.size() - 120, fh);
  std::fclose(fh);
  if (r != img.size() - 120) {
    set_err("gqf_deserialize: truncated image");
    return 0;
  }
  QF* q = nullptr;
  qf_malloc_device(&q, nbits, true);
  if (!q) return 0;
  if (gqf_import(q, img.data(), img.size()) != 0) {
    qf_destroy_device(q);
    return 0;
  }
  *out = q;
  return img.size();
}

int gqf_profile(QF* qf, int enable) {
  HostFilter* f = lookup(qf);
  if (!f) return -1;
  std::lock_guard<std::mutex> lk(f->mu);
  f->prof = enable != 0;
  for (int i = 0; i < GQF_PROF_PHASES; i++) { f->prof_ms[i] = 0; f->prof_calls[i] = 0; f->prof_keys[i] = 0; }
  return 0;
}

int gqf_profile_read(QF* qf, double* ms, uint64_t* calls, uint64_t* keys) {
  HostFilter* f = lookup(qf);
  if (!f) return -1;
  std::lock_guard<std::mutex> lk(f->mu);
  for (int i = 0; i < GQF_PROF_PHASES; i++) {
    for (auto& pr : f->pending[i]) {
      float t = 0;
      if (!ck(cudaEventSynchronize(pr.second), "event sync")) return -1;
      cudaEventElapsedTime(&t, pr.first, pr.second);
      f->prof_ms[i] += t;
      f->spare.push_back(pr.first);
      f->spare.push_back(pr.second);
    }
    f->pending[i].clear();
    if (ms) ms[i] = f->prof_ms[i];
    if (calls) calls[i] = f->prof_calls[i];
    if (keys) keys[i] = f->prof_keys[i];
  }
  return 0;
}


// ------------------------------------------------------------- enumeration

namespace {

// Counts f's pairs per block and scans them into *start (device, allocated
// here on `st`; the caller frees it).  Returns the total, or UINT64_MAX.
uint64_t enum_prepare(HostFilter* f, cudaStream_t st, uint32_t** start) {
  const uint64_t nb = f->h.nblocks;
  *start = nullptr;
  if (64 * nb >= (1ULL << 32)) {
    set_err("enumeration supports tables of at most 2^31 slots");
    return UINT64_MAX;
  }
  uint32_t* buf = nullptr;  // cnt[nb] | start[nb + 1] | cursor[nb] | scan scratch
  const uint64_t words = 3 * nb + 1 + nb / 4096 + 4;
  if (!ck(cudaMallocAsync((void**)&buf, words * sizeof(uint32_t), st), "cudaMallocAsync")) return UINT64_MAX;
  Partition tp{};
  tp.region_count = buf;
  tp.region_start = buf + nb;
  tp.cursor = buf + 2 * nb + 1;
  tp.deferred = buf + 3 * nb + 1;
  tp.nregions = (uint32_t)nb;
  uint32_t total = 0;
  if (!ck(launch_enum_count(f->g, tp.region_count, st), "enumerate") || !ck(launch_region_scan(tp, st), "scan") ||
      !ck(cudaMemcpyAsync(&total, tp.region_start + nb, 4, cudaMemcpyDeviceToHost, st), "memcpy") ||
      !ck(cudaStreamSynchronize(st), "sync")) {
    cudaFreeAsync(buf, st);
    return UINT64_MAX;
  }
  *start = buf;  // the counts come first; the starts follow at buf + nb
  return total;
}

// Inserts (hash, count) pairs into f with the counted rebuild (or (key,
// count) pairs, hashed for f, when key_is_hash is 0).
int insert_pairs(HostFilter* f, const uint64_t* h, const uint32_t* c, uint64_t n, cudaStream_t st,
                 int key_is_hash = 1) {
  std::lock_guard<std::mutex> lk(f->mu);
  if (n == 0) return 0;
  if (!ensure_partition(f, n, true, st)) return -1;
  Partition p = f->part;
  if (!ck(launch_partition_counted(f->g, p, h, c, n, nullptr, key_is_hash, status_ptr(f), st), "partition") ||
      !ck(launch_merge_regions(p, st), "merge_regions") ||
      !ck(launch_rebuild(f->g, p, Op::kInsert, f->dqf, status_ptr(f), st, sparse_max_for(f, n)), "rebuild"))
    return -1;
  return 0;
}

// The pairs of several filters, concatenated, as hashes (or keys, with
// as_keys) and uint32 counts in one device allocation (freed by the caller);
// *n gets the total.
bool collect_pairs(std::vector<HostFilter*> fs, cudaStream_t st, uint64_t** h, uint32_t** c, uint64_t* n,
                   int as_keys = 0) {
  std::vector<uint32_t*> starts;
  std::vector<uint64_t> counts;
  uint64_t total = 0;
  bool good = true;
  for (HostFilter* f : fs) {
    uint32_t* st_buf = nullptr;
    const uint64_t k = enum_prepare(f, st, &st_buf);
    if (k == UINT64_MAX) {
      good = false;
      break;
    }
    starts.push_back(st_buf);
    counts.push_back(k);
    total += k;
  }
  *h = nullptr;
  *c = nullptr;
  uint32_t* flag = nullptr;
  if (good)
    good = ck(cudaMallocAsync((void**)h, (total ? total : 1) * 8, st), "cudaMallocAsync") &&
           ck(cudaMallocAsync((void**)c, (total ? total : 1) * 4, st), "cudaMallocAsync") &&
           ck(cudaMallocAsync((void**)&flag, 4, st), "cudaMallocAsync") && ck(cudaMemsetAsync(flag, 0, 4, st), "memset");
  uint64_t at = 0;
  for (size_t i = 0; good && i < starts.size(); i++) {
    good = ck(launch_enum_write(fs[i]->g, starts[i] + fs[i]->h.nblocks, as_keys, *h + at, nullptr, *c + at, flag,
                                st),
              "enumerate");
    at += counts[i];
  }
  uint32_t over = 0;
  if (good)
    good = ck(cudaMemcpyAsync(&over, flag, 4, cudaMemcpyDeviceToHost, st), "memcpy") &&
           ck(cudaStreamSynchronize(st), "sync");
  if (good && over) {
    set_err("a counter above 2^32 - 1 cannot be carried by this operation");
    good = false;
  }
  for (uint32_t* b : starts) cudaFreeAsync(b, st);
  if (flag) cudaFreeAsync(flag, st);
  if (!good) {
    if (*h) cudaFreeAsync(*h, st);
    if (*c) cudaFreeAsync(*c, st);
    *h = nullptr;
    *c = nullptr;
    return false;
  }
  *n = total;
  return true;
}

// The reference iterates the larger filter and probes the smaller
// (qf_inner_product / qf_intersect, src/gqf.cu:4010-4080): "larger" by table
// bytes, ties to the second filter.
void disk_and_mem(HostFilter* a, HostFilter* b, HostFilter** disk, HostFilter** mem) {
  if (a->h.nblocks > b->h.nblocks) {
    *disk = a;
    *mem = b;
  } else {
    *disk = b;
    *mem = a;
  }
}

}  // namespace

int gqf_enumerate(QF* qf, uint64_t* hashes, uint64_t* counts, uint64_t cap, uint64_t* n, int as_keys) {
  HostFilter* f = lookup(qf);
  if (!f) return -1;
  cudaStream_t st = 0;
  uint32_t* buf = nullptr;
  const uint64_t total = enum_prepare(f, st, &buf);
  if (total == UINT64_MAX) return -1;
  if (n) *n = total;
  int rc = 0;
  if (hashes) {
    if (total > cap) {
      set_err("gqf_enumerate: output holds fewer pairs than the filter has (see *n)");
      rc = -1;
    } else if (!ck(launch_enum_write(f->g, buf + f->h.nblocks, as_keys, hashes, counts, nullptr, nullptr, st),
                   "enumerate") || !ck(cudaStreamSynchronize(st), "sync")) {
      rc = -1;
    }
  }
  cudaFreeAsync(buf, st);
  cudaStreamSynchronize(st);
  return rc;
}

int gqf_multi_merge(QF* const* in, int nin, QF* out) {
  HostFilter* r = lookup(out);
  if (!r || nin < 0 || (nin && !in)) return -1;
  std::vector<HostFilter*> fs;
  for (int i = 0; i < nin; i++) {
    HostFilter* f = lookup(in[i]);
    if (!f) return -1;
    fs.push_back(f);
  }
  cudaStream_t st = 0;
  uint64_t* h = nullptr;
  uint32_t* c = nullptr;
  uint64_t n = 0;
  if (!collect_pairs(fs, st, &h, &c, &n)) return -1;  // every input read before the output changes
  const int rc = insert_pairs(r, h, c, n, st);
  cudaFreeAsync(h, st);
  cudaFreeAsync(c, st);
  return ck(cudaStreamSynchronize(st), "sync") ? rc : -1;
}

// Grows the table under the same handle: every stored key (the inverse hash
// of each stored hash, the key modulo 2^(nbits + 8)) with its count goes
// into a 2^new_nbits-slot table, hashed over new_nbits + 8 bits.
int gqf_resize(QF* qf, int new_nbits) {
  HostFilter* f = lookup(qf);
  if (!f) return -1;
  if (new_nbits < (int)f->h.nbits || new_nbits > 36) {
    set_err("gqf_resize: new_nbits must lie in [nbits, 36]");
    return -1;
  }
  if (new_nbits == (int)f->h.nbits) return 0;
  if (!ck(cudaStreamSynchronize(f->stream), "sync")) return -1;
  cudaStream_t st = 0;
  uint64_t* keys = nullptr;
  uint32_t* c = nullptr;
  uint64_t n = 0;
  if (!collect_pairs({f}, st, &keys, &c, &n, 1)) return -1;
  bool ok = ck(cudaStreamSynchronize(st), "sync");
  if (ok) {
    std::lock_guard<std::mutex> lk(f->mu);
    quotient_filter nh = f->h;
    ok = alloc_table(nh, new_nbits);
    if (ok) {
      cudaFree(f->h.blocks);
      cudaFree(f->h.locks);
      if (f->packed) cudaFree(f->packed);
      f->packed = nullptr;
      f->h = nh;
      set_geometry(f);
      if (f->auto_region) f->log_region = auto_log_region(new_nbits);
      ok = ck(cudaMemcpy(f->dqf, &f->h, sizeof(quotient_filter), cudaMemcpyHostToDevice), "cudaMemcpy descriptor");
    }
  }
  int rc = ok ? insert_pairs(f, keys, c, n, st, 0) : -1;
  cudaFreeAsync(keys, st);
  cudaFreeAsync(c, st);
  if (!ck(cudaStreamSynchronize(st), "sync")) rc = -1;
  return rc;
}

int gqf_merge(QF* a, QF* b, QF* out) {
  QF* in[2] = {a, b};
  return gqf_multi_merge(in, 2, out);
}

int gqf_intersect(QF* a, QF* b, QF* out) {
  HostFilter *fa = lookup(a), *fb = lookup(b), *fr = lookup(out);
  if (!fa || !fb || !fr) return -1;
  HostFilter *disk, *mem;
  disk_and_mem(fa, fb, &disk, &mem);
  cudaStream_t st = 0;
  uint32_t* buf = nullptr;
  const uint64_t total = enum_prepare(disk, st, &buf);
  if (total == UINT64_MAX) return -1;
  uint64_t *h = nullptr, *cc = nullptr, *kh = nullptr;
  uint32_t *kc = nullptr, *flag = nullptr;
  unsigned long long* nk = nullptr;
  unsigned long long kept = 0;
  uint32_t over = 0;
  const uint64_t m = total ? total : 1;
  bool good = ck(cudaMallocAsync((void**)&h, m * 8, st), "cudaMallocAsync") &&
              ck(cudaMallocAsync((void**)&cc, m * 8, st), "cudaMallocAsync") &&
              ck(cudaMallocAsync((void**)&kh, m * 8, st), "cudaMallocAsync") &&
              ck(cudaMallocAsync((void**)&kc, m * 4, st), "cudaMallocAsync") &&
              ck(cudaMallocAsync((void**)&flag, 16, st), "cudaMallocAsync") &&
              ck(cudaMemsetAsync(flag, 0, 16, st), "memset");
  nk = reinterpret_cast<unsigned long long*>(flag + 2);
  good = good && ck(launch_enum_write(disk->g, buf + disk->h.nblocks, 0, h, cc, nullptr, nullptr, st), "enumerate") &&
         ck(launch_pair_probe(mem->g, h, cc, total, nullptr, kh, kc, nk, flag, st), "probe") &&
         ck(cudaMemcpyAsync(&kept, nk, 8, cudaMemcpyDeviceToHost, st), "memcpy") &&
         ck(cudaMemcpyAsync(&over, flag, 4, cudaMemcpyDeviceToHost, st), "memcpy") &&
         ck(cudaStreamSynchronize(st), "sync");
  if (good && over) {
    set_err("a counter above 2^32 - 1 cannot be carried by this operation");
    good = false;
  }
  int rc = good ? insert_pairs(fr, kh, kc, kept, st) : -1;
  for (void* p : {(void*)buf, (void*)h, (void*)cc, (void*)kh, (void*)kc, (void*)flag})
    if (p) cudaFreeAsync(p, st);
  if (!ck(cudaStreamSynchronize(st), "sync")) rc = -1;
  return rc;
}

uint64_t gqf_inner_product(QF* a, QF* b) {
  HostFilter *fa = lookup(a), *fb = lookup(b);
  if (!fa || !fb) return 0;
  HostFilter *disk, *mem;
  disk_and_mem(fa, fb, &disk, &mem);
  cudaStream_t st = 0;
  uint32_t* buf = nullptr;
  const uint64_t total = enum_prepare(disk, st, &buf);
  if (total == UINT64_MAX) return 0;
  uint64_t *h = nullptr, *cc = nullptr;
  unsigned long long* acc = nullptr;
  unsigned long long out = 0;
  const uint64_t m = total ? total : 1;
  const bool good = ck(cudaMallocAsync((void**)&h, m * 8, st), "cudaMallocAsync") &&
                    ck(cudaMallocAsync((void**)&cc, m * 8, st), "cudaMallocAsync") &&
                    ck(cudaMallocAsync((void**)&acc, 8, st), "cudaMallocAsync") &&
                    ck(cudaMemsetAsync(acc, 0, 8, st), "memset") &&
                    ck(launch_enum_write(disk->g, buf + disk->h.nblocks, 0, h, cc, nullptr, nullptr, st),
                       "enumerate") &&
                    ck(launch_pair_probe(mem->g, h, cc, total, acc, nullptr, nullptr, nullptr, nullptr, st), "probe") &&
                    ck(cudaMemcpyAsync(&out, acc, 8, cudaMemcpyDeviceToHost, st), "memcpy") &&
                    ck(cudaStreamSynchronize(st), "sync");
  for (void* p : {(void*)buf, (void*)h, (void*)cc, (void*)acc})
    if (p) cudaFreeAsync(p, st);
  cudaStreamSynchronize(st);
  return good ? (uint64_t)out : 0;
}

uint64_t gqf_launch_count(void) { return g_launches.load(); }

int gqf_debug_serial_apply(QF* qf, const uint64_t* hashes, uint64_t n, int op) {
  HostFilter* f = lookup(qf);
  if (!f) return -1;
  return ck(launch_serial_apply(f->dqf, hashes, n, op, f->stream), "serial_apply") ? 0 : -1;
}

}  // extern "C"
