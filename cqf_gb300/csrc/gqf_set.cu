// Filter sets: many independent filters of uneven sizes served by one launch
// per phase.
//
// The reference has one filter per QF handle; serving thousands of small
// filters with it means thousands of qf_malloc_device / bulk_insert /
// bulk_get calls, each with its own allocation, host readback and launch
// sequence (src/gqf.cu:2123-2220, :3184-3400).  A set keeps all its filters'
// blocks in one device arena and numbers the regions of all filters one after
// another (FilterSet in gqf_kernels.cuh), so a batch spanning every filter is
// one partition pass, one rebuild launch per parity and one probe launch,
// whatever the number of filters.  Keys arrive as one array with CSR offsets
// (filter f owns keys[offsets[f] .. offsets[f+1])).  All scratch is sized at
// creation: the operations allocate nothing, so a sequence of them can be
// captured into a CUDA graph and replayed.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "gqf_probe.cuh"
#include "gqf_rebuild_impl.cuh"
#include "../../include/gqf.h"

using namespace gqf;

struct gqf_set {
  uint32_t n = 0;
  std::vector<quotient_filter> h;  // host mirrors of the descriptors
  quotient_filter* dqfs = nullptr;  // device descriptors
  Block* arena = nullptr;
  uint64_t arena_blocks = 0;
  uint8_t* aux = nullptr;           // status word @0, stats @128
  uint32_t* region_base = nullptr;  // device, n + 1
  uint32_t nregions = 0;
  uint32_t region_cap = 0;
  Partition part{};
  uint64_t key_cap = 0;
  int log_region = 11;
  uint32_t sparse_max = GQF_SPARSE_AUTO;
  std::string err;
};

namespace gqf {
namespace {

thread_local std::string g_set_err;

int fail(const std::string& m) {
  g_set_err = m;
  internal_set_error(m.c_str());
  return -1;
}

bool ok(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return true;
  fail(std::string(what) + ": " + cudaGetErrorString(e));
  return false;
}

int grid_for_keys(uint64_t n) {
  uint64_t want = (n + 255) / 256, cap = (uint64_t)sm_count() * 16;
  return (int)std::max<uint64_t>(1, std::min(want, cap));
}

// The filter of key i: lane 0 of each warp searches the offsets for the
// warp's first key, then every lane steps forward over the (rare) filter
// boundaries inside the warp's 32 keys.  offsets has n + 1 entries.
__device__ __forceinline__ uint32_t filter_of(const uint64_t* __restrict__ offsets, uint32_t n, uint64_t i,
                                             uint64_t warp_first) {
  uint32_t f = 0;
  if ((threadIdx.x & 31) == 0) {
    uint32_t lo = 0, hi = n;  // last f with offsets[f] <= warp_first
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (offsets[mid] <= warp_first) lo = mid;
      else hi = mid;
    }
    f = lo;
  }
  f = __shfl_sync(0xffffffffu, f, 0);
  while (f + 1 < n && offsets[f + 1] <= i) f++;
  return f;
}

// Hash of key i of filter f, or false (a QF_KEY_IS_HASH key out of range).
__device__ __forceinline__ bool set_hash(const quotient_filter& q, uint64_t k, int key_is_hash, uint64_t* h) {
  if (key_is_hash) {
    if (k >= q.range) return false;
    *h = k;
  } else {
    *h = hash64(k, q.range - 1);
  }
  return true;
}

template <bool SCATTER>
__global__ void __launch_bounds__(256) k_set_partition(const quotient_filter* __restrict__ qfs, uint32_t n,
                                                       const uint32_t* __restrict__ region_base,
                                                       const uint64_t* __restrict__ keys,
                                                       const uint64_t* __restrict__ offsets, uint64_t total,
                                                       int key_is_hash, int shift, uint32_t* region_count,
                                                       uint32_t* cursor, uint32_t* out, uint32_t* status) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t nr = (total + 31) & ~31ULL;
  const unsigned lane = threadIdx.x & 31;
  const uint64_t local_mask = (1ULL << shift) - 1ULL;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nr; i += stride) {
    const uint64_t first = i - lane;
    const uint32_t f = filter_of(offsets, n, i < total ? i : total - 1, first < total ? first : total - 1);
    uint64_t h = 0;
    bool valid = false;
    if (i < total) {
      valid = set_hash(qfs[f], __ldcs(keys + i), key_is_hash, &h);
      if (!valid && !SCATTER && status) atomicOr(status, kStBadKey);
    }
    const uint32_t R = valid ? region_base[f] + (uint32_t)(h >> shift) : 0xFFFFFFFFu;
    const unsigned peers = __match_any_sync(0xffffffffu, R);
    const unsigned leader = __ffs(peers) - 1;
    if (!SCATTER) {
      if (valid && lane == leader) atomicAdd(&region_count[R], (uint32_t)__popc(peers));
    } else {
      uint32_t base = 0;
      if (valid && lane == leader) base = atomicAdd(&cursor[R], (uint32_t)__popc(peers));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (valid) out[base + __popc(peers & ((1u << lane) - 1u))] = (uint32_t)(h & local_mask);
    }
  }
}

__global__ void __launch_bounds__(256) k_set_get(const quotient_filter* __restrict__ qfs, uint32_t n,
                                                 const uint64_t* __restrict__ keys,
                                                 const uint64_t* __restrict__ offsets, uint64_t total,
                                                 int key_is_hash, uint64_t* __restrict__ out) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t nr = (total + 31) & ~31ULL;
  const unsigned lane = threadIdx.x & 31;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nr; i += stride) {
    const uint64_t first = i - lane;
    const uint32_t f = filter_of(offsets, n, i < total ? i : total - 1, first < total ? first : total - 1);
    if (i >= total) continue;
    const quotient_filter& q = qfs[f];
    uint64_t h = 0;
    uint64_t c = 0;
    if (set_hash(q, __ldcs(keys + i), key_is_hash, &h)) c = probe(q.blocks, q.nblocks, h);
    __stcs(out + i, c);
  }
}

uint32_t regions_of(const quotient_filter& q, int log_region) {
  const uint64_t r = q.nslots >> log_region;
  return (uint32_t)(r ? r : 1);
}

// Numbers the regions of all filters for log_region (each filter's count
// rounded up to even) into the device table.
bool layout_regions(gqf_set* s, int log_region) {
  std::vector<uint32_t> base(s->n + 1, 0);
  uint64_t tot = 0;
  for (uint32_t f = 0; f < s->n; f++) {
    base[f] = (uint32_t)tot;
    tot += (regions_of(s->h[f], log_region) + 1) & ~1u;
  }
  if (tot + 2 > s->region_cap) {
    fail("filter set: region table too small");
    return false;
  }
  base[s->n] = (uint32_t)tot;
  if (!ok(cudaMemcpy(s->region_base, base.data(), base.size() * 4, cudaMemcpyHostToDevice), "cudaMemcpy"))
    return false;
  s->nregions = (uint32_t)tot;
  s->log_region = log_region;
  s->part.nregions = s->nregions;
  s->part.log_region = log_region;
  return true;
}

uint32_t set_sparse_for(const gqf_set* s, uint64_t n) {
  if (s->sparse_max != GQF_SPARSE_AUTO) return s->sparse_max;
  uint32_t t = s->nregions / 1400;
  t = t < 16 ? 16 : t > 256 ? 256 : t;
  return 2 * (n / std::max<uint32_t>(1, s->nregions)) <= t ? t : 0;
}

int set_update(gqf_set* s, const uint64_t* keys, const uint64_t* offsets, uint64_t total, uint8_t flags,
               Op op, cudaStream_t st) {
  if (!s) return fail("null filter set");
  if (total == 0) return 0;
  if (!keys || !offsets) return fail("filter set: null keys or offsets");
  if (total > s->key_cap) return fail("filter set: batch larger than the set's max_batch_keys");
  uint32_t* status = reinterpret_cast<uint32_t*>(s->aux);
  const int shift = 8 + s->log_region;
  Partition p = s->part;
  p.counts = nullptr;
  const int kih = (flags & QF_KEY_IS_HASH) ? 1 : 0;
  const int grid = grid_for_keys(total);
  if (!ok(cudaMemsetAsync(p.region_count, 0, (p.nregions + 1) * sizeof(uint32_t), st), "memset")) return -1;
  k_set_partition<false><<<grid, 256, 0, st>>>(s->dqfs, s->n, s->region_base, keys, offsets, total, kih, shift,
                                               p.region_count, p.cursor, p.keys, status);
  count_launch();
  if (!ok(launch_region_scan(p, st), "scan")) return -1;
  k_set_partition<true><<<grid, 256, 0, st>>>(s->dqfs, s->n, s->region_base, keys, offsets, total, kih, shift,
                                              p.region_count, p.cursor, p.keys, status);
  count_launch();
  FilterSet loc{s->dqfs, s->region_base, s->n};
  if (!ok(run_rebuild(loc, p, op, status, st, set_sparse_for(s, total)), "rebuild")) return -1;
  return 0;
}

}  // namespace
}  // namespace gqf

extern "C" {

int gqf_set_create(uint32_t n, const int* nbits, uint64_t max_batch_keys, gqf_set** out) {
  if (!out) return fail("null output");
  *out = nullptr;
  if (n == 0 || !nbits) return fail("filter set: need at least one filter");
  if (max_batch_keys == 0 || max_batch_keys > 0xFFFFFFF0ULL) return fail("filter set: max_batch_keys in [1, 2^32)");
  gqf_set* s = new gqf_set();
  s->n = n;
  s->h.resize(n);
  uint64_t blocks = 0;
  uint64_t regions11 = 0;
  for (uint32_t f = 0; f < n; f++) {
    if (nbits[f] < 6 || nbits[f] > 32) {
      delete s;
      return fail("filter set: nbits must be in [6, 32]");
    }
    quotient_filter& q = s->h[f];
    q = quotient_filter{};
    q.nslots = 1ULL << nbits[f];
    q.xnslots = q.nslots + (uint64_t)(10 * std::sqrt((double)q.nslots));  // qf_init, src/gqf.cu:1950-1951
    q.nblocks = (q.xnslots + 63) / 64;
    q.range = q.nslots << 8;
    q.nbits = (uint32_t)nbits[f];
    q.key_bits = (uint32_t)nbits[f] + 8;
    blocks += q.nblocks;
    regions11 += (regions_of(q, kMinLogRegion) + 1) & ~1u;
  }
  s->arena_blocks = blocks;
  s->region_cap = (uint32_t)(regions11 + 2);
  s->key_cap = max_batch_keys;
  const uint64_t cap = s->region_cap;
  uint32_t* tables = nullptr;
  bool good = ok(cudaMalloc((void**)&s->arena, blocks * sizeof(Block)), "cudaMalloc arena") &&
              ok(cudaMemset(s->arena, 0, blocks * sizeof(Block)), "cudaMemset arena") &&
              ok(cudaMalloc((void**)&s->aux, 256), "cudaMalloc aux") &&
              ok(cudaMemset(s->aux, 0, 256), "cudaMemset aux") &&
              ok(cudaMalloc((void**)&s->dqfs, n * sizeof(quotient_filter)), "cudaMalloc descriptors") &&
              ok(cudaMalloc((void**)&s->region_base, (n + 1) * sizeof(uint32_t)), "cudaMalloc region table") &&
              ok(cudaMalloc((void**)&tables, 5 * cap * sizeof(uint32_t)), "cudaMalloc region arrays") &&
              ok(cudaMalloc((void**)&s->part.keys, max_batch_keys * sizeof(uint32_t)), "cudaMalloc keys");
  if (good) {
    uint64_t at = 0;
    for (uint32_t f = 0; f < n; f++) {
      s->h[f].blocks = s->arena + at;
      s->h[f].status = reinterpret_cast<uint32_t*>(s->aux);
      at += s->h[f].nblocks;
    }
    good = ok(cudaMemcpy(s->dqfs, s->h.data(), n * sizeof(quotient_filter), cudaMemcpyHostToDevice), "cudaMemcpy");
    s->part.region_count = tables;
    s->part.region_start = tables + cap;
    s->part.cursor = tables + 2 * cap;
    s->part.deferred = tables + 3 * cap;
    s->part.retry = tables + 4 * cap;
    s->part.stats = reinterpret_cast<unsigned long long*>(s->aux + 128);
    good = good && layout_regions(s, kMinLogRegion);
  }
  if (!good) {
    if (tables) cudaFree(tables);
    if (s->part.keys) cudaFree(s->part.keys);
    if (s->arena) cudaFree(s->arena);
    if (s->aux) cudaFree(s->aux);
    if (s->dqfs) cudaFree(s->dqfs);
    if (s->region_base) cudaFree(s->region_base);
    delete s;
    return -1;
  }
  *out = s;
  return 0;
}

void gqf_set_destroy(gqf_set* s) {
  if (!s) return;
  cudaDeviceSynchronize();
  cudaFree(s->part.region_count);
  cudaFree(s->part.keys);
  cudaFree(s->arena);
  cudaFree(s->aux);
  cudaFree(s->dqfs);
  cudaFree(s->region_base);
  delete s;
}

int gqf_set_insert(gqf_set* s, const uint64_t* keys, const uint64_t* offsets, uint64_t total, uint8_t flags,
                   void* stream) {
  return set_update(s, keys, offsets, total, flags, Op::kInsert, (cudaStream_t)stream);
}

int gqf_set_delete(gqf_set* s, const uint64_t* keys, const uint64_t* offsets, uint64_t total, uint8_t flags,
                   void* stream) {
  return set_update(s, keys, offsets, total, flags, Op::kDelete, (cudaStream_t)stream);
}

int gqf_set_get(gqf_set* s, const uint64_t* keys, const uint64_t* offsets, uint64_t total, uint64_t* counts,
                uint8_t flags, void* stream) {
  if (!s) return fail("null filter set");
  if (total == 0) return 0;
  if (!keys || !offsets || !counts) return fail("filter set: null keys, offsets or counts");
  k_set_get<<<grid_for_keys(total) * 2, 256, 0, (cudaStream_t)stream>>>(
      s->dqfs, s->n, keys, offsets, total, (flags & QF_KEY_IS_HASH) ? 1 : 0, counts);
  count_launch();
  return ok(cudaGetLastError(), "set get") ? 0 : -1;
}

int gqf_set_reset(gqf_set* s, void* stream) {
  if (!s) return fail("null filter set");
  cudaStream_t st = (cudaStream_t)stream;
  return ok(cudaMemsetAsync(s->arena, 0, s->arena_blocks * sizeof(Block), st), "memset") &&
                 ok(cudaMemsetAsync(s->aux, 0, 256, st), "memset")
             ? 0
             : -1;
}

int gqf_set_config(gqf_set* s, int log_region, uint32_t sparse_max) {
  if (!s) return fail("null filter set");
  if (log_region < kMinLogRegion || log_region > kMaxLogRegion) return fail("log_region must be 11, 12 or 13");
  if (!layout_regions(s, log_region)) return -1;
  s->sparse_max = sparse_max;
  return 0;
}

int gqf_set_get_config(gqf_set* s, int* log_region, uint32_t* sparse_max) {
  if (!s) return fail("null filter set");
  if (log_region) *log_region = s->log_region;
  if (sparse_max) *sparse_max = s->sparse_max;
  return 0;
}

int gqf_set_tune(gqf_set* s, const uint64_t* keys, const uint64_t* offsets, uint64_t total, uint8_t flags,
                 double* best_ms) {
  if (!s) return fail("null filter set");
  cudaEvent_t e0, e1;
  if (!ok(cudaEventCreate(&e0), "event") || !ok(cudaEventCreate(&e1), "event")) return -1;
  double best = 1e30;
  int best_lr = s->log_region;
  uint32_t best_sp = s->sparse_max;
  for (int lr = kMinLogRegion; lr <= kMaxLogRegion; lr++) {
    for (uint32_t sp : {0u, (uint32_t)GQF_SPARSE_AUTO}) {
      if (gqf_set_config(s, lr, sp) != 0) continue;
      double t = 1e30;
      for (int rep = 0; rep < 2; rep++) {  // the first run also configures the kernels
        gqf_set_reset(s, nullptr);
        cudaEventRecord(e0, 0);
        if (set_update(s, keys, offsets, total, flags, Op::kInsert, 0) != 0) break;
        cudaEventRecord(e1, 0);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        t = std::min(t, (double)ms);
      }
      if (t < best) {
        best = t;
        best_lr = lr;
        best_sp = sp;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  gqf_set_reset(s, nullptr);
  if (best_ms) *best_ms = best;
  if (cudaDeviceSynchronize() != cudaSuccess) return fail("filter set tune failed");
  return gqf_set_config(s, best_lr, best_sp);
}

uint64_t gqf_set_export_size(gqf_set* s, uint32_t i) {
  if (!s || i >= s->n) return 0;
  return 120 + 81 * s->h[i].nblocks;
}

int gqf_set_export(gqf_set* s, uint32_t i, uint8_t* out, uint64_t size) {
  if (!s || i >= s->n || !out) return fail("filter set export: bad arguments");
  const quotient_filter& q = s->h[i];
  if (size < 120 + 81 * q.nblocks) return fail("filter set export: buffer too small");
  Geom g{q.blocks, q.nslots, q.xnslots, q.nblocks, q.range, q.range - 1, q.nbits};
  uint8_t* dev = nullptr;
  bool good = ok(cudaMalloc((void**)&dev, 81 * q.nblocks), "cudaMalloc") &&
              ok(launch_export(g, dev, 0), "export") &&
              ok(cudaMemcpy(out + 120, dev, 81 * q.nblocks, cudaMemcpyDeviceToHost), "cudaMemcpy");
  if (dev) cudaFree(dev);
  if (!good) return -1;
  // the reference's qfmetadata for a filter of this size (as gqf_export writes)
  uint64_t meta[15] = {0};
  meta[0] = 1018874902021329732ULL;  // MAGIC_NUMBER
  meta[1] = (uint64_t)QF_HASH_INVERTIBLE;
  meta[2] = 81 * q.nblocks;
  meta[4] = q.nslots;
  meta[5] = q.xnslots;
  meta[6] = q.key_bits;
  meta[8] = 8;
  meta[9] = 8;
  meta[10] = q.range;
  meta[11] = q.nblocks;
  std::memcpy(out, meta, 120);
  return 0;
}

int gqf_set_get_status(gqf_set* s, uint32_t* status) {
  if (!s || !status) return fail("filter set status: bad arguments");
  return ok(cudaMemcpy(status, s->aux, 4, cudaMemcpyDeviceToHost), "cudaMemcpy") ? 0 : -1;
}

}  // extern "C"
