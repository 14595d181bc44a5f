// Point API: device-callable single-key operations under region-pair locks
// (src/gqf.cu:2531-3162).  The reference spins on its 16-bit locks without a
// bound (lock_16, src/gqf.cu:2534); here every wait has an iteration cap,
// after which the operation returns QF_TIMEOUT and sets the filter's timeout
// status bit, so a lost lock can never hang the GPU.
//
// Compiled twice: into the shared library (with the batch kernels below) and,
// with -rdc, into libgqf_gb300_device.a for callers that invoke point_* from
// their own kernels, as the reference's callers do.
#include "gqf_kernels.cuh"
#include "../../include/gqf.cuh"

namespace gqf {
namespace {

__device__ __forceinline__ uint32_t* lock_word(const quotient_filter* qf, uint64_t idx) {
  return qf->locks + idx * kLockStride;
}

__device__ __forceinline__ bool try_lock(const quotient_filter* qf, uint64_t idx) {
  if (idx >= qf->nlocks) return true;  // past the last lock: nothing to guard
  return atomicCAS(lock_word(qf, idx), 0u, 1u) == 0u;
}

__device__ __forceinline__ bool lock_bounded(const quotient_filter* qf, uint64_t idx) {
  uint32_t limit = qf->lock_spin_limit;
  unsigned ns = 32;
  for (uint32_t i = 0; i < limit; i++) {
    if (try_lock(qf, idx)) return true;
    __nanosleep(ns);
    if (ns < 1024) ns <<= 1;
  }
  atomicOr(qf->status, kStTimeout);
  return false;
}

__device__ __forceinline__ void unlock(const quotient_filter* qf, uint64_t idx) {
  if (idx >= qf->nlocks) return;
  __threadfence();
  atomicExch(lock_word(qf, idx), 0u);
}

// Both locks of the pair (lock_index, lock_index + 1), in increasing order,
// as the reference takes them (src/gqf.cu:2985-3003).
__device__ __forceinline__ bool lock_pair(const quotient_filter* qf, uint64_t idx) {
  if (!lock_bounded(qf, idx)) return false;
  if (!lock_bounded(qf, idx + 1)) {
    unlock(qf, idx);
    return false;
  }
  return true;
}

__device__ __forceinline__ uint64_t to_hash(const quotient_filter* qf, uint64_t key, uint8_t flags) {
  if ((flags & QF_KEY_IS_HASH) != QF_KEY_IS_HASH) key = hash64(key, qf->range - 1);
  return key % qf->range;
}

}  // namespace
}  // namespace gqf

using namespace gqf;

extern "C" {

// point_insert (src/gqf.cu:2970-3021)
__device__ qf_returns point_insert(QF* qf, uint64_t key, uint8_t value, uint8_t flags) {
  (void)value;
  uint64_t hash = to_hash(qf, key, flags);
  uint64_t li = (hash >> 8) / kLockRegion;
  if (!lock_pair(qf, li)) return QF_TIMEOUT;
  int ret = Serial(qf).insert1(hash);
  unlock(qf, li + 1);
  unlock(qf, li);
  if (ret < 0) {
    atomicOr(qf->status, kStFull);
    return QF_FULL;
  }
  return QF_ITEM_INSERTED;
}

// point_insert_not_exists (src/gqf.cu:2911-2967)
__device__ qf_returns point_insert_not_exists(QF* qf, uint64_t key, uint8_t value, uint8_t& returnedVal,
                                              uint8_t flags) {
  (void)value;
  uint64_t hash = to_hash(qf, key, flags);
  uint64_t li = (hash >> 8) / kLockRegion;
  if (!lock_pair(qf, li)) return QF_TIMEOUT;
  uint8_t q = 0;
  int ret = Serial(qf).insert1_if_not_exists(hash, &q);
  unlock(qf, li + 1);
  unlock(qf, li);
  if (ret == QF_ITEM_FOUND) returnedVal = q;
  if (ret == QF_FULL) atomicOr(qf->status, kStFull);
  return (qf_returns)ret;
}

// point_query (src/gqf.cu:3024-3052): no locks.
__device__ uint64_t point_query(QF* qf, uint64_t key, uint8_t value, uint8_t& returnedVal, uint8_t flags) {
  (void)value;
  uint64_t hash = to_hash(qf, key, flags);
  returnedVal = 0;  // qf_query's value is remainder & BITMASK(0)
  return Serial(qf).count(hash);
}

// point_query_concurrent (src/gqf.cu:3055-3109): the same under the locks.
__device__ uint64_t point_query_concurrent(QF* qf, uint64_t key, uint8_t value, uint8_t& returnedVal,
                                           uint8_t flags) {
  (void)value;
  uint64_t hash = to_hash(qf, key, flags);
  uint64_t li = (hash >> 8) / kLockRegion;
  returnedVal = 0;
  if (!lock_pair(qf, li)) return 0;
  uint64_t c = Serial(qf).count(hash);
  unlock(qf, li + 1);
  unlock(qf, li);
  return c;
}

// point_bulk_insert (src/gqf.cu:3153-3162): one thread per key, keys hashed.
__global__ void point_bulk_insert(QF* qf, uint64_t* hashes, uint64_t nitems) {
  uint64_t tid = threadIdx.x + (uint64_t)blockIdx.x * blockDim.x;
  if (tid >= nitems) return;
  point_insert(qf, hashes[tid], 0, 0);
}

}  // extern "C"

#ifndef GQF_DEVICE_LIBRARY_ONLY
namespace gqf {
namespace {

__global__ void k_point_insert(QF* qf, const uint64_t* keys, uint64_t n, uint8_t flags, int8_t* rets) {
  uint64_t i = threadIdx.x + (uint64_t)blockIdx.x * blockDim.x;
  if (i >= n) return;
  qf_returns r = point_insert(qf, keys[i], 0, flags);
  if (rets) rets[i] = (int8_t)r;
}

__global__ void k_point_insert_not_exists(QF* qf, const uint64_t* keys, uint64_t n, uint8_t flags,
                                          int8_t* rets, uint8_t* vals) {
  uint64_t i = threadIdx.x + (uint64_t)blockIdx.x * blockDim.x;
  if (i >= n) return;
  uint8_t v = 0;
  qf_returns r = point_insert_not_exists(qf, keys[i], 0, v, flags);
  if (rets) rets[i] = (int8_t)r;
  if (vals) vals[i] = v;
}

__global__ void k_point_query(QF* qf, const uint64_t* keys, uint64_t n, uint8_t flags, int concurrent,
                              uint64_t* counts) {
  uint64_t i = threadIdx.x + (uint64_t)blockIdx.x * blockDim.x;
  if (i >= n) return;
  uint8_t v = 0;
  counts[i] = concurrent ? point_query_concurrent(qf, keys[i], 0, v, flags)
                         : point_query(qf, keys[i], 0, v, flags);
}

// point_bulk_get (src/gqf.cu:3112-3132): misses counted with one atomic.
__global__ void k_point_get_misses(QF* qf, const uint64_t* keys, uint64_t n, unsigned long long* misses) {
  uint64_t i = threadIdx.x + (uint64_t)blockIdx.x * blockDim.x;
  if (i >= n) return;
  uint8_t v = 0;
  if (point_query(qf, keys[i] % qf->range, 0, v, QF_NO_LOCK) == 0) atomicAdd(misses, 1ULL);
}

}  // namespace

cudaError_t launch_point_insert(quotient_filter* dqf, const uint64_t* keys, uint64_t n, uint8_t flags,
                                int8_t* rets, cudaStream_t st) {
  if (!n) return cudaSuccess;
  k_point_insert<<<(unsigned)((n + 31) / 32), 32, 0, st>>>(dqf, keys, n, flags, rets);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_point_insert_not_exists(quotient_filter* dqf, const uint64_t* keys, uint64_t n,
                                           uint8_t flags, int8_t* rets, uint8_t* vals,
                                           cudaStream_t st) {
  if (!n) return cudaSuccess;
  k_point_insert_not_exists<<<(unsigned)((n + 31) / 32), 32, 0, st>>>(dqf, keys, n, flags, rets, vals);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_point_query(quotient_filter* dqf, const uint64_t* keys, uint64_t n, uint8_t flags,
                               int concurrent, uint64_t* counts, cudaStream_t st) {
  if (!n) return cudaSuccess;
  k_point_query<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(dqf, keys, n, flags, concurrent, counts);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_point_get_misses(quotient_filter* dqf, const uint64_t* keys, uint64_t n,
                                    unsigned long long* misses, cudaStream_t st) {
  if (!n) return cudaSuccess;
  k_point_get_misses<<<(unsigned)((n + 511) / 512), 512, 0, st>>>(dqf, keys, n, misses);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_point_bulk_insert(quotient_filter* dqf, uint64_t* keys, uint64_t n, cudaStream_t st) {
  if (!n) return cudaSuccess;
  point_bulk_insert<<<(unsigned)((n + 31) / 32), 32, 0, st>>>(dqf, keys, n);
  count_launch();
  return cudaGetLastError();
}

}  // namespace gqf
#endif
