// Thin C driver over the reference GQF host path (src/gqf.cu), compiled from
// the reference's own sources into oracle/_ref/libgqf_ref.so.
//
// TEST INFRASTRUCTURE ONLY.  It is used here (x86) to pin the C restatement
// in oracle/gqf_oracle.c and to generate the committed golden fixtures.  The
// product never loads it.
//
// Every entry point drives the reference exactly the way its bulk API does
// on the device (src/gqf.cu:3184-3419): keys are hashed with hash_64 under
// BITMASK(nbits+8) (src/gqf.cu:2615-2630), sorted, assigned to 8192-slot
// regions (src/gqf.cu:2646-2750), and each region's keys are applied in order
// with qf_insert / qf_remove under QF_NO_LOCK | QF_KEY_IS_HASH
// (src/gqf.cu:2759-2906), even regions first, then odd ones.
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <algorithm>
#include <vector>

#include "gqf.cuh"
#include "gqf_int.cuh"
#include "hashutil.cuh"

// Defined in src/gqf.cu:2383 with C++ linkage but not declared in its header.
__host__ __device__ qf_returns qf_insert_not_exists(QF* qf, uint64_t key, uint64_t value,
                                                    uint64_t count, uint8_t flags,
                                                    uint8_t* retvalue);

namespace {
const uint64_t kRegion = 8192;  // NUM_SLOTS_TO_LOCK, src/gqf.cu:58

uint64_t mask_bits(uint64_t n) { return n >= 64 ? ~0ULL : ((1ULL << n) - 1); }

// Apply fn to every hash, region by region: even regions first, then odd
// ones; inside a region ascending (insert) or descending (delete) order.
template <class F>
void even_odd(QF* qf, std::vector<uint64_t>& h, bool backwards, F fn) {
  std::sort(h.begin(), h.end());
  uint64_t num_locks = qf->runtimedata->num_locks;
  std::vector<uint64_t> start(num_locks + 1, h.size());
  size_t i = 0;
  for (uint64_t r = 0; r < num_locks; r++) {
    while (i < h.size() && (h[i] >> 8) < kRegion * r) i++;
    start[r] = i;
  }
  start[num_locks] = h.size();
  for (int parity = 0; parity < 2; parity++)
    for (uint64_t r = parity; r < num_locks; r += 2) {
      if (!backwards)
        for (size_t k = start[r]; k < start[r + 1]; k++) fn(h[k]);
      else
        for (size_t k = start[r + 1]; k > start[r]; k--) fn(h[k - 1]);
    }
}
}  // namespace

extern "C" {

void* ref_new(int nbits) {
  QF* qf = (QF*)calloc(1, sizeof(QF));
  // qf_malloc_device's host half: rbits 8, vbits 0, INVERTIBLE, seed 0
  // (src/gqf.cu:2128-2140).
  qf_malloc(qf, 1ULL << nbits, nbits + 8, 0, QF_HASH_INVERTIBLE, false, 0);
  qf_set_auto_resize(qf, false);
  return qf;
}

void ref_free(void* p) {
  QF* qf = (QF*)p;
  qf_free(qf);
  free(qf);
}

uint64_t ref_hash(uint64_t key, uint64_t nbits) { return hash_64(key, mask_bits(nbits + 8)); }

uint64_t ref_total_bytes(void* p) {
  QF* qf = (QF*)p;
  return sizeof(qfmetadata) + qf->metadata->total_size_in_bytes;
}

// Copies the 120-byte metadata followed by the packed 81-byte blocks.
uint64_t ref_dump(void* p, uint8_t* out, uint64_t len) {
  QF* qf = (QF*)p;
  uint64_t need = sizeof(qfmetadata) + qf->metadata->total_size_in_bytes;
  if (len < need) return need;
  memcpy(out, qf->metadata, sizeof(qfmetadata));
  memcpy(out + sizeof(qfmetadata), qf->blocks, qf->metadata->total_size_in_bytes);
  return need;
}

int ref_insert_hash(void* p, uint64_t hash, uint64_t count) {
  return qf_insert((QF*)p, hash, 0, count, QF_NO_LOCK | QF_KEY_IS_HASH);
}

int ref_remove_hash(void* p, uint64_t hash, uint64_t count) {
  return qf_remove((QF*)p, hash, 0, count, QF_NO_LOCK | QF_KEY_IS_HASH);
}

uint64_t ref_count_hash(void* p, uint64_t hash) {
  return qf_count_key_value((QF*)p, hash, 0, QF_NO_LOCK | QF_KEY_IS_HASH);
}

// bulk_insert (src/gqf.cu:3184) on the host: hash, sort, even/odd regions.
void ref_bulk_insert(void* p, uint64_t n, const uint64_t* keys, int key_is_hash) {
  QF* qf = (QF*)p;
  std::vector<uint64_t> h(keys, keys + n);
  if (!key_is_hash)
    for (auto& x : h) x = hash_64(x, mask_bits(qf->metadata->key_bits));
  even_odd(qf, h, false, [&](uint64_t x) { qf_insert(qf, x, 0, 1, QF_NO_LOCK | QF_KEY_IS_HASH); });
}

// bulk_insert_reduce (src/gqf.cu:3238): hash, sort, run-length counts,
// then qf_insert(hash, count) per unique hash in even/odd regions.
void ref_bulk_insert_reduce(void* p, uint64_t n, const uint64_t* keys, int key_is_hash) {
  QF* qf = (QF*)p;
  std::vector<uint64_t> h(keys, keys + n);
  if (!key_is_hash)
    for (auto& x : h) x = hash_64(x, mask_bits(qf->metadata->key_bits));
  std::sort(h.begin(), h.end());
  std::vector<uint64_t> u, c;
  for (size_t i = 0; i < h.size();) {
    size_t j = i;
    while (j < h.size() && h[j] == h[i]) j++;
    u.push_back(h[i]);
    c.push_back(j - i);
    i = j;
  }
  // even_odd sorts again; u is already sorted and unique, so the index of
  // each unique hash is recovered by binary search.
  std::vector<uint64_t> uu = u;
  even_odd(qf, uu, false, [&](uint64_t x) {
    size_t k = std::lower_bound(u.begin(), u.end(), x) - u.begin();
    qf_insert(qf, x, 0, c[k], QF_NO_LOCK | QF_KEY_IS_HASH);
  });
}

// bulk_delete (src/gqf.cu:3316): the region walk goes backwards
// (src/gqf.cu:2892).
void ref_bulk_delete(void* p, uint64_t n, const uint64_t* keys, int key_is_hash) {
  QF* qf = (QF*)p;
  std::vector<uint64_t> h(keys, keys + n);
  if (!key_is_hash)
    for (auto& x : h) x = hash_64(x, mask_bits(qf->metadata->key_bits));
  even_odd(qf, h, true, [&](uint64_t x) { qf_remove(qf, x, 0, 1, QF_NO_LOCK | QF_KEY_IS_HASH); });
}

// bulk_get (src/gqf.cu:3386-3399): hashes inside qf_count_key_value.
void ref_bulk_get(void* p, uint64_t n, const uint64_t* keys, uint64_t* out) {
  QF* qf = (QF*)p;
  for (uint64_t i = 0; i < n; i++) out[i] = qf_count_key_value(qf, keys[i], 0, QF_NO_LOCK);
}

// qf_insert_not_exists / qf_query (src/gqf.cu:2383, :3520): the point API's
// bodies without the locks.
int ref_insert_not_exists_hash(void* p, uint64_t hash, uint8_t* retval) {
  uint8_t v = 0;
  int r = (int)qf_insert_not_exists((QF*)p, hash, 0, 1, QF_NO_LOCK | QF_KEY_IS_HASH, &v);
  *retval = v;
  return r;
}

uint64_t ref_query_hash(void* p, uint64_t hash) {
  uint64_t v = 0;
  return qf_query((QF*)p, hash, &v, QF_NO_LOCK | QF_KEY_IS_HASH);
}

// Byte layout of the reference's device-visible structs as its compiler laid
// them out: what a driver-API launcher must build in device memory.
void ref_layout(uint64_t* out) {
  out[0] = sizeof(QF);
  out[1] = offsetof(QF, runtimedata);
  out[2] = offsetof(QF, metadata);
  out[3] = offsetof(QF, blocks);
  out[4] = sizeof(qfruntime);
  out[5] = offsetof(qfruntime, num_locks);
  out[6] = offsetof(qfruntime, locks);
  out[7] = offsetof(qfruntime, buffers);
  out[8] = offsetof(qfruntime, buffer_sizes);
  out[9] = sizeof(qfmetadata);
  out[10] = sizeof(qfblock);
  out[11] = offsetof(qfruntime, wait_times);
}

}  // extern "C"
