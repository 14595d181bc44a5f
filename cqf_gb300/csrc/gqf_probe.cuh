// The probe of one hash (bulk_get and the filter-set get): restates
// qf_count_key_value (src/gqf.cu:3479-3517).  Header-only so that every
// kernel that probes inlines it.
#pragma once
#include "gqf_device.cuh"

namespace gqf {

static __device__ __forceinline__ uint64_t ld_u64(const unsigned long long* p) { return __ldg(p); }

// Walks one run from `start`; returns the count for `rem` or 0.  The slots
// come through a 16-byte register window and the runends through a one-word
// register cache seeded with the home block's word, so a probe costs one
// header load and usually one slot load, whatever the L1 hit rate.
static __device__ __forceinline__ uint64_t scan_run(const Block* __restrict__ B, uint64_t nblocks,
                                             uint64_t start, uint32_t rem, uint64_t home,
                                             uint64_t home_runends) {
  uint64_t cb = home;
  uint64_t cw = home_runends;
  uint64_t ci = ~0ULL;  // 16-slot chunk index held in `chunk`
  uint4 chunk = make_uint4(0, 0, 0, 0);
  auto is_end = [&](uint64_t i) -> int {
    uint64_t bi = i >> 6;
    if (bi != cb) {
      cb = bi;
      cw = bi < nblocks ? ld_u64(&B[bi].runends) : 0;
    }
    return (int)((cw >> (i & 63)) & 1ULL);
  };
  auto get = [&](uint64_t i) -> uint64_t {
    uint64_t c = i >> 4;
    if (c != ci) {
      ci = c;
      uint64_t bi = i >> 6;
      chunk = bi < nblocks ? __ldg(reinterpret_cast<const uint4*>(&B[bi].slots[(i & 63) & ~15ULL]))
                           : make_uint4(0, 0, 0, 0);
    }
    const uint32_t k = (uint32_t)(i & 15);
    const uint32_t w = k < 8 ? (k < 4 ? chunk.x : chunk.y) : (k < 12 ? chunk.z : chunk.w);
    return (w >> (8 * (k & 3))) & 0xFFu;
  };
  uint32_t cr;
  uint64_t cc, ce;
  const uint64_t lim = 64 * nblocks;
  while (start < lim) {
    ce = decode_counter(get, is_end, start, &cr, &cc, lim);
    if (cr == rem) return cc;
    if (is_end(ce)) return 0;
    start = ce + 1;
  }
  return 0;
}

static __device__ __forceinline__ uint64_t probe(const Block* __restrict__ B, uint64_t nblocks, uint64_t h) {
  const uint64_t q = h >> 8;
  const uint32_t rem = (uint32_t)(h & 255);
  const uint64_t b = q >> 6;
  const int j = (int)(q & 63);
  const ulonglong2 hdr = __ldg(reinterpret_cast<const ulonglong2*>(&B[b]));
  const uint64_t occ = hdr.x;
  if (!((occ >> j) & 1ULL)) return 0;
  const uint64_t off = __ldg(&B[b].offset);
  const int rank = __popcll(occ & ((1ULL << j) - 1ULL));
  uint64_t start;
  if (rank == 0) {
    start = 64 * b + off;
    if (start < q) start = q;
  } else {
    uint64_t pos = 64 * b + off;
    uint64_t rb = pos >> 6;
    uint64_t w = (rb == b ? hdr.y : ld_u64(&B[rb].runends)) & (~0ULL << (pos & 63));
    int k = rank - 1;
    int c = __popcll(w);
    while (k >= c) {
      k -= c;
      rb++;
      if (rb >= nblocks) return 0;
      w = ld_u64(&B[rb].runends);
      c = __popcll(w);
    }
    uint64_t e = 64 * rb + (uint64_t)select64(w, k);
    start = e + 1 > q ? e + 1 : q;
  }
  return scan_run(B, nblocks, start, rem, b, hdr.y);
}

}  // namespace gqf
