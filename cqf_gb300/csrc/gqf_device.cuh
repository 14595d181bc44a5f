// Device-side storage layout and single-key operations of the GB300 GQF.
//
// Storage: 96-byte blocks of 64 slots, laid out for 32-byte sectors:
//   [ 0, 8)  occupieds  bit j set when quotient 64b+j has a run
//   [ 8,16)  runends    bit j set when slot 64b+j ends a run
//   [16,20)  offset     EXACT count of leading slots of this block that hold
//                       runs of quotients < 64b (the reference stores a
//                       uint8 saturating at 255, include/gqf_int.cuh:38-57)
//   [20,32)  padding
//   [32,96)  slots      one 8-bit remainder (or counter digit) per slot
// One probe touches the header sector plus one or two slot sectors.  The
// reference's packed 81-byte format is produced only on export.
//
// The single-key operations below restate the reference's algorithms
// (src/gqf.cu:619-1933) on this layout.  Because offsets are exact, the
// reference's saturation fallback (block_offset, src/gqf.cu:619-630) is not
// needed; every operation yields the same canonical layout as the reference.
#pragma once
#include <cstdint>

#ifndef GQF_HD
#define GQF_HD __host__ __device__ __forceinline__
#endif
#ifndef GQF_HDF
#define GQF_HDF __host__ __device__
#endif

namespace gqf {

constexpr uint64_t kSlotsPerBlock = 64;
constexpr uint64_t kLockRegion = 8192;  // point-API lock granularity (src/gqf.cu:58)
constexpr int kLockStride = 32;         // one 32-bit lock word per 128-byte line

// Status bits accumulated in the filter's device status word.
enum : uint32_t {
  kStFull = 1u << 0,      // an insert found no free slot before xnslots
  kStTimeout = 1u << 1,   // a bounded wait (lock, barrier) gave up
  kStBadKey = 1u << 2,    // a QF_KEY_IS_HASH key was >= range and was skipped
  kStDeferred = 1u << 3,  // a region fell back to the serial path (informational)
  kStOverflow = 1u << 4,  // a counter or region exceeded an internal limit
};

struct __align__(32) Block {
  unsigned long long occupieds;
  unsigned long long runends;
  uint32_t offset;
  uint32_t pad0;
  unsigned long long pad1;
  uint8_t slots[64];
};
static_assert(sizeof(Block) == 96, "block is three 32-byte sectors");

}  // namespace gqf

// The device-resident descriptor.  The QF* handed out by qf_malloc_device
// points at one of these in device memory, as the reference's does
// (src/gqf.cu:2212-2217).
struct quotient_filter {
  gqf::Block* blocks;
  uint64_t nslots;
  uint64_t xnslots;
  uint64_t nblocks;
  uint64_t range;      // 2^(nbits+8)
  uint32_t nbits;
  uint32_t key_bits;   // nbits + 8
  uint32_t* locks;     // point-API locks, kLockStride apart
  uint64_t nlocks;
  uint32_t* status;    // device status word
  uint32_t lock_spin_limit;
  uint32_t pad;
};

namespace gqf {

GQF_HD uint64_t bitmask(int n) { return n >= 64 ? ~0ULL : ((1ULL << n) - 1ULL); }

// hash_64 (src/hashutil.cu:132-142): Thomas Wang's invertible 64-bit mix,
// restricted to the low key_bits bits.  Its shift-and-add steps are products
// by constants modulo 2^64, written as such: ~k + (k << 21) = k * (2^21 - 1)
// - 1, k + (k << 3) + (k << 8) = k * 265, k + (k << 2) + (k << 4) = k * 21,
// k + (k << 31) = k * (2^31 + 1).
GQF_HD uint64_t hash64(uint64_t key, uint64_t mask) {
  key = (key * ((1ULL << 21) - 1ULL) - 1ULL) & mask;
  key = key ^ key >> 24;
  key = (key * 265ULL) & mask;
  key = key ^ key >> 14;
  key = (key * 21ULL) & mask;
  key = key ^ key >> 28;
  key = (key * ((1ULL << 31) + 1ULL)) & mask;
  return key;
}

// hash_64i (src/hashutil.cu:146-170): the inverse of hash64 under the same
// mask, undoing its steps in reverse order (used to report keys, as the
// reference's qfi_get_key does for invertible filters).
GQF_HD uint64_t hash64i(uint64_t key, uint64_t mask) {
  uint64_t tmp;
  tmp = key - (key << 31);  // invert key + (key << 31)
  key = (key - (tmp << 31)) & mask;
  tmp = key ^ key >> 28;  // invert key ^ key >> 28
  key = key ^ tmp >> 28;
  key = (key * 14933078535860113213ull) & mask;  // inverse of 21 mod 2^64
  tmp = key ^ key >> 14;  // invert key ^ key >> 14
  tmp = key ^ tmp >> 14;
  tmp = key ^ tmp >> 14;
  key = key ^ tmp >> 14;
  key = (key * 15244667743933553977ull) & mask;  // inverse of 265 mod 2^64
  tmp = key ^ key >> 24;  // invert key ^ key >> 24
  key = key ^ tmp >> 24;
  tmp = ~key;  // invert ~key + (key << 21)
  tmp = ~(key - (tmp << 21));
  tmp = ~(key - (tmp << 21));
  key = ~(key - (tmp << 21)) & mask;
  return key;
}

GQF_HD int popc64(uint64_t v) {
#ifdef __CUDA_ARCH__
  return __popcll(v);
#else
  return __builtin_popcountll(v);
#endif
}

// Position of the k-th (0-based) set bit of x, or 64.  Binary search over
// popcounts of halves; branch-free selects on the device.
GQF_HD int select64(uint64_t x, int k) {
  if (k < 0 || k >= popc64(x)) return 64;
  int pos = 0, c;
  c = popc64(x & 0xFFFFFFFFULL); if (k >= c) { k -= c; x >>= 32; pos += 32; }
  c = popc64(x & 0xFFFFULL);     if (k >= c) { k -= c; x >>= 16; pos += 16; }
  c = popc64(x & 0xFFULL);       if (k >= c) { k -= c; x >>= 8;  pos += 8; }
  c = popc64(x & 0xFULL);        if (k >= c) { k -= c; x >>= 4;  pos += 4; }
  c = popc64(x & 0x3ULL);        if (k >= c) { k -= c; x >>= 2;  pos += 2; }
  c = (int)(x & 1ULL);           if (k >= c) { pos += 1; }
  return pos;
}

// ---------------------------------------------------------------- counters

// encode_counter (src/gqf.cu:1216-1273) written forwards: fills out[0..len)
// and returns len (0..12).
GQF_HD int encode_counter(uint32_t rem, uint64_t counter, uint8_t* out) {
  if (counter == 0) return 0;
  if (counter == 1) { out[0] = (uint8_t)rem; return 1; }
  if (counter == 2) { out[0] = out[1] = (uint8_t)rem; return 2; }
  if (counter == 3) {
    out[0] = (uint8_t)rem; out[1] = rem == 0 ? 0 : 0; out[2] = (uint8_t)rem;
    return 3;
  }
  // digits are produced least significant first into a scratch array
  uint8_t dig[12];
  int nd = 0;
  uint64_t base = rem ? 254 : 255;
  uint64_t c = counter - (rem ? 3 : 4);
  uint64_t digit = 0;
  do {
    digit = c % base + 1;
    if (rem && digit >= rem) digit++;
    dig[nd++] = (uint8_t)digit;
    c /= base;
  } while (c);
  int len = 0;
  out[len++] = (uint8_t)rem;
  if (rem && digit >= rem) out[len++] = 0;
  for (int i = nd - 1; i >= 0; i--) out[len++] = dig[i];
  if (rem == 0) out[len++] = 0;
  out[len++] = (uint8_t)rem;
  return len;
}

GQF_HD int counter_len(uint32_t rem, uint64_t counter) {
  uint8_t tmp[16];
  return encode_counter(rem, counter, tmp);
}

// decode_counter (src/gqf.cu:1276-1345) over any slot/runend accessor.
// Returns the index of the counter's last slot.  `lim` bounds the digit walk
// (one past the last slot that exists): on a run without a runend the
// reference walks off the table; here the walk stops at the table's end.
template <class Get, class IsEnd>
GQF_HD uint64_t decode_counter(Get get, IsEnd is_end, uint64_t index, uint32_t* remainder,
                               uint64_t* count, uint64_t lim = ~0ULL) {
  uint64_t rem = get(index);
  *remainder = (uint32_t)rem;
  if (is_end(index)) { *count = 1; return index; }
  uint64_t digit = get(index + 1);
  if (is_end(index + 1)) { *count = digit == rem ? 2 : 1; return index + (digit == rem ? 1 : 0); }
  if (rem > 0 && digit >= rem) { *count = digit == rem ? 2 : 1; return index + (digit == rem ? 1 : 0); }
  if (rem > 0 && digit == 0 && get(index + 2) == rem) { *count = 3; return index + 2; }
  if (rem == 0 && digit == 0) {
    if (get(index + 2) == 0) { *count = 3; return index + 2; }
    *count = 2;
    return index + 1;
  }
  uint64_t cnt = 0;
  uint64_t base = 256 - (rem ? 2 : 1);
  uint64_t end = index + 1;
  while (digit != rem && !is_end(end) && end + 1 < lim) {
    if (digit > rem) digit--;
    if (digit && rem) digit--;
    cnt = cnt * base + digit;
    end++;
    digit = get(end);
  }
  if (rem) { *count = cnt + 3; return end; }
  if (is_end(end) || get(end + 1) != 0) { *count = 1; return index; }
  *count = cnt + 4;
  return end + 1;
}

// ------------------------------------------------- a filter in global memory

// Accessors and single-key operations over the descriptor, used by the point
// API and by the serial fallback of the bulk path.  All of them run on one
// thread; callers serialise access (locks or a single fallback thread).
struct Serial {
  Block* b;
  uint64_t nslots, xnslots, nblocks;
  // Every walk below stops at the table's end (64 * nblocks slots), where the
  // reference's would run on past its allocation.

  __host__ __device__ explicit Serial(const quotient_filter* f)
      : b(f->blocks), nslots(f->nslots), xnslots(f->xnslots), nblocks(f->nblocks) {}

  GQF_HDF uint64_t get_slot(uint64_t i) const {
    return (i / 64 < nblocks) ? b[i / 64].slots[i % 64] : 0;
  }
  GQF_HDF void set_slot(uint64_t i, uint64_t v) const {
    if (i / 64 < nblocks) b[i / 64].slots[i % 64] = (uint8_t)v;
  }
  GQF_HDF int is_runend(uint64_t i) const {
    return (i / 64 < nblocks) ? (int)((b[i / 64].runends >> (i % 64)) & 1ULL) : 0;
  }
  GQF_HDF int is_occupied(uint64_t i) const {
    return (i / 64 < nblocks) ? (int)((b[i / 64].occupieds >> (i % 64)) & 1ULL) : 0;
  }
  GQF_HDF unsigned long long& run_word(uint64_t i) const { return b[i / 64].runends; }
  GQF_HDF unsigned long long& occ_word(uint64_t i) const { return b[i / 64].occupieds; }

  // run_end (src/gqf.cu:632-679) with exact block offsets.
  GQF_HDF uint64_t run_end(uint64_t x) const {
    uint64_t bi = x / 64, j = x % 64;
    uint64_t off = b[bi].offset;
    uint64_t occ = b[bi].occupieds;
    uint64_t rank = popc64(occ & ((2ULL << j) - 1ULL));
    if (rank == 0) return off <= j ? x : 64 * bi + off - 1;
    uint64_t rb = bi + off / 64;
    int ignore = (int)(off % 64);
    int k = (int)rank - 1;
    for (;;) {
      if (rb >= nblocks) return 64 * rb;  // corrupt or out of range
      uint64_t w = b[rb].runends & ~bitmask(ignore);
      int c = popc64(w);
      if (k < c) {
        uint64_t e = 64 * rb + select64(w, k);
        return e < x ? x : e;
      }
      k -= c;
      rb++;
      ignore = 0;
    }
  }

  // offset_lower_bound (src/gqf.cu:681-705)
  GQF_HDF int64_t offset_lower_bound(uint64_t slot) const {
    const Block& bk = b[slot / 64];
    uint64_t so = slot % 64;
    uint64_t boff = bk.offset;
    uint64_t occ = bk.occupieds & bitmask((int)so + 1);
    if (boff <= so) {
      uint64_t runs = (bk.runends & bitmask((int)so)) >> boff;
      return popc64(occ) - popc64(runs);
    }
    return (int64_t)(boff - so) + popc64(occ);
  }

  GQF_HDF int is_empty(uint64_t slot) const { return offset_lower_bound(slot) == 0; }
  GQF_HDF int might_be_empty(uint64_t slot) const {
    return !is_occupied(slot) && !is_runend(slot);
  }

  // find_first_empty_slot (src/gqf.cu:728-771)
  GQF_HDF uint64_t find_first_empty_slot(uint64_t from) const {
    for (;;) {
      if (from / 64 >= nblocks) return from;
      int64_t t = offset_lower_bound(from);
      if (t <= 0) return from;
      from += (uint64_t)t;
    }
  }

  // Slots as aligned 8-byte words: word k holds slots 8k .. 8k+7 (byte j of
  // the word is slot 8k + j).  A block's slots start 32 bytes into it, so
  // every such word is 8-byte aligned.
  GQF_HDF unsigned long long& slot_word(uint64_t k) const {
    return reinterpret_cast<unsigned long long*>(b[k >> 3].slots)[k & 7];
  }
  // The 8 slots starting at slot i (any alignment; i + 8 <= 64 * nblocks).
  GQF_HDF unsigned long long slots8(uint64_t i) const {
    const uint64_t k = i >> 3;
    const int sh = (int)(i & 7) * 8;
    const unsigned long long lo = slot_word(k);
    if (!sh) return lo;
    return (lo >> sh) | (slot_word(k + 1) << (64 - sh));
  }

  // shift_slots (src/gqf.cu:973): slots [first, last] move up by distance.
  // Whole aligned destination words at a time, highest first (a destination
  // word's sources all lie below it); bytes outside the destination range
  // keep their values.
  GQF_HDF void shift_slots(uint64_t first, uint64_t last, uint64_t distance) const {
    if (last + 1 <= first) return;
    const uint64_t dlo = first + distance, dhi = last + distance;
    if (distance == 0 || dhi >= 64 * nblocks) {  // (a full table) the byte loop stops at the end
      for (uint64_t i = last + 1; i-- > first;) set_slot(i + distance, get_slot(i));
      return;
    }
    for (uint64_t k = dhi >> 3;; k--) {
      const uint64_t ws = 8 * k;
      const uint64_t lo = ws > dlo ? ws : dlo, hi = ws + 7 < dhi ? ws + 7 : dhi;
      unsigned long long mask = 0;
      for (uint64_t j = lo; j <= hi; j++) mask |= 0xFFULL << (8 * (j - ws));
      unsigned long long src;
      if (ws >= distance) {
        src = slots8(ws - distance);
      } else {  // the word's lowest bytes have no source: only [lo, hi] matters
        src = 0;
        for (uint64_t j = lo; j <= hi; j++) src |= (unsigned long long)get_slot(j - distance) << (8 * (j - ws));
      }
      unsigned long long& w = slot_word(k);
      w = (w & ~mask) | (src & mask);
      if (ws <= dlo) break;
    }
  }

  // shift_remainders (src/gqf.cu:897-937): slots [start, empty) move up one.
  GQF_HDF void shift_remainders(uint64_t start, uint64_t empty) const {
    if (empty > start) shift_slots(start, empty - 1, 1);
  }

  // shift_runends (src/gqf.cu:984-1011): runend bits of [first, last] move up
  // by distance; bits in [first, first+distance) are cleared.  last may be
  // first - 1 (an empty range), which only clears, as the reference does.
  // Whole runends words at a time, highest first.
  GQF_HDF void shift_runends(uint64_t first, uint64_t last, uint64_t distance) const {
    if (last + 1 > first) {
      const uint64_t dlo = first + distance, dhi = last + distance;
      if (distance == 0 || distance >= 64 || dhi >= 64 * nblocks) {
        for (uint64_t i = last + 1; i-- > first;) {
          uint64_t d = i + distance;
          unsigned long long bit = (run_word(i) >> (i % 64)) & 1ULL;
          run_word(d) = (run_word(d) & ~(1ULL << (d % 64))) | (bit << (d % 64));
        }
      } else {
        for (uint64_t k = dhi >> 6;; k--) {
          const uint64_t ws = 64 * k;
          const uint64_t lo = ws > dlo ? ws : dlo, hi = ws + 63 < dhi ? ws + 63 : dhi;
          const unsigned long long mask = (hi - ws == 63 ? ~0ULL : ((2ULL << (hi - ws)) - 1ULL)) &
                                          ~((1ULL << (lo - ws)) - 1ULL);
          const unsigned long long cur = b[k].runends;
          const unsigned long long prev = k ? b[k - 1].runends : 0ULL;  // still unmoved
          const unsigned long long src = (cur << distance) | (prev >> (64 - distance));
          b[k].runends = (cur & ~mask) | (src & mask);
          if (ws <= dlo) break;
        }
      }
    }
    const uint64_t cend = first + distance - 1 < last + distance ? first + distance - 1 : last + distance;
    for (uint64_t i = first; i <= cend && distance; i++) run_word(i) &= ~(1ULL << (i % 64));
  }

  // find_next_n_empty_slots (src/gqf.cu:964)
  GQF_HDF void find_next_n_empty_slots(uint64_t from, uint64_t n, uint64_t* idx) const {
    while (n) {
      idx[--n] = find_first_empty_slot(from);
      from = idx[n] + 1;
    }
  }

  // Window check of a key-by-key update (not in the reference): applying
  // changes that add at most `grow` slots (0 for removals) to the runs of
  // quotients below region_end touches nothing at or past `bound` if the
  // max(grow, 1)-th empty slot after T, the end of those runs, lies below
  // `bound`.  Every change happens at or before T, or moves slots up to the
  // first empty slot after the change, and each added slot consumes one
  // empty slot; a removal only moves slots down inside its cluster, which
  // ends at the first empty slot after it.  region_end is a block boundary
  // below nslots.
  GQF_HDF bool sparse_fits(uint64_t region_end, uint64_t grow, uint64_t bound) const {
    uint64_t x = region_end + b[region_end / 64].offset;  // T + 1
    const uint64_t need = grow ? grow : 1;
    for (uint64_t j = 0; j < need; j++) {
      if (x >= bound) return false;
      x = find_first_empty_slot(x);
      if (x >= bound) return false;
      x++;
    }
    return true;
  }

  // Upper bound on the slots an insert of `count` copies of one hash adds.
  GQF_HDF static uint64_t insert_growth(uint64_t count) {
    if (count <= 1) return 1;
    uint8_t enc[16];
    int a = encode_counter(0, count, enc), c = encode_counter(1, count, enc);
    return (uint64_t)(a > c ? a : c) + 1;
  }

  // insert_replace_slots_and_shift_remainders_and_runends_and_offsets
  // (src/gqf.cu:1013-1097).  Offsets are exact, so they add without
  // saturating.
  GQF_HDF bool insert_replace(int operation, uint64_t bucket, uint64_t overwrite,
                                 const uint8_t* rems, uint64_t total, uint64_t noverwrites) const {
    uint64_t empties[16];
    int64_t ninserts = (int64_t)total - (int64_t)noverwrites;
    uint64_t insert_index = overwrite + noverwrites;
    if (ninserts > 0) {
      find_next_n_empty_slots(insert_index, (uint64_t)ninserts, empties);
      if (empties[0] >= xnslots) return false;
      for (int64_t j = 0; j < ninserts - 1; j++)
        shift_slots(empties[j + 1] + 1, empties[j] - 1, (uint64_t)(j + 1));
      shift_slots(insert_index, empties[ninserts - 1] - 1, (uint64_t)ninserts);
      for (int64_t j = 0; j < ninserts - 1; j++)
        shift_runends(empties[j + 1] + 1, empties[j] - 1, (uint64_t)(j + 1));
      shift_runends(insert_index, empties[ninserts - 1] - 1, (uint64_t)ninserts);
      for (uint64_t i = noverwrites; i + 1 < total; i++)
        run_word(overwrite + i) &= ~(1ULL << ((overwrite + i) % 64));
      uint64_t last = overwrite + total - 1;
      if (operation == 0) {
        run_word(last) |= 1ULL << (last % 64);
      } else if (operation == 1) {
        uint64_t p = overwrite + noverwrites - 1;
        run_word(p) &= ~(1ULL << (p % 64));
        run_word(last) |= 1ULL << (last % 64);
      } else {
        run_word(last) &= ~(1ULL << (last % 64));
      }
      int64_t npre = 0;
      for (uint64_t i = bucket / 64 + 1; i <= empties[0] / 64; i++) {
        while (npre < ninserts && empties[ninserts - 1 - npre] / 64 < i) npre++;
        b[i].offset += (uint32_t)(ninserts - npre);
      }
    }
    for (uint64_t i = 0; i < total; i++) set_slot(overwrite + i, rems[i]);
    return true;
  }

  // remove_replace_slots_and_shift_remainders_and_runends_and_offsets
  // (src/gqf.cu:1099-1201) with exact offsets.
  GQF_HDF void remove_replace(int operation, uint64_t bucket, uint64_t overwrite,
                                 const uint8_t* rems, uint64_t total, uint64_t old_length) const {
    for (uint64_t i = 0; i < total; i++) set_slot(overwrite + i, rems[i]);
    if (is_runend(overwrite + old_length - 1)) {
      if (total > 0) {
        run_word(overwrite + total - 1) |= 1ULL << ((overwrite + total - 1) % 64);
      } else if (overwrite > bucket && !is_runend(overwrite - 1)) {
        run_word(overwrite - 1) |= 1ULL << ((overwrite - 1) % 64);
      }
    }
    uint64_t original_bucket = bucket;
    uint64_t current_bucket = bucket;
    uint64_t current_slot = overwrite + total;
    uint64_t current_distance = old_length - total;
    while (current_distance > 0 && current_slot + current_distance <= 64 * nblocks) {
      if (is_runend(current_slot + current_distance - 1)) {
        do {
          current_bucket++;
        } while (current_bucket < current_slot + current_distance && !is_occupied(current_bucket));
      }
      if (current_bucket <= current_slot) {
        set_slot(current_slot, get_slot(current_slot + current_distance));
        if (is_runend(current_slot) != is_runend(current_slot + current_distance))
          run_word(current_slot) ^= 1ULL << (current_slot % 64);
        current_slot++;
      } else if (current_bucket <= current_slot + current_distance) {
        for (uint64_t k = current_slot; k < current_slot + current_distance; k++) {
          set_slot(k, 0);
          run_word(k) &= ~(1ULL << (k % 64));
        }
        current_distance = current_slot + current_distance - current_bucket;
        current_slot = current_bucket;
      } else {
        current_distance = 0;
      }
    }
    if (operation && !total) occ_word(bucket) &= ~(1ULL << (bucket % 64));
    uint64_t ob = original_bucket / 64;
    if (old_length > total) {
      while (ob + 1 < nblocks) {
        uint64_t last_q = 64 * ob + 63;
        uint64_t re = run_end(last_q);
        uint32_t want = re / 64 == ob ? 0u : (uint32_t)(re - last_q);
        if (b[ob + 1].offset == want) break;
        b[ob + 1].offset = want;
        ob++;
      }
    }
  }

  // insert1 (src/gqf.cu:1523-1765).  Returns >= 0, or -1 when full.
  GQF_HDF int insert1(uint64_t hash) const {
    uint64_t rem = hash & 255, q = hash >> 8, qo = q % 64;
    if (is_empty(q)) {
      run_word(q) |= 1ULL << qo;
      set_slot(q, rem);
      occ_word(q) |= 1ULL << qo;
      return 0;
    }
    uint64_t runend_index = run_end(q);
    int operation = 0;
    uint64_t insert_index = runend_index + 1;
    uint64_t new_value = rem;
    uint64_t runstart = q == 0 ? 0 : run_end(q - 1) + 1;
    if (is_occupied(q)) {
      uint64_t cur = get_slot(runstart);
      uint64_t zero_terminator = runstart;
      if (cur == 0) {
        uint64_t t = runstart + 1;
        while (t < runend_index && get_slot(t) != 0) t++;
        if (t < runend_index && get_slot(t + 1) == 0)
          zero_terminator = t + 1;
        else if (runstart < runend_index && get_slot(runstart + 1) == 0)
          zero_terminator = runstart + 1;
        if (rem != 0) {
          runstart = zero_terminator + 1;
          cur = get_slot(runstart);
        }
      }
      while (cur < rem && runstart <= runend_index) {
        if (runstart < runend_index && get_slot(runstart + 1) < cur) {
          runstart = runstart + 2;
          while (runstart < runend_index && get_slot(runstart) != cur) runstart++;
          runstart++;
        } else {
          runstart++;
        }
        cur = get_slot(runstart);
      }
      if (runstart > runend_index) {
        operation = 1; insert_index = runstart; new_value = rem;
      } else if (cur != rem) {
        operation = 2; insert_index = runstart; new_value = rem;
      } else if (runstart == runend_index || (rem > 0 && get_slot(runstart + 1) > rem) ||
                 (rem == 0 && zero_terminator == runstart)) {
        operation = 2; insert_index = runstart; new_value = rem;
      } else if ((rem > 0 && get_slot(runstart + 1) == rem) ||
                 (rem == 0 && zero_terminator == runstart + 1)) {
        operation = 2; insert_index = runstart + 1; new_value = 0;
      } else if (rem == 0 && zero_terminator == runstart + 2) {
        operation = 2; insert_index = runstart + 1; new_value = 1;
      } else {
        insert_index = runstart + 1;
        while (get_slot(insert_index + 1) != rem && insert_index + 1 < 64 * nblocks) insert_index++;
        uint64_t digit, carry;
        do {
          carry = 0;
          digit = get_slot(insert_index);
          if (digit == 0) { digit++; if (digit == cur) digit++; }
          digit = (digit + 1) & 255;
          if (digit == 0) { digit++; carry = 1; }
          if (digit == cur) digit = (digit + 1) & 255;
          if (digit == 0) { digit++; carry = 1; }
          set_slot(insert_index, digit);
          insert_index--;
        } while (insert_index > runstart && carry);
        if (insert_index == runstart && (carry > 0 || (cur != 0 && digit >= cur))) {
          operation = 2;
          insert_index = runstart + 1;
          new_value = carry ? 2 : 0;
        } else {
          operation = -1;
        }
      }
    }
    if (operation >= 0) {
      uint64_t empty = find_first_empty_slot(runend_index + 1);
      if (empty >= xnslots) return -1;
      shift_remainders(insert_index, empty);
      set_slot(insert_index, new_value);
      shift_runends(insert_index, empty - 1, 1);
      if (operation == 0) {
        run_word(insert_index) |= 1ULL << (insert_index % 64);
      } else if (operation == 1) {
        run_word(insert_index - 1) &= ~(1ULL << ((insert_index - 1) % 64));
        run_word(insert_index) |= 1ULL << (insert_index % 64);
      } else {
        run_word(insert_index) &= ~(1ULL << (insert_index % 64));
      }
      for (uint64_t i = q / 64 + 1; i <= empty / 64; i++) b[i].offset++;
    }
    occ_word(q) |= 1ULL << qo;
    return (int)(insert_index > q ? insert_index - q : 0);
  }

  // insert (src/gqf.cu:1768-1873): count > 1.  Returns >= 0 or -1 when full.
  GQF_HDF int insert(uint64_t hash, uint64_t count) const {
    uint64_t rem = hash & 255, q = hash >> 8, qo = q % 64;
    uint64_t runend_index = run_end(q);
    if (might_be_empty(q) && runend_index == q) {
      run_word(q) |= 1ULL << qo;
      set_slot(q, rem);
      occ_word(q) |= 1ULL << qo;
      if (count > 1) return insert(hash, count - 1);
      return 0;
    }
    uint8_t nv[16];
    uint64_t runstart = q == 0 ? 0 : run_end(q - 1) + 1;
    bool ok;
    if (!is_occupied(q)) {
      int len = encode_counter((uint32_t)rem, count, nv);
      ok = insert_replace(0, q, runstart, nv, (uint64_t)len, 0);
    } else {
      uint32_t cr;
      uint64_t cc;
      auto g = [&](uint64_t i) { return get_slot(i); };
      auto e = [&](uint64_t i) { return is_runend(i); };
      const uint64_t lim = 64 * nblocks;
      uint64_t ce = decode_counter(g, e, runstart, &cr, &cc, lim);
      while (cr < rem && !is_runend(ce) && ce + 1 < lim) {
        runstart = ce + 1;
        ce = decode_counter(g, e, runstart, &cr, &cc, lim);
      }
      if (cr < rem) {
        int len = encode_counter((uint32_t)rem, count, nv);
        ok = insert_replace(1, q, ce + 1, nv, (uint64_t)len, 0);
      } else if (cr == rem) {
        int len = encode_counter((uint32_t)rem, cc + count, nv);
        ok = insert_replace(is_runend(ce) ? 1 : 2, q, runstart, nv, (uint64_t)len, ce - runstart + 1);
      } else {
        int len = encode_counter((uint32_t)rem, count, nv);
        ok = insert_replace(2, q, runstart, nv, (uint64_t)len, 0);
      }
    }
    if (!ok) return -1;
    occ_word(q) |= 1ULL << qo;
    return 0;
  }

  // _remove (src/gqf.cu:1876-1933).  Returns -1 when the hash is absent.
  GQF_HDF int remove(uint64_t hash, uint64_t count) const {
    uint64_t rem = hash & 255, q = hash >> 8;
    if (!is_occupied(q)) return -1;
    uint64_t runstart = q == 0 ? 0 : run_end(q - 1) + 1;
    uint64_t original = runstart;
    uint32_t cr;
    uint64_t cc;
    auto g = [&](uint64_t i) { return get_slot(i); };
    auto e = [&](uint64_t i) { return is_runend(i); };
    const uint64_t lim = 64 * nblocks;
    uint64_t ce = decode_counter(g, e, runstart, &cr, &cc, lim);
    while (cr < rem && !is_runend(ce) && ce + 1 < lim) {
      runstart = ce + 1;
      ce = decode_counter(g, e, runstart, &cr, &cc, lim);
    }
    if (cr != rem) return -1;
    int only = (original == runstart && is_runend(ce)) ? 1 : 0;
    uint8_t nv[16];
    int len = encode_counter((uint32_t)rem, count > cc ? 0 : cc - count, nv);
    remove_replace(only, q, runstart, nv, (uint64_t)len, ce - runstart + 1);
    return 0;
  }

  // qf_count_key_value (src/gqf.cu:3479-3517) on a hash.
  GQF_HDF uint64_t count(uint64_t hash) const {
    uint64_t rem = hash & 255, q = hash >> 8;
    if (!is_occupied(q)) return 0;
    uint64_t runstart = q == 0 ? 0 : run_end(q - 1) + 1;
    if (runstart < q) runstart = q;
    auto g = [&](uint64_t i) { return get_slot(i); };
    auto e = [&](uint64_t i) { return is_runend(i); };
    uint32_t cr;
    uint64_t cc, ce;
    const uint64_t lim = 64 * nblocks;
    do {
      ce = decode_counter(g, e, runstart, &cr, &cc, lim);
      if (cr == rem) return cc;
      runstart = ce + 1;
    } while (!is_runend(ce) && runstart < lim);
    return 0;
  }

  // insert1_if_not_exists (src/gqf.cu:1364-1520).  Returns the qf_returns
  // code: 0 inserted, 1 found, 2 full.  The reference reports the found
  // value as get_slot(..) && BITMASK(0), which is always 0 (src/gqf.cu:1454).
  GQF_HDF int insert1_if_not_exists(uint64_t hash, uint8_t* value) const {
    uint64_t rem = hash & 255, q = hash >> 8, qo = q % 64;
    if (is_empty(q)) {
      run_word(q) |= 1ULL << qo;
      set_slot(q, rem);
      occ_word(q) |= 1ULL << qo;
      return 0;
    }
    uint64_t runend_index = run_end(q);
    int operation = 0;
    uint64_t insert_index = runend_index + 1;
    uint64_t runstart = q == 0 ? 0 : run_end(q - 1) + 1;
    if (is_occupied(q)) {
      uint64_t cur = get_slot(runstart);
      while (cur < rem && runstart <= runend_index) {
        runstart++;
        cur = get_slot(runstart);
      }
      if (runstart > runend_index) {
        operation = 1; insert_index = runstart;
      } else if (cur != rem) {
        operation = 2; insert_index = runstart;
      } else {
        *value = 0;
        return 1;
      }
    }
    uint64_t empty = find_first_empty_slot(runend_index + 1);
    if (empty >= xnslots) return 2;
    shift_remainders(insert_index, empty);
    set_slot(insert_index, rem);
    shift_runends(insert_index, empty - 1, 1);
    if (operation == 0) {
      run_word(insert_index) |= 1ULL << (insert_index % 64);
    } else if (operation == 1) {
      run_word(insert_index - 1) &= ~(1ULL << ((insert_index - 1) % 64));
      run_word(insert_index) |= 1ULL << (insert_index % 64);
    } else {
      run_word(insert_index) &= ~(1ULL << (insert_index % 64));
    }
    for (uint64_t i = q / 64 + 1; i <= empty / 64; i++) b[i].offset++;
    occ_word(q) |= 1ULL << qo;
    return 0;
  }
};

}  // namespace gqf
