/* CPU oracle for the GQF bulk hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference counting quotient filter
 * (PASSIONLab/cqf) on its own packed storage format.  Each function names the
 * reference function it restates (src/gqf.cu unless noted).  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may load this code,
 * as the test oracle or as the timed CPU baseline; the product never calls it.
 *
 * Deviations from the reference, none of which change a result the reference
 * produces without crashing:
 *  - bitselect is a portable binary search instead of x86 pdep/tzcnt
 *    (src/gqf.cu:496-507); both return the position of the rank-th set bit,
 *    or 64.
 *  - Slot reads past the allocated blocks return 0 and every walk stops at
 *    the end of the table, where the reference asserts, reads out of bounds
 *    or loops forever (src/gqf.cu:535, :728-770, :1133-1190, :1326-1334,
 *    :1660-1661); only tables pushed past full reach these states.
 *  - The metadata counters nelts / ndistinct_elts / noccupied_slots stay 0,
 *    as they do in the reference (every modify_metadata is commented out).
 */
#include "gqf_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define SPB 64ULL                 /* QF_SLOTS_PER_BLOCK, include/gqf_int.cuh:35 */
#define REGION_SLOTS 8192ULL      /* NUM_SLOTS_TO_LOCK, src/gqf.cu:58 */
#define BITMASK(n) ((n) >= 64 ? ~0ULL : ((1ULL << (n)) - 1ULL))
#define MAGIC_NUMBER 1018874902021329732ULL /* include/gqf_int.cuh:23 */

/* include/gqf_int.cuh:38-57 with QF_BITS_PER_SLOT 8: 81 bytes. */
typedef struct __attribute__((__packed__)) {
  uint8_t offset;
  uint64_t occupieds;
  uint64_t runends;
  uint8_t slots[64];
} oblock;

/* include/gqf_int.cuh:96-113: 120 bytes with natural alignment. */
typedef struct {
  uint64_t magic_endian_number;
  int32_t hash_mode;
  uint32_t reserved;
  uint64_t total_size_in_bytes;
  uint32_t seed;
  uint64_t nslots;
  uint64_t xnslots;
  uint64_t key_bits;
  uint64_t value_bits;
  uint64_t key_remainder_bits;
  uint64_t bits_per_slot;
  uint64_t range;
  uint64_t nblocks;
  uint64_t nelts;
  uint64_t ndistinct_elts;
  uint64_t noccupied_slots;
} ometa;

struct oqf {
  ometa* meta;
  oblock* blocks;
  uint8_t* buffer;
  uint64_t nslots, xnslots, nblocks, key_bits, range, num_locks;
};

_Static_assert(sizeof(oblock) == 81, "packed block");
_Static_assert(sizeof(ometa) == 120, "metadata header");

/* ---------------------------------------------------------------- hashing */

/* Thomas Wang's invertible mix, hash_64 (src/hashutil.cu:132-142). */
uint64_t oqf_hash64(uint64_t key, uint64_t mask) {
  key = (~key + (key << 21)) & mask;
  key = key ^ key >> 24;
  key = ((key + (key << 3)) + (key << 8)) & mask;
  key = key ^ key >> 14;
  key = ((key + (key << 2)) + (key << 4)) & mask;
  key = key ^ key >> 28;
  key = (key + (key << 31)) & mask;
  return key;
}

/* Its inverse, hash_64i (src/hashutil.cu:146-176). */
uint64_t oqf_hash64i(uint64_t key, uint64_t mask) {
  uint64_t tmp;
  tmp = (key - (key << 31));
  key = (key - (tmp << 31)) & mask;
  tmp = key ^ key >> 28;
  key = key ^ tmp >> 28;
  key = (key * 14933078535860113213ull) & mask;
  tmp = key ^ key >> 14;
  tmp = key ^ tmp >> 14;
  tmp = key ^ tmp >> 14;
  key = key ^ tmp >> 14;
  key = (key * 15244667743933553977ull) & mask;
  tmp = key ^ key >> 24;
  key = key ^ tmp >> 24;
  tmp = ~key;
  tmp = ~(key - (tmp << 21));
  tmp = ~(key - (tmp << 21));
  key = ~(key - (tmp << 21)) & mask;
  return key;
}

/* splitmix64 (Steele, Lea, Flood 2014): the synthetic key generator. */
void oqf_splitmix64(uint64_t seed, uint64_t n, uint64_t* out) {
  uint64_t x = seed;
  for (uint64_t i = 0; i < n; i++) {
    uint64_t z = (x += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    out[i] = z ^ (z >> 31);
  }
}

/* ------------------------------------------------------------- sizing */

/* qf_init (src/gqf.cu:1939-1996) + qf_malloc (:2073) for nslots = 2^nbits,
 * key_bits = nbits + 8, value_bits = 0, QF_HASH_INVERTIBLE, seed 0. */
oqf* oqf_new(int nbits) {
  oqf* qf = (oqf*)calloc(1, sizeof(oqf));
  uint64_t nslots = 1ULL << nbits;
  uint64_t xnslots = nslots + 10 * sqrt((double)nslots);
  uint64_t nblocks = (xnslots + SPB - 1) / SPB;
  uint64_t size = nblocks * sizeof(oblock);
  qf->buffer = (uint8_t*)calloc(1, sizeof(ometa) + size);
  qf->meta = (ometa*)qf->buffer;
  qf->blocks = (oblock*)(qf->buffer + sizeof(ometa));
  ometa* m = qf->meta;
  m->magic_endian_number = MAGIC_NUMBER;
  m->hash_mode = 1; /* QF_HASH_INVERTIBLE, include/gqf.cuh:45-49 */
  m->reserved = 0;
  m->total_size_in_bytes = size;
  m->seed = 0;
  m->nslots = nslots;
  m->xnslots = xnslots;
  m->key_bits = nbits + 8;
  m->value_bits = 0;
  m->key_remainder_bits = 8;
  m->bits_per_slot = 8;
  m->range = nslots << 8;
  m->nblocks = nblocks;
  qf->nslots = nslots;
  qf->xnslots = xnslots;
  qf->nblocks = nblocks;
  qf->key_bits = nbits + 8;
  qf->range = m->range;
  qf->num_locks = xnslots / REGION_SLOTS + 2;
  return qf;
}

void oqf_free(oqf* qf) {
  if (!qf) return;
  free(qf->buffer);
  free(qf);
}

uint64_t oqf_nslots(const oqf* qf) { return qf->nslots; }
uint64_t oqf_xnslots(const oqf* qf) { return qf->xnslots; }
uint64_t oqf_nblocks(const oqf* qf) { return qf->nblocks; }
uint64_t oqf_range(const oqf* qf) { return qf->range; }
uint64_t oqf_total_bytes(const oqf* qf) { return sizeof(ometa) + qf->nblocks * sizeof(oblock); }

uint64_t oqf_dump(const oqf* qf, uint8_t* out, uint64_t len) {
  uint64_t need = oqf_total_bytes(qf);
  if (out && len >= need) memcpy(out, qf->buffer, need);
  return need;
}

int oqf_load(oqf* qf, const uint8_t* in, uint64_t len) {
  if (len != oqf_total_bytes(qf)) return -1;
  memcpy(qf->buffer, in, len);
  return 0;
}

/* -------------------------------------- metadata bits, src/gqf.cu:143-630 */

static inline oblock* get_block(const oqf* qf, uint64_t i) { return &qf->blocks[i]; }
static inline int popcnt(uint64_t v) { return __builtin_popcountll(v); }

/* popcntv (src/gqf.cu:172) */
static inline int popcntv(uint64_t val, int ignore) {
  if (ignore % 64) return popcnt(val & ~BITMASK(ignore % 64));
  return popcnt(val);
}

/* bitrank (src/gqf.cu:181): ones up to and including bit pos */
static inline int bitrank(uint64_t val, int pos) {
  val = val & ((2ULL << pos) - 1);
  return popcnt(val);
}

/* bitselect (src/gqf.cu:496): position of the rank-th (0-based) one, or 64 */
static inline uint64_t bitselect(uint64_t val, int rank) {
  if (rank < 0 || rank >= popcnt(val)) return 64;
  int pos = 0, c;
  c = popcnt(val & 0xFFFFFFFFULL); if (rank >= c) { rank -= c; val >>= 32; pos += 32; }
  c = popcnt(val & 0xFFFFULL);     if (rank >= c) { rank -= c; val >>= 16; pos += 16; }
  c = popcnt(val & 0xFFULL);       if (rank >= c) { rank -= c; val >>= 8;  pos += 8; }
  c = popcnt(val & 0xFULL);        if (rank >= c) { rank -= c; val >>= 4;  pos += 4; }
  c = popcnt(val & 0x3ULL);        if (rank >= c) { rank -= c; val >>= 2;  pos += 2; }
  c = (int)(val & 1ULL);           if (rank >= c) { pos += 1; }
  return (uint64_t)pos;
}

/* bitselectv (src/gqf.cu:514) */
static inline uint64_t bitselectv(uint64_t val, int ignore, int rank) {
  return bitselect(val & ~BITMASK(ignore % 64), rank);
}

/* The packed words are unaligned: access them through a 1-aligned type. */
typedef uint64_t __attribute__((aligned(1), may_alias)) u64u;
static inline u64u* occ_word(const oqf* qf, uint64_t i) {
  return (u64u*)((uint8_t*)get_block(qf, i / SPB) + 1);
}
static inline u64u* run_word(const oqf* qf, uint64_t i) {
  return (u64u*)((uint8_t*)get_block(qf, i / SPB) + 9);
}

/* is_runend / is_occupied (src/gqf.cu:519-529) */
static inline int is_runend(const oqf* qf, uint64_t i) {
  if (i / SPB >= qf->nblocks) return 0;
  return (*run_word(qf, i) >> (i % SPB)) & 1ULL;
}
static inline int is_occupied(const oqf* qf, uint64_t i) {
  if (i / SPB >= qf->nblocks) return 0;
  return (*occ_word(qf, i) >> (i % SPB)) & 1ULL;
}

/* get_slot / set_slot (src/gqf.cu:533-546) */
static inline uint64_t get_slot(const oqf* qf, uint64_t i) {
  if (i / SPB >= qf->nblocks) return 0;
  return get_block(qf, i / SPB)->slots[i % SPB];
}
static inline void set_slot(const oqf* qf, uint64_t i, uint64_t v) {
  if (i / SPB >= qf->nblocks) return;
  get_block(qf, i / SPB)->slots[i % SPB] = (uint8_t)(v & 0xFF);
}

static uint64_t run_end(const oqf* qf, uint64_t hash_bucket_index);

/* block_offset (src/gqf.cu:619): the stored byte, or a run_end walk when it
 * has saturated at 255. */
static uint64_t block_offset(const oqf* qf, uint64_t blockidx) {
  if (get_block(qf, blockidx)->offset < 255) return get_block(qf, blockidx)->offset;
  return run_end(qf, SPB * blockidx - 1) - SPB * blockidx + 1;
}

/* run_end (src/gqf.cu:632-679) */
static uint64_t run_end(const oqf* qf, uint64_t hash_bucket_index) {
  uint64_t bucket_block_index = hash_bucket_index / SPB;
  uint64_t bucket_intrablock_offset = hash_bucket_index % SPB;
  uint64_t bucket_blocks_offset = block_offset(qf, bucket_block_index);
  uint64_t bucket_intrablock_rank =
      bitrank(get_block(qf, bucket_block_index)->occupieds, (int)bucket_intrablock_offset);

  if (bucket_intrablock_rank == 0) {
    if (bucket_blocks_offset <= bucket_intrablock_offset)
      return hash_bucket_index;
    else
      return SPB * bucket_block_index + bucket_blocks_offset - 1;
  }

  uint64_t runend_block_index = bucket_block_index + bucket_blocks_offset / SPB;
  uint64_t runend_ignore_bits = bucket_blocks_offset % SPB;
  uint64_t runend_rank = bucket_intrablock_rank - 1;
  uint64_t runend_block_offset = bitselectv(get_block(qf, runend_block_index)->runends,
                                            (int)runend_ignore_bits, (int)runend_rank);
  if (runend_block_offset == SPB) {
    if (bucket_blocks_offset == 0 && bucket_intrablock_rank == 0) {
      return hash_bucket_index;
    } else {
      do {
        runend_rank -= popcntv(get_block(qf, runend_block_index)->runends, (int)runend_ignore_bits);
        runend_block_index++;
        if (runend_block_index >= qf->nblocks) return SPB * runend_block_index; /* guard */
        runend_ignore_bits = 0;
        runend_block_offset = bitselectv(get_block(qf, runend_block_index)->runends,
                                         (int)runend_ignore_bits, (int)runend_rank);
      } while (runend_block_offset == SPB);
    }
  }

  uint64_t runend_index = SPB * runend_block_index + runend_block_offset;
  if (runend_index < hash_bucket_index)
    return hash_bucket_index;
  else
    return runend_index;
}

/* offset_lower_bound (src/gqf.cu:681-705) */
static int offset_lower_bound(const oqf* qf, uint64_t slot_index) {
  const oblock* b = get_block(qf, slot_index / SPB);
  const uint64_t slot_offset = slot_index % SPB;
  const uint64_t boffset = b->offset;
  const uint64_t occupieds = b->occupieds & BITMASK(slot_offset + 1);
  if (boffset <= slot_offset) {
    const uint64_t runends = (b->runends & BITMASK(slot_offset)) >> boffset;
    return popcnt(occupieds) - popcnt(runends);
  }
  return (int)(boffset - slot_offset + popcnt(occupieds));
}

/* is_empty / might_be_empty (src/gqf.cu:707-716) */
static inline int is_empty(const oqf* qf, uint64_t slot_index) {
  return offset_lower_bound(qf, slot_index) == 0;
}
static inline int might_be_empty(const oqf* qf, uint64_t slot_index) {
  return !is_occupied(qf, slot_index) && !is_runend(qf, slot_index);
}

/* find_first_empty_slot (src/gqf.cu:728-771) */
static uint64_t find_first_empty_slot(const oqf* qf, uint64_t from) {
  for (;;) {
    if (from / SPB >= qf->nblocks) return from; /* guard: past the last block */
    int t = offset_lower_bound(qf, from);
    if (t <= 0) break; /* the reference asserts t >= 0 */
    from = from + t;
  }
  return from;
}

/* ------------------------------------------ shifting, src/gqf.cu:828-1011 */

/* shift_into_b (src/gqf.cu:828) */
static inline uint64_t shift_into_b(uint64_t a, uint64_t b, int bstart, int bend, int amount) {
  const uint64_t a_component = bstart == 0 ? (a >> (64 - amount)) : 0;
  const uint64_t b_shifted_mask = BITMASK(bend - bstart) << bstart;
  const uint64_t b_shifted = ((b_shifted_mask & b) << amount) & b_shifted_mask;
  const uint64_t b_mask = ~b_shifted_mask;
  return a_component | b_shifted | (b & b_mask);
}

/* shift_remainders (src/gqf.cu:897-937): move slots [start, empty) up by one */
static void shift_remainders(oqf* qf, uint64_t start_index, uint64_t empty_index) {
  uint64_t start_block = start_index / SPB;
  uint64_t start_offset = start_index % SPB;
  uint64_t empty_block = empty_index / SPB;
  uint64_t empty_offset = empty_index % SPB;
  while (start_block < empty_block) {
    memmove(&get_block(qf, empty_block)->slots[1], &get_block(qf, empty_block)->slots[0],
            empty_offset);
    get_block(qf, empty_block)->slots[0] = get_block(qf, empty_block - 1)->slots[SPB - 1];
    empty_block--;
    empty_offset = SPB - 1;
  }
  memmove(&get_block(qf, empty_block)->slots[start_offset + 1],
          &get_block(qf, empty_block)->slots[start_offset], empty_offset - start_offset);
}

/* find_next_n_empty_slots (src/gqf.cu:964) */
static void find_next_n_empty_slots(oqf* qf, uint64_t from, uint64_t n, uint64_t* indices) {
  while (n) {
    indices[--n] = find_first_empty_slot(qf, from);
    from = indices[n] + 1;
  }
}

/* shift_slots (src/gqf.cu:973) */
static void shift_slots(oqf* qf, int64_t first, uint64_t last, uint64_t distance) {
  int64_t i;
  if (distance == 1)
    shift_remainders(qf, first, last + 1);
  else
    for (i = (int64_t)last; i >= first; i--) set_slot(qf, i + distance, get_slot(qf, i));
}

/* shift_runends (src/gqf.cu:984-1011) */
static void shift_runends(oqf* qf, int64_t first, uint64_t last, uint64_t distance) {
  uint64_t first_word = first / 64;
  uint64_t bstart = first % 64;
  uint64_t last_word = (last + distance + 1) / 64;
  uint64_t bend = (last + distance + 1) % 64;
  if (last_word != first_word) {
    *run_word(qf, 64 * last_word) = shift_into_b(*run_word(qf, 64 * (last_word - 1)),
                                                 *run_word(qf, 64 * last_word), 0, (int)bend,
                                                 (int)distance);
    bend = 64;
    last_word--;
    while (last_word != first_word) {
      *run_word(qf, 64 * last_word) = shift_into_b(*run_word(qf, 64 * (last_word - 1)),
                                                   *run_word(qf, 64 * last_word), 0, (int)bend,
                                                   (int)distance);
      last_word--;
    }
  }
  *run_word(qf, 64 * last_word) =
      shift_into_b(0, *run_word(qf, 64 * last_word), (int)bstart, (int)bend, (int)distance);
}

/* insert_replace_slots_and_shift_remainders_and_runends_and_offsets
 * (src/gqf.cu:1013-1097) */
static int insert_replace_slots(oqf* qf, int operation, uint64_t bucket_index,
                                uint64_t overwrite_index, const uint64_t* remainders,
                                uint64_t total_remainders, uint64_t noverwrites) {
  uint64_t empties[67];
  uint64_t i;
  int64_t j;
  int64_t ninserts = (int64_t)total_remainders - (int64_t)noverwrites;
  uint64_t insert_index = overwrite_index + noverwrites;

  if (ninserts > 0) {
    find_next_n_empty_slots(qf, insert_index, ninserts, empties);
    if (empties[0] >= qf->xnslots) return 0;
    for (j = 0; j < ninserts - 1; j++) shift_slots(qf, empties[j + 1] + 1, empties[j] - 1, j + 1);
    shift_slots(qf, insert_index, empties[ninserts - 1] - 1, ninserts);

    for (j = 0; j < ninserts - 1; j++)
      shift_runends(qf, empties[j + 1] + 1, empties[j] - 1, j + 1);
    shift_runends(qf, insert_index, empties[ninserts - 1] - 1, ninserts);

    for (i = noverwrites; i < total_remainders - 1; i++)
      *run_word(qf, overwrite_index + i) &= ~(1ULL << ((overwrite_index + i) % SPB));

    switch (operation) {
      case 0: /* insert into empty bucket */
        *run_word(qf, overwrite_index + total_remainders - 1) |=
            1ULL << ((overwrite_index + total_remainders - 1) % SPB);
        break;
      case 1: /* append to bucket */
        *run_word(qf, overwrite_index + noverwrites - 1) &=
            ~(1ULL << ((overwrite_index + noverwrites - 1) % SPB));
        *run_word(qf, overwrite_index + total_remainders - 1) |=
            1ULL << ((overwrite_index + total_remainders - 1) % SPB);
        break;
      case 2: /* insert into bucket */
        *run_word(qf, overwrite_index + total_remainders - 1) &=
            ~(1ULL << ((overwrite_index + total_remainders - 1) % SPB));
        break;
      default:
        abort();
    }

    int64_t npreceding_empties = 0;
    for (i = bucket_index / SPB + 1; i <= empties[0] / SPB; i++) {
      while (npreceding_empties < ninserts &&
             empties[ninserts - 1 - npreceding_empties] / SPB < i)
        npreceding_empties++;
      if (get_block(qf, i)->offset + ninserts - npreceding_empties < 255)
        get_block(qf, i)->offset += (uint8_t)(ninserts - npreceding_empties);
      else
        get_block(qf, i)->offset = 255;
    }
  }

  for (i = 0; i < total_remainders; i++) set_slot(qf, overwrite_index + i, remainders[i]);
  return 1;
}

/* remove_replace_slots_and_shift_remainders_and_runends_and_offsets
 * (src/gqf.cu:1099-1201) */
static int remove_replace_slots(oqf* qf, int operation, uint64_t bucket_index,
                                uint64_t overwrite_index, const uint64_t* remainders,
                                uint64_t total_remainders, uint64_t old_length) {
  uint64_t i;
  for (i = 0; i < total_remainders; i++) set_slot(qf, overwrite_index + i, remainders[i]);

  if (is_runend(qf, overwrite_index + old_length - 1)) {
    if (total_remainders > 0) {
      *run_word(qf, overwrite_index + total_remainders - 1) |=
          1ULL << ((overwrite_index + total_remainders - 1) % 64);
    } else if (overwrite_index > bucket_index && !is_runend(qf, overwrite_index - 1)) {
      *run_word(qf, overwrite_index - 1) |= 1ULL << ((overwrite_index - 1) % 64);
    }
  }

  uint64_t original_bucket = bucket_index;
  uint64_t current_bucket = bucket_index;
  uint64_t current_slot = overwrite_index + total_remainders;
  uint64_t current_distance = old_length - total_remainders;
  int ret_current_distance = (int)current_distance;

  while (current_distance > 0 && current_slot + current_distance <= SPB * qf->nblocks) {
    if (is_runend(qf, current_slot + current_distance - 1)) {
      do {
        current_bucket++;
      } while (current_bucket < current_slot + current_distance &&
               !is_occupied(qf, current_bucket));
    }
    if (current_bucket <= current_slot) {
      set_slot(qf, current_slot, get_slot(qf, current_slot + current_distance));
      if (is_runend(qf, current_slot) != is_runend(qf, current_slot + current_distance))
        *run_word(qf, current_slot) ^= 1ULL << (current_slot % 64);
      current_slot++;
    } else if (current_bucket <= current_slot + current_distance) {
      uint64_t k;
      for (k = current_slot; k < current_slot + current_distance; k++) {
        set_slot(qf, k, 0);
        *run_word(qf, k) &= ~(1ULL << (k % 64));
      }
      current_distance = current_slot + current_distance - current_bucket;
      current_slot = current_bucket;
    } else {
      current_distance = 0;
    }
  }

  if (operation && !total_remainders)
    *occ_word(qf, bucket_index) &= ~(1ULL << (bucket_index % 64));

  uint64_t original_block = original_bucket / SPB;
  if (old_length > total_remainders) {
    for (;;) {
      if (original_block + 1 >= qf->nblocks) break; /* guard */
      uint64_t last_occupieds_hash_index = SPB * original_block + (SPB - 1);
      uint64_t runend_index = run_end(qf, last_occupieds_hash_index);
      if (runend_index / SPB == original_block) {
        if (get_block(qf, original_block + 1)->offset == 0) break;
        get_block(qf, original_block + 1)->offset = 0;
      } else {
        /* the reference stores the difference into a uint8_t (truncating) */
        if (get_block(qf, original_block + 1)->offset == (runend_index - last_occupieds_hash_index))
          break;
        get_block(qf, original_block + 1)->offset =
            (uint8_t)(runend_index - last_occupieds_hash_index);
      }
      original_block++;
    }
  }
  return ret_current_distance;
}

/* ------------------------------------ counters, src/gqf.cu:1207-1345 */

/* encode_counter (src/gqf.cu:1216-1273): writes backwards from `slots`,
 * returns the first digit. */
static uint64_t* encode_counter(uint64_t remainder, uint64_t counter, uint64_t* slots) {
  uint64_t digit = remainder;
  uint64_t base = (1ULL << 8) - 1;
  uint64_t* p = slots;
  if (counter == 0) return p;
  *--p = remainder;
  if (counter == 1) return p;
  if (counter == 2) {
    *--p = remainder;
    return p;
  }
  if (counter == 3 && remainder == 0) {
    *--p = remainder;
    *--p = remainder;
    return p;
  }
  if (counter == 3 && remainder > 0) {
    *--p = 0;
    *--p = remainder;
    return p;
  }
  if (remainder == 0)
    *--p = remainder;
  else
    base--;
  if (remainder)
    counter -= 3;
  else
    counter -= 4;
  do {
    digit = counter % base;
    digit++;
    if (remainder && digit >= remainder) digit++;
    *--p = digit;
    counter /= base;
  } while (counter);
  if (remainder && digit >= remainder) *--p = 0;
  *--p = remainder;
  return p;
}

/* decode_counter (src/gqf.cu:1276-1345): returns the last slot of the
 * counter that starts at index. */
static uint64_t decode_counter(const oqf* qf, uint64_t index, uint64_t* remainder,
                               uint64_t* count) {
  uint64_t base, rem, cnt, digit, end;
  *remainder = rem = get_slot(qf, index);
  if (is_runend(qf, index)) {
    *count = 1;
    return index;
  }
  digit = get_slot(qf, index + 1);
  if (is_runend(qf, index + 1)) {
    *count = digit == rem ? 2 : 1;
    return index + (digit == rem ? 1 : 0);
  }
  if (rem > 0 && digit >= rem) {
    *count = digit == rem ? 2 : 1;
    return index + (digit == rem ? 1 : 0);
  }
  if (rem > 0 && digit == 0 && get_slot(qf, index + 2) == rem) {
    *count = 3;
    return index + 2;
  }
  if (rem == 0 && digit == 0) {
    if (get_slot(qf, index + 2) == 0) {
      *count = 3;
      return index + 2;
    } else {
      *count = 2;
      return index + 1;
    }
  }
  cnt = 0;
  base = (1ULL << 8) - (rem ? 2 : 1);
  end = index + 1;
  while (digit != rem && !is_runend(qf, end) && end + 1 < SPB * qf->nblocks) {
    if (digit > rem) digit--;
    if (digit && rem) digit--;
    cnt = cnt * base + digit;
    end++;
    digit = get_slot(qf, end);
  }
  if (rem) {
    *count = cnt + 3;
    return end;
  }
  if (is_runend(qf, end) || get_slot(qf, end + 1) != 0) {
    *count = 1;
    return index;
  }
  *count = cnt + 4;
  return end + 1;
}

/* ------------------------------------- single-key ops, src/gqf.cu:1364-1933 */

/* insert1_if_not_exists (src/gqf.cu:1364-1520) */
static int insert1_if_not_exists(oqf* qf, uint64_t hash, uint8_t* value) {
  uint64_t hash_remainder = hash & BITMASK(8);
  uint64_t hash_bucket_index = hash >> 8;
  uint64_t hash_bucket_block_offset = hash_bucket_index % SPB;
  uint64_t compare_remainder = hash_remainder; /* value_bits == 0 */

  if (is_empty(qf, hash_bucket_index)) {
    *run_word(qf, hash_bucket_index) |= 1ULL << hash_bucket_block_offset;
    set_slot(qf, hash_bucket_index, hash_remainder);
    *occ_word(qf, hash_bucket_index) |= 1ULL << hash_bucket_block_offset;
  } else {
    uint64_t runend_index = run_end(qf, hash_bucket_index);
    int operation = 0;
    uint64_t insert_index = runend_index + 1;
    uint64_t new_value = hash_remainder;
    uint64_t runstart_index = hash_bucket_index == 0 ? 0 : run_end(qf, hash_bucket_index - 1) + 1;

    if (is_occupied(qf, hash_bucket_index)) {
      uint64_t current_remainder = get_slot(qf, runstart_index);
      while (current_remainder < compare_remainder && runstart_index <= runend_index) {
        runstart_index++;
        current_remainder = get_slot(qf, runstart_index);
      }
      if (runstart_index > runend_index) {
        operation = 1;
        insert_index = runstart_index;
        new_value = hash_remainder;
      } else if (current_remainder != compare_remainder) {
        operation = 2;
        insert_index = runstart_index;
        new_value = hash_remainder;
      } else {
        /* get_slot(...) && BITMASK(value_bits) with value_bits 0: always 0
         * (src/gqf.cu:1454) */
        *value = 0;
        return 1; /* QF_ITEM_FOUND */
      }
    }

    uint64_t empty_slot_index = find_first_empty_slot(qf, runend_index + 1);
    if (empty_slot_index >= qf->xnslots) return 2; /* QF_FULL */
    shift_remainders(qf, insert_index, empty_slot_index);
    set_slot(qf, insert_index, new_value);
    shift_runends(qf, insert_index, empty_slot_index - 1, 1);
    switch (operation) {
      case 0:
        *run_word(qf, insert_index) |= 1ULL << (insert_index % SPB);
        break;
      case 1:
        *run_word(qf, insert_index - 1) &= ~(1ULL << ((insert_index - 1) % SPB));
        *run_word(qf, insert_index) |= 1ULL << (insert_index % SPB);
        break;
      case 2:
        *run_word(qf, insert_index) &= ~(1ULL << (insert_index % SPB));
        break;
    }
    uint64_t i;
    for (i = hash_bucket_index / SPB + 1; i <= empty_slot_index / SPB; i++)
      if (get_block(qf, i)->offset < 255) get_block(qf, i)->offset++;
    *occ_word(qf, hash_bucket_index) |= 1ULL << hash_bucket_block_offset;
  }
  return 0; /* QF_ITEM_INSERTED */
}

/* insert1 (src/gqf.cu:1523-1765): count 1, incrementing a counter in place
 * when the remainder is already present. */
static int insert1(oqf* qf, uint64_t hash) {
  int ret_distance = 0;
  uint64_t hash_remainder = hash & BITMASK(8);
  uint64_t hash_bucket_index = hash >> 8;
  uint64_t hash_bucket_block_offset = hash_bucket_index % SPB;

  if (is_empty(qf, hash_bucket_index)) {
    *run_word(qf, hash_bucket_index) |= 1ULL << hash_bucket_block_offset;
    set_slot(qf, hash_bucket_index, hash_remainder);
    *occ_word(qf, hash_bucket_index) |= 1ULL << hash_bucket_block_offset;
    return 0;
  }

  uint64_t runend_index = run_end(qf, hash_bucket_index);
  int operation = 0;
  uint64_t insert_index = runend_index + 1;
  uint64_t new_value = hash_remainder;
  uint64_t runstart_index = hash_bucket_index == 0 ? 0 : run_end(qf, hash_bucket_index - 1) + 1;

  if (is_occupied(qf, hash_bucket_index)) {
    uint64_t current_remainder = get_slot(qf, runstart_index);
    uint64_t zero_terminator = runstart_index;

    if (current_remainder == 0) {
      uint64_t t = runstart_index + 1;
      while (t < runend_index && get_slot(qf, t) != 0) t++;
      if (t < runend_index && get_slot(qf, t + 1) == 0)
        zero_terminator = t + 1;
      else if (runstart_index < runend_index && get_slot(qf, runstart_index + 1) == 0)
        zero_terminator = runstart_index + 1;
      if (hash_remainder != 0) {
        runstart_index = zero_terminator + 1;
        current_remainder = get_slot(qf, runstart_index);
      }
    }

    while (current_remainder < hash_remainder && runstart_index <= runend_index) {
      if (runstart_index < runend_index && get_slot(qf, runstart_index + 1) < current_remainder) {
        runstart_index = runstart_index + 2;
        while (runstart_index < runend_index && get_slot(qf, runstart_index) != current_remainder)
          runstart_index++;
        runstart_index++;
      } else {
        runstart_index++;
      }
      current_remainder = get_slot(qf, runstart_index);
    }

    if (runstart_index > runend_index) {
      operation = 1;
      insert_index = runstart_index;
      new_value = hash_remainder;
    } else if (current_remainder != hash_remainder) {
      operation = 2;
      insert_index = runstart_index;
      new_value = hash_remainder;
    } else if (runstart_index == runend_index ||
               (hash_remainder > 0 && get_slot(qf, runstart_index + 1) > hash_remainder) ||
               (hash_remainder == 0 && zero_terminator == runstart_index)) {
      operation = 2;
      insert_index = runstart_index;
      new_value = hash_remainder;
    } else if ((hash_remainder > 0 && get_slot(qf, runstart_index + 1) == hash_remainder) ||
               (hash_remainder == 0 && zero_terminator == runstart_index + 1)) {
      operation = 2;
      insert_index = runstart_index + 1;
      new_value = 0;
    } else if (hash_remainder == 0 && zero_terminator == runstart_index + 2) {
      operation = 2;
      insert_index = runstart_index + 1;
      new_value = 1;
    } else {
      insert_index = runstart_index + 1;
      while (get_slot(qf, insert_index + 1) != hash_remainder && insert_index + 1 < SPB * qf->nblocks)
        insert_index++;
      uint64_t digit, carry;
      do {
        carry = 0;
        digit = get_slot(qf, insert_index);
        if (digit == 0) {
          digit++;
          if (digit == current_remainder) digit++;
        }
        digit = (digit + 1) & BITMASK(8);
        if (digit == 0) {
          digit++;
          carry = 1;
        }
        if (digit == current_remainder) digit = (digit + 1) & BITMASK(8);
        if (digit == 0) {
          digit++;
          carry = 1;
        }
        set_slot(qf, insert_index, digit);
        insert_index--;
      } while (insert_index > runstart_index && carry);

      if (insert_index == runstart_index &&
          (carry > 0 || (current_remainder != 0 && digit >= current_remainder))) {
        operation = 2;
        insert_index = runstart_index + 1;
        if (!carry)
          new_value = 0;
        else
          new_value = 2;
      } else {
        operation = -1;
      }
    }
  }

  if (operation >= 0) {
    uint64_t empty_slot_index = find_first_empty_slot(qf, runend_index + 1);
    if (empty_slot_index >= qf->xnslots) return -1; /* QF_NO_SPACE */
    shift_remainders(qf, insert_index, empty_slot_index);
    set_slot(qf, insert_index, new_value);
    ret_distance = (int)(insert_index - hash_bucket_index);
    shift_runends(qf, insert_index, empty_slot_index - 1, 1);
    switch (operation) {
      case 0:
        *run_word(qf, insert_index) |= 1ULL << (insert_index % SPB);
        break;
      case 1:
        *run_word(qf, insert_index - 1) &= ~(1ULL << ((insert_index - 1) % SPB));
        *run_word(qf, insert_index) |= 1ULL << (insert_index % SPB);
        break;
      case 2:
        *run_word(qf, insert_index) &= ~(1ULL << (insert_index % SPB));
        break;
    }
    uint64_t i;
    for (i = hash_bucket_index / SPB + 1; i <= empty_slot_index / SPB; i++)
      if (get_block(qf, i)->offset < 255) get_block(qf, i)->offset++;
  }
  *occ_word(qf, hash_bucket_index) |= 1ULL << hash_bucket_block_offset;
  return ret_distance;
}

/* insert (src/gqf.cu:1768-1873): count > 1, re-encoding the counter. */
static int insert_count(oqf* qf, uint64_t hash, uint64_t count) {
  int ret_distance = 0;
  uint64_t hash_remainder = hash & BITMASK(8);
  uint64_t hash_bucket_index = hash >> 8;
  uint64_t hash_bucket_block_offset = hash_bucket_index % SPB;
  uint64_t runend_index = run_end(qf, hash_bucket_index);

  if (might_be_empty(qf, hash_bucket_index) && runend_index == hash_bucket_index) {
    *run_word(qf, hash_bucket_index) |= 1ULL << hash_bucket_block_offset;
    set_slot(qf, hash_bucket_index, hash_remainder);
    *occ_word(qf, hash_bucket_index) |= 1ULL << hash_bucket_block_offset;
    if (count > 1) insert_count(qf, hash, count - 1); /* src/gqf.cu:1799 */
  } else {
    uint64_t new_values[67];
    int64_t runstart_index = hash_bucket_index == 0 ? 0 : run_end(qf, hash_bucket_index - 1) + 1;
    int ret;
    if (!is_occupied(qf, hash_bucket_index)) {
      uint64_t* p = encode_counter(hash_remainder, count, &new_values[67]);
      ret = insert_replace_slots(qf, 0, hash_bucket_index, runstart_index, p,
                                 &new_values[67] - p, 0);
      if (!ret) return -1;
      ret_distance = (int)(runstart_index - hash_bucket_index);
    } else {
      uint64_t current_remainder, current_count, current_end;
      current_end = decode_counter(qf, runstart_index, &current_remainder, &current_count);
      while (current_remainder < hash_remainder && !is_runend(qf, current_end) &&
             current_end + 1 < SPB * qf->nblocks) {
        runstart_index = current_end + 1;
        current_end = decode_counter(qf, runstart_index, &current_remainder, &current_count);
      }
      if (current_remainder < hash_remainder) {
        uint64_t* p = encode_counter(hash_remainder, count, &new_values[67]);
        ret = insert_replace_slots(qf, 1, hash_bucket_index, current_end + 1, p,
                                   &new_values[67] - p, 0);
        if (!ret) return -1;
        ret_distance = (int)((current_end + 1) - hash_bucket_index);
      } else if (current_remainder == hash_remainder) {
        uint64_t* p = encode_counter(hash_remainder, current_count + count, &new_values[67]);
        ret = insert_replace_slots(qf, is_runend(qf, current_end) ? 1 : 2, hash_bucket_index,
                                   runstart_index, p, &new_values[67] - p,
                                   current_end - runstart_index + 1);
        if (!ret) return -1;
        ret_distance = (int)(runstart_index - hash_bucket_index);
      } else {
        uint64_t* p = encode_counter(hash_remainder, count, &new_values[67]);
        ret = insert_replace_slots(qf, 2, hash_bucket_index, runstart_index, p,
                                   &new_values[67] - p, 0);
        if (!ret) return -1;
        ret_distance = (int)(runstart_index - hash_bucket_index);
      }
    }
    *occ_word(qf, hash_bucket_index) |= 1ULL << hash_bucket_block_offset;
  }
  return ret_distance;
}

/* _remove (src/gqf.cu:1876-1933) */
static int remove_count(oqf* qf, uint64_t hash, uint64_t count) {
  uint64_t hash_remainder = hash & BITMASK(8);
  uint64_t hash_bucket_index = hash >> 8;
  uint64_t current_remainder, current_count, current_end;
  uint64_t new_values[67];

  if (!is_occupied(qf, hash_bucket_index)) return -1;

  uint64_t runstart_index = hash_bucket_index == 0 ? 0 : run_end(qf, hash_bucket_index - 1) + 1;
  uint64_t original_runstart_index = runstart_index;
  int only_item_in_the_run = 0;

  current_end = decode_counter(qf, runstart_index, &current_remainder, &current_count);
  while (current_remainder < hash_remainder && !is_runend(qf, current_end) &&
         current_end + 1 < SPB * qf->nblocks) {
    runstart_index = current_end + 1;
    current_end = decode_counter(qf, runstart_index, &current_remainder, &current_count);
  }
  if (current_remainder != hash_remainder) return -1;
  if (original_runstart_index == runstart_index && is_runend(qf, current_end))
    only_item_in_the_run = 1;

  uint64_t* p = encode_counter(hash_remainder, count > current_count ? 0 : current_count - count,
                               &new_values[67]);
  return remove_replace_slots(qf, only_item_in_the_run, hash_bucket_index, runstart_index, p,
                              &new_values[67] - p, current_end - runstart_index + 1);
}

/* ------------------------------------------------ keyed wrappers */

/* qf_insert (src/gqf.cu:2456-2528) with QF_KEY_IS_HASH */
int oqf_insert(oqf* qf, uint64_t hash, uint64_t count) {
  if (count == 0) return 0;
  if (count == 1) return insert1(qf, hash);
  return insert_count(qf, hash, count);
}

/* qf_remove (src/gqf.cu:3443-3458) with QF_KEY_IS_HASH */
int oqf_remove(oqf* qf, uint64_t hash, uint64_t count) {
  if (count == 0) return 1;
  return remove_count(qf, hash, count);
}

/* qf_count_key_value (src/gqf.cu:3479-3517) with QF_KEY_IS_HASH */
uint64_t oqf_count(const oqf* qf, uint64_t hash) {
  uint64_t hash_remainder = hash & BITMASK(8);
  int64_t hash_bucket_index = (int64_t)(hash >> 8);
  if (!is_occupied(qf, hash_bucket_index)) return 0;
  int64_t runstart_index = hash_bucket_index == 0 ? 0 : (int64_t)run_end(qf, hash_bucket_index - 1) + 1;
  if (runstart_index < hash_bucket_index) runstart_index = hash_bucket_index;
  uint64_t current_remainder, current_count, current_end;
  do {
    current_end = decode_counter(qf, runstart_index, &current_remainder, &current_count);
    if (current_remainder == hash_remainder) return current_count;
    runstart_index = current_end + 1;
  } while (!is_runend(qf, current_end) && (uint64_t)runstart_index < SPB * qf->nblocks);
  return 0;
}

/* qf_insert_not_exists (src/gqf.cu:2383-2453) with QF_KEY_IS_HASH, count 1.
 * Returns the qf_returns code: 0 inserted, 1 found, 2 full. */
int oqf_insert_not_exists(oqf* qf, uint64_t hash, uint8_t* retval) {
  return insert1_if_not_exists(qf, hash, retval);
}

/* qf_query (src/gqf.cu:3520-3556) with QF_KEY_IS_HASH */
uint64_t oqf_query(const oqf* qf, uint64_t hash, uint64_t* value) {
  uint64_t hash_remainder = hash & BITMASK(8);
  int64_t hash_bucket_index = (int64_t)(hash >> 8);
  *value = 0;
  if (!is_occupied(qf, hash_bucket_index)) return 0;
  int64_t runstart_index = hash_bucket_index == 0 ? 0 : (int64_t)run_end(qf, hash_bucket_index - 1) + 1;
  if (runstart_index < hash_bucket_index) runstart_index = hash_bucket_index;
  uint64_t current_remainder, current_count, current_end;
  do {
    current_end = decode_counter(qf, runstart_index, &current_remainder, &current_count);
    *value = 0; /* current_remainder & BITMASK(value_bits = 0) */
    if (current_remainder == hash_remainder) return current_count;
    runstart_index = current_end + 1;
  } while (!is_runend(qf, current_end) && (uint64_t)runstart_index < SPB * qf->nblocks);
  return 0;
}

/* ------------------------------------------------------ bulk emulation */

/* LSD radix sort on the low `bits` bits (the hashes never exceed them). */
static void radix_sort(uint64_t* data, uint64_t n, int bits) {
  if (n < 2) return;
  uint64_t* tmp = (uint64_t*)malloc(n * sizeof(uint64_t));
  uint64_t* src = data;
  uint64_t* dst = tmp;
  uint64_t cnt[2048];
  for (int shift = 0; shift < bits; shift += 11) {
    memset(cnt, 0, sizeof(cnt));
    for (uint64_t i = 0; i < n; i++) cnt[(src[i] >> shift) & 2047]++;
    uint64_t s = 0;
    for (int d = 0; d < 2048; d++) {
      uint64_t c = cnt[d];
      cnt[d] = s;
      s += c;
    }
    for (uint64_t i = 0; i < n; i++) dst[cnt[(src[i] >> shift) & 2047]++] = src[i];
    uint64_t* t = src;
    src = dst;
    dst = t;
  }
  if (src != data) memcpy(data, src, n * sizeof(uint64_t));
  free(tmp);
}

typedef enum { OP_INSERT1, OP_INSERT_COUNT, OP_REMOVE } bulk_op;

typedef struct {
  oqf* qf;
  const uint64_t* h;      /* sorted hashes */
  const uint64_t* counts; /* per-hash counts (reduce) or NULL */
  const uint64_t* start;  /* region boundaries, num_locks + 1 entries */
  bulk_op op;
  int parity, tid, nthreads;
} region_job;

static void run_region(const region_job* j, uint64_t r) {
  uint64_t a = j->start[r], b = j->start[r + 1], k;
  switch (j->op) {
    case OP_INSERT1: /* insert_from_buffers_hashed, src/gqf.cu:2759 */
      for (k = a; k < b; k++) oqf_insert(j->qf, j->h[k], 1);
      break;
    case OP_INSERT_COUNT: /* insert_from_buffers_thrust, src/gqf.cu:2806 */
      for (k = a; k < b; k++) oqf_insert(j->qf, j->h[k], j->counts[k]);
      break;
    case OP_REMOVE: /* delete_from_buffers_hashed walks backwards, src/gqf.cu:2892 */
      for (k = b; k > a; k--) oqf_remove(j->qf, j->h[k - 1], 1);
      break;
  }
}

static void* region_worker(void* arg) {
  const region_job* j = (const region_job*)arg;
  uint64_t nl = j->qf->num_locks;
  uint64_t r = (uint64_t)j->parity + 2ULL * (uint64_t)j->tid;
  for (; r < nl; r += 2ULL * (uint64_t)j->nthreads) run_region(j, r);
  return NULL;
}

/* set_buffers_binary / set_buffer_lens (src/gqf.cu:2646-2750): region r
 * holds the sorted hashes with quotient in [8192 r, 8192 (r+1)). */
static void region_bounds(const oqf* qf, const uint64_t* h, uint64_t n, uint64_t* start) {
  uint64_t i = 0;
  for (uint64_t r = 0; r < qf->num_locks; r++) {
    while (i < n && (h[i] >> 8) < REGION_SLOTS * r) i++;
    start[r] = i;
  }
  start[qf->num_locks] = n;
}

static void run_even_odd(oqf* qf, const uint64_t* h, const uint64_t* counts, uint64_t n,
                         bulk_op op, int nthreads) {
  uint64_t* start = (uint64_t*)malloc((qf->num_locks + 1) * sizeof(uint64_t));
  region_bounds(qf, h, n, start);
  if (nthreads < 1) nthreads = 1;
  for (int parity = 0; parity < 2; parity++) {
    region_job jobs[256];
    pthread_t th[256];
    int nt = nthreads > 256 ? 256 : nthreads;
    for (int t = 0; t < nt; t++) {
      jobs[t].qf = qf; jobs[t].h = h; jobs[t].counts = counts; jobs[t].start = start;
      jobs[t].op = op; jobs[t].parity = parity; jobs[t].tid = t; jobs[t].nthreads = nt;
    }
    if (nt == 1) {
      region_worker(&jobs[0]);
    } else {
      for (int t = 0; t < nt; t++) pthread_create(&th[t], NULL, region_worker, &jobs[t]);
      for (int t = 0; t < nt; t++) pthread_join(th[t], NULL);
    }
  }
  free(start);
}

/* hash_all (src/gqf.cu:2615-2640) into a fresh array, then thrust::sort. */
static uint64_t* hash_and_sort(const oqf* qf, uint64_t n, const uint64_t* keys, int key_is_hash) {
  uint64_t* h = (uint64_t*)malloc((n ? n : 1) * sizeof(uint64_t));
  uint64_t mask = BITMASK(qf->key_bits);
  for (uint64_t i = 0; i < n; i++) h[i] = key_is_hash ? keys[i] : oqf_hash64(keys[i], mask);
  int bits = key_is_hash ? 64 : (int)qf->key_bits;
  radix_sort(h, n, bits);
  return h;
}

/* bulk_insert (src/gqf.cu:3184-3232) */
void oqf_bulk_insert(oqf* qf, uint64_t n, const uint64_t* keys, int key_is_hash, int nthreads) {
  uint64_t* h = hash_and_sort(qf, n, keys, key_is_hash);
  run_even_odd(qf, h, NULL, n, OP_INSERT1, nthreads);
  free(h);
}

/* bulk_insert_reduce (src/gqf.cu:3238-3313): reduce_by_key on the sorted
 * hashes, then insert each unique hash with its multiplicity. */
void oqf_bulk_insert_reduce(oqf* qf, uint64_t n, const uint64_t* keys, int key_is_hash,
                            int nthreads) {
  uint64_t* h = hash_and_sort(qf, n, keys, key_is_hash);
  uint64_t* c = (uint64_t*)malloc((n ? n : 1) * sizeof(uint64_t));
  uint64_t u = 0;
  for (uint64_t i = 0; i < n;) {
    uint64_t j = i;
    while (j < n && h[j] == h[i]) j++;
    h[u] = h[i];
    c[u] = j - i;
    u++;
    i = j;
  }
  run_even_odd(qf, h, c, u, OP_INSERT_COUNT, nthreads);
  free(c);
  free(h);
}

/* bulk_delete (src/gqf.cu:3316-3363) */
void oqf_bulk_delete(oqf* qf, uint64_t n, const uint64_t* keys, int key_is_hash, int nthreads) {
  uint64_t* h = hash_and_sort(qf, n, keys, key_is_hash);
  run_even_odd(qf, h, NULL, n, OP_REMOVE, nthreads);
  free(h);
}

typedef struct {
  const oqf* qf;
  const uint64_t* keys;
  uint64_t* out;
  uint64_t lo, hi, misses;
} get_job;

static void* get_worker(void* arg) {
  get_job* j = (get_job*)arg;
  uint64_t mask = BITMASK(j->qf->key_bits), m = 0;
  for (uint64_t i = j->lo; i < j->hi; i++) {
    uint64_t c = oqf_count(j->qf, oqf_hash64(j->keys[i], mask));
    if (j->out) j->out[i] = c;
    if (c < 1) m++;
  }
  j->misses = m;
  return NULL;
}

static uint64_t run_gets(const oqf* qf, uint64_t n, const uint64_t* keys, uint64_t* out,
                         int nthreads) {
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 256) nthreads = 256;
  get_job jobs[256];
  pthread_t th[256];
  for (int t = 0; t < nthreads; t++) {
    jobs[t].qf = qf; jobs[t].keys = keys; jobs[t].out = out;
    jobs[t].lo = n * (uint64_t)t / nthreads;
    jobs[t].hi = n * (uint64_t)(t + 1) / nthreads;
    jobs[t].misses = 0;
  }
  if (nthreads == 1) {
    get_worker(&jobs[0]);
  } else {
    for (int t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, get_worker, &jobs[t]);
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
  }
  uint64_t m = 0;
  for (int t = 0; t < nthreads; t++) m += jobs[t].misses;
  return m;
}

/* bulk_get (src/gqf.cu:3386-3401): hashes inside qf_count_key_value */
void oqf_bulk_get(const oqf* qf, uint64_t n, const uint64_t* keys, uint64_t* out, int nthreads) {
  run_gets(qf, n, keys, out, nthreads);
}

/* bulk_get_misses_wrapper (src/gqf.cu:3404-3419): count of keys with
 * count < 1 */
uint64_t oqf_bulk_get_misses(const oqf* qf, uint64_t n, const uint64_t* keys, int nthreads) {
  return run_gets(qf, n, keys, NULL, nthreads);
}
