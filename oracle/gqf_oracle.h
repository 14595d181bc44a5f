/* CPU oracle for the GQF bulk hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * counting quotient filter (PASSIONLab/cqf, src/gqf.cu and src/hashutil.cu)
 * on the reference's own storage format: packed 81-byte blocks
 * (include/gqf_int.cuh:38-57) behind a 120-byte metadata header
 * (include/gqf_int.cuh:96-113).  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py may load it, and only as the test oracle or a
 * timed CPU baseline; the product never calls it.
 *
 * Pinned against the reference itself: tests/test_oracle.py compares it word
 * for word with oracle/_ref (the reference compiled from its sources here,
 * x86 only) and with the committed fixtures under tests/golden/.
 */
#ifndef GQF_ORACLE_H
#define GQF_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oqf oqf;

/* Sizing follows qf_init (src/gqf.cu:1939-1996) for qf_malloc_device's
 * parameters: 2^nbits slots, key_bits = nbits + 8, value_bits = 0. */
oqf* oqf_new(int nbits);
void oqf_free(oqf* qf);
uint64_t oqf_nslots(const oqf* qf);
uint64_t oqf_xnslots(const oqf* qf);
uint64_t oqf_nblocks(const oqf* qf);
uint64_t oqf_range(const oqf* qf);
/* 120-byte metadata + nblocks * 81 bytes, identical to the reference buffer. */
uint64_t oqf_total_bytes(const oqf* qf);
uint64_t oqf_dump(const oqf* qf, uint8_t* out, uint64_t len);
/* Replace the filter contents with a dump (same nbits). Returns 0 on success. */
int oqf_load(oqf* qf, const uint8_t* in, uint64_t len);

uint64_t oqf_hash64(uint64_t key, uint64_t mask);   /* hash_64, src/hashutil.cu:132 */
uint64_t oqf_hash64i(uint64_t key, uint64_t mask);  /* hash_64i, src/hashutil.cu:146 */
void oqf_splitmix64(uint64_t seed, uint64_t n, uint64_t* out);

/* Single-hash operations with QF_NO_LOCK | QF_KEY_IS_HASH semantics. */
int oqf_insert(oqf* qf, uint64_t hash, uint64_t count);  /* qf_insert, src/gqf.cu:2456 */
int oqf_remove(oqf* qf, uint64_t hash, uint64_t count);  /* qf_remove, src/gqf.cu:3443 */
uint64_t oqf_count(const oqf* qf, uint64_t hash);        /* qf_count_key_value, :3479 */
int oqf_insert_not_exists(oqf* qf, uint64_t hash, uint8_t* retval); /* :2383 */
uint64_t oqf_query(const oqf* qf, uint64_t hash, uint64_t* value);  /* qf_query, :3520 */

/* Bulk operations as the reference's bulk API performs them (hash, sort,
 * 8192-slot regions, even regions then odd ones).  nthreads > 1 runs the
 * regions of one parity on that many threads, the way the reference's
 * device launch runs them concurrently. */
void oqf_bulk_insert(oqf* qf, uint64_t n, const uint64_t* keys, int key_is_hash, int nthreads);
void oqf_bulk_insert_reduce(oqf* qf, uint64_t n, const uint64_t* keys, int key_is_hash,
                            int nthreads);
void oqf_bulk_delete(oqf* qf, uint64_t n, const uint64_t* keys, int key_is_hash, int nthreads);
void oqf_bulk_get(const oqf* qf, uint64_t n, const uint64_t* keys, uint64_t* out, int nthreads);
uint64_t oqf_bulk_get_misses(const oqf* qf, uint64_t n, const uint64_t* keys, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
