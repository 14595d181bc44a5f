/*
 * gqf.h -- C ABI of the GB300 counting quotient filter (libgqf_gb300.so).
 *
 * Drop-in for the host half of PASSIONLab/cqf's GQF API (include/gqf.cuh of
 * the reference, whose extern "C" block opens at include/gqf.cuh:19).  Every
 * entry point below names the reference declaration it replaces.  Plain C:
 * pointers, sizes and integers only, so it binds from C, C++, cgo, ctypes or
 * JNI without CUDA headers.  Device pointers are passed as ordinary pointers.
 *
 * Semantics kept from the reference:
 *   - qf_malloc_device returns a DEVICE pointer to the filter descriptor; the
 *     host must not dereference it (src/gqf.cu:2212-2217).
 *   - Keys are 64-bit; with QF_KEY_IS_HASH clear they are hashed with the
 *     reference's invertible hash_64 under 2^(nbits+8)-1, so two keys that
 *     agree modulo 2^(nbits+8) are the same key (src/hashutil.cu:132).
 *   - Bulk calls are asynchronous on the filter's stream (the legacy default
 *     stream unless gqf_set_stream is called), like the reference's.
 *   - The layout after any sequence of calls is word-for-word the reference's
 *     (gqf_export gives the reference's packed bytes).
 *
 * Differences, all documented at the entry points:
 *   - bulk_insert / bulk_insert_reduce / bulk_delete leave `keys` unmodified
 *     (the reference overwrote them with sorted hashes, src/gqf.cu:3206-3209;
 *     every caller in the reference regenerates keys afterwards).
 *   - Failures never print, assert or trap on the device: they accumulate in
 *     a status word read with gqf_get_status.
 */
#ifndef GQF_GB300_H
#define GQF_GB300_H

#include <stdbool.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* include/gqf.cuh:22-23 */
typedef struct quotient_filter quotient_filter;
typedef quotient_filter QF;

/* include/gqf.cuh:45-49 */
enum qf_hashmode { QF_HASH_DEFAULT, QF_HASH_INVERTIBLE, QF_HASH_NONE };

/* include/gqf.cuh:52-56; QF_TIMEOUT is new: a bounded lock wait gave up. */
enum qf_returns { QF_ITEM_INSERTED, QF_ITEM_FOUND, QF_FULL, QF_TIMEOUT };

/* include/gqf.cuh:74-80 */
#define QF_NO_LOCK (0x01)
#define QF_TRY_ONCE_LOCK (0x02)
#define QF_WAIT_FOR_LOCK (0x04)
#define QF_KEY_IS_HASH (0x08)

/* include/gqf.cuh:213-215 */
#define QF_NO_SPACE (-1)
#define QF_COULDNT_LOCK (-2)
#define QF_DOESNT_EXIST (-3)

/* Status bits returned by gqf_get_status. */
#define GQF_STATUS_FULL (1u << 0)     /* an insert found no free slot (keys dropped) */
#define GQF_STATUS_TIMEOUT (1u << 1)  /* a bounded device wait gave up */
#define GQF_STATUS_BAD_KEY (1u << 2)  /* a QF_KEY_IS_HASH key >= 2^(nbits+8) was skipped */
#define GQF_STATUS_DEFERRED (1u << 3) /* a region took the serial path (informational) */
#define GQF_STATUS_OVERFLOW (1u << 4) /* an internal limit was exceeded */

/* ----------------------------------------------------------- reference API */

/* include/gqf.cuh:87.  2^nbits slots, 8-bit remainders.  bulk_config is
 * accepted for compatibility; both the bulk and the point paths are ready.
 * On failure *qf is set to NULL and gqf_last_error() says why. */
void qf_malloc_device(QF** qf, int nbits, bool bulk_config);

/* include/gqf.cuh:88 */
void qf_destroy_device(QF* qf);

/* include/gqf.cuh:109.  Inserts nvals device-resident keys (count 1 each). */
void bulk_insert(QF* qf, uint64_t nvals, uint64_t* keys, uint8_t flags);

/* include/gqf.cuh:112.  Same result as bulk_insert; for skewed batches:
 * equal keys are merged into counts on the device before they are inserted
 * (the reference sorts and runs reduce_by_key, src/gqf.cu:3238-3313). */
void bulk_insert_reduce(QF* qf, uint64_t nvals, uint64_t* keys, uint8_t flags);

/* include/gqf.cuh:115.  Decrements each key's count by one (absent keys are
 * ignored; a count reaching 0 removes the key). */
void bulk_delete(QF* qf, uint64_t nvals, uint64_t* keys, uint8_t flags);

/* include/gqf.cuh:118.  returns[i] = count of vals[i] (0 if absent). */
void bulk_get(QF* qf, uint64_t nvals, uint64_t* vals, uint64_t* returns);

/* include/gqf.cuh:136.  Number of vals with count < 1; synchronises. */
uint64_t bulk_get_misses_wrapper(QF* qf, uint64_t* vals, uint64_t nvals);

/* include/gqf.cuh:128.  Point-API lookups of nitems keys; returns the number
 * not found; synchronises. */
uint64_t point_get_wrapper(QF* qf, uint64_t* hashes, uint64_t nitems);

/* ------------------------------------------------------------- extensions */

/* Host launcher for the reference's point_bulk_insert kernel
 * (include/gqf.cuh:130, src/gqf.cu:3153): point_insert per key, keys hashed. */
int gqf_point_bulk_insert(QF* qf, uint64_t* keys, uint64_t nitems);

/* Batched point-API calls, one device thread per key (the reference's
 * point_insert / point_insert_not_exists / point_query(_concurrent),
 * include/gqf.cuh:94-103).  rets / vals / counts are device arrays. */
int gqf_point_insert_batch(QF* qf, const uint64_t* keys, uint64_t n, uint8_t flags, int8_t* rets);
int gqf_point_insert_not_exists_batch(QF* qf, const uint64_t* keys, uint64_t n, uint8_t flags,
                                      int8_t* rets, uint8_t* vals);
int gqf_point_query_batch(QF* qf, const uint64_t* keys, uint64_t n, uint8_t flags, int concurrent,
                          uint64_t* counts);

/* Asynchronous bulk calls with an explicit CUDA stream (cudaStream_t passed
 * as void*; NULL = legacy default stream).  The plain entry points above use
 * the filter's stream. */
int gqf_bulk_insert_async(QF* qf, uint64_t nvals, const uint64_t* keys, uint8_t flags, void* stream);
int gqf_bulk_insert_reduce_async(QF* qf, uint64_t nvals, const uint64_t* keys, uint8_t flags,
                                 void* stream);
int gqf_bulk_delete_async(QF* qf, uint64_t nvals, const uint64_t* keys, uint8_t flags, void* stream);

/* No counterpart in the reference's bulk API: its k-mer counting
 * (src/gqf_verify.cu:117-245) cuts ASCII k-mers on the host and hashes each
 * string.  Here the reads stay on the device: nreads fixed-length reads of
 * read_len bytes (ACGT, either case), k in [1, 32], read_len - k + 1 <= 4096.
 * Each k-mer is 2-bit packed (A=0 C=1 G=2 T=3, first base in the high bits)
 * and canonicalised (the smaller of the k-mer and its reverse complement);
 * windows holding another byte are skipped.
 *   gqf_bulk_insert_kmers: bulk_insert_reduce of the reads' canonical k-mers.
 *   gqf_kmers_extract:     out[read * (read_len - k + 1) + pos] = the k-mer at
 *                          pos, or UINT64_MAX for a skipped window.
 * reads and out are device pointers; stream as above.  Returns 0 or -1. */
int gqf_bulk_insert_kmers(QF* qf, const uint8_t* reads, uint64_t nreads, uint32_t read_len, uint32_t k,
                          void* stream);
int gqf_kmers_extract(const uint8_t* reads, uint64_t nreads, uint32_t read_len, uint32_t k, uint64_t* out,
                      void* stream);
int gqf_bulk_get_async(QF* qf, uint64_t nvals, const uint64_t* vals, uint64_t* returns, uint8_t flags,
                       void* stream);

/* No counterpart in the reference.  bulk_insert for callers that must not
 * allocate device memory while they run (a process whose device budget is
 * fixed at start-up, a plugin whose host framework owns all device memory, a
 * loop that cannot take cudaMalloc's implicit synchronisation).  Same result
 * as bulk_insert, with the same key-by-key threshold (gqf_set_sparse_max); it
 * calls no allocator.  It runs on `stream`: NULL means the legacy default
 * stream, as for the other *_async calls, not the filter's stream set by
 * gqf_set_stream.  The current device must be the filter's own (the device
 * current at qf_malloc_device); otherwise the call is refused with -1.  The
 * batch is partitioned into one fixed array of GQF_NOALLOC_SCRATCH_BYTES
 * inside the library's device image, held by every GPU that loads the
 * library: a batch may hold at most
 *   (GQF_NOALLOC_SCRATCH_BYTES - 20 * (nslots / 2^region_log + 2), rounded up
 *    to 256) / 4 keys
 * (about 3.87 million at 2^28 slots with the default 2^12-quotient regions,
 * 4.03 million with gqf_set_region_log 13); larger batches are refused with
 * -1 and a message in gqf_last_error.  The first call on each device, with
 * that device current, looks up the array's address: make it before any
 * stream capture.  All calls share the array, so calls that overlap on the
 * GPU race and must be serialised by the caller.  Returns 0 on success. */
#define GQF_NOALLOC_SCRATCH_BYTES (16u << 20)
int gqf_bulk_insert_noalloc(QF* qf, uint64_t nvals, const uint64_t* keys, uint8_t flags, void* stream);

/* ------------------------------------------------------------ serving loop
 * No counterpart in the reference (its bulk calls run one at a time on the
 * caller's device buffers).  A server keeps one filter resident and runs
 * requests submitted from any host thread through a staging ring of
 * staging_bytes in device memory (0 = a quarter of the free memory, at most
 * 4 GiB): requests are admitted in arrival order as ring space frees up,
 * consecutive requests of one kind (gets; inserts and counted inserts;
 * deletes; QF_KEY_IS_HASH batches apart) run as one launch, and the copies of
 * later launches overlap the compute of earlier ones.  Every request's result
 * equals running the requests one by one in submission order.
 *
 * gqf_server_submit: op is GQF_OP_*; keys (and, for a get, counts: n
 *   uint64 results) are host pointers -- pinned memory lets the copies run
 *   asynchronously -- or device pointers with GQF_SERVE_DEVICE_PTRS in
 *   flags; QF_KEY_IS_HASH may be or-ed in.  Buffers must stay valid until the
 *   request completes.  Returns a ticket >= 0, or -1.
 * gqf_server_poll: 1 done, 0 pending, -1 failed / unknown ticket.
 * gqf_server_wait: blocks until done, frees the ticket, and stores the
 *   request's latency (submission to completion, ms); 0 or -1.
 * gqf_server_drain: waits until nothing is queued or in flight.
 * gqf_server_stats: out[0..7] = requests completed, launches, keys, p50 ms,
 *   p99 ms, max ms, staging bytes, peak staging bytes in use.
 * While a server runs, other calls on its filter must not overlap it. */
typedef struct gqf_server gqf_server;
#define GQF_OP_GET 0
#define GQF_OP_INSERT 1
#define GQF_OP_DELETE 2
#define GQF_OP_INSERT_REDUCE 3
#define GQF_SERVE_DEVICE_PTRS (1u << 8)
#define GQF_SERVE_STATS 8
int gqf_server_create(QF* qf, uint64_t staging_bytes, gqf_server** out);
int64_t gqf_server_submit(gqf_server* s, int op, const uint64_t* keys, uint64_t n, uint64_t* counts,
                          uint32_t flags);
int gqf_server_poll(gqf_server* s, int64_t ticket);
int gqf_server_wait(gqf_server* s, int64_t ticket, double* latency_ms);
int gqf_server_drain(gqf_server* s);
int gqf_server_stats(gqf_server* s, double* out, int n);
int gqf_server_reset_stats(gqf_server* s);
void gqf_server_destroy(gqf_server* s);

/* ---------------------------------------------- enumeration and set algebra
 * The reference's iterator and the operations built on it, run on the GPU
 * (host-only in the reference: qfi_get_hash / qfi_get_key / qfi_next,
 * src/gqf.cu:3774-3893; qf_merge :3896; qf_multi_merge :3945;
 * qf_inner_product :4010; qf_intersect :4047).  All take device filters,
 * synchronise, and leave their inputs unchanged.
 *   gqf_enumerate: every (hash, count) in increasing hash order, the
 *     iterator's order, into device arrays of `cap` entries (counts may be
 *     NULL); *n gets the number of pairs.  hashes = NULL only counts them.
 *     as_keys reports keys (the inverse hash, as qfi_get_key does for the
 *     invertible hash) instead of hashes.  Tables up to 2^31 slots.
 *   gqf_merge / gqf_multi_merge: inserts every pair of the inputs into `out`
 *     (as hashes, like the reference); `out` may be one of the inputs.
 *   gqf_intersect: the pairs of the larger input (by table size, ties to b)
 *     whose hash the other input holds, inserted into `out`.
 *   gqf_inner_product: sum over the larger input's pairs of count times the
 *     other input's count of the same hash (0 on error).
 * Counters above 2^32 - 1 cannot be carried into `out` (-1). */
int gqf_enumerate(QF* qf, uint64_t* hashes, uint64_t* counts, uint64_t cap, uint64_t* n, int as_keys);
int gqf_merge(QF* a, QF* b, QF* out);
int gqf_multi_merge(QF* const* in, int nin, QF* out);
int gqf_intersect(QF* a, QF* b, QF* out);
uint64_t gqf_inner_product(QF* a, QF* b);

/* Resize: replaces qf_resize_malloc / qf_resize (src/gqf.cu:2301-2372, host
 * filters only in the reference).  Grows the table to 2^new_nbits slots under
 * the same QF handle and re-inserts every stored key with its count (counted
 * rebuild); synchronises.  The reference keeps key_bits, so its resized
 * filter stores narrower remainders (a 2^20-slot filter with 28 key bits
 * resized to 2^21 slots keeps 7-bit remainders); this filter's slots are 8
 * bits, so key_bits grows with the table (new_nbits + 8) and the false-
 * positive rate stays that of a filter built at the new size.  Stored keys
 * are recovered through the invertible hash, as qfi_get_key does, modulo
 * 2^(nbits + 8): keys that fit those bits give exactly the filter built at
 * the new size from the same multiset; wider keys keep their low bits (keys
 * that collided stay merged).  new_nbits in [nbits, 36]; counters above
 * 2^32 - 1 cannot be carried (-1).  On -1 after the old table was released,
 * the filter is left empty at the new size. */
int gqf_resize(QF* qf, int new_nbits);

/* ------------------------------------------------------------- filter sets
 * No counterpart in the reference (one QF handle per filter, one bulk call
 * sequence per filter).  A set holds n independent filters (filter f has
 * 2^nbits[f] slots) in one device arena; a batch for all of them is one
 * array of device keys with device CSR offsets (offsets[0] = 0, filter f
 * owns keys[offsets[f] .. offsets[f+1]), offsets[n] = total) and runs as one
 * partition pass, one rebuild launch per parity and one probe launch.  Each
 * filter's contents, counts and exported bytes equal those of a QF of the
 * same size given the same keys.  Scratch for max_batch_keys keys is
 * allocated at creation; the operations allocate nothing and only enqueue
 * work on `stream`, so they can be captured into a CUDA graph (make one
 * call of each kind before capturing: the first call configures kernels).
 *   gqf_set_tune:   times inserts of the given batch under each region size
 *                   and key-by-key setting, keeps the fastest, and leaves the
 *                   set empty; *best_ms gets the best time.
 *   gqf_set_config: region size (11, 12, 13) and key-by-key threshold
 *                   (as gqf_set_sparse_max; GQF_SPARSE_AUTO by default).
 *   gqf_set_export: filter i in the reference's packed format (as gqf_export).
 * Returns 0, or -1 with gqf_last_error set. */
typedef struct gqf_set gqf_set;
int gqf_set_create(uint32_t n, const int* nbits, uint64_t max_batch_keys, gqf_set** out);
void gqf_set_destroy(gqf_set* s);
int gqf_set_insert(gqf_set* s, const uint64_t* keys, const uint64_t* offsets, uint64_t total, uint8_t flags,
                   void* stream);
int gqf_set_delete(gqf_set* s, const uint64_t* keys, const uint64_t* offsets, uint64_t total, uint8_t flags,
                   void* stream);
int gqf_set_get(gqf_set* s, const uint64_t* keys, const uint64_t* offsets, uint64_t total, uint64_t* counts,
                uint8_t flags, void* stream);
int gqf_set_reset(gqf_set* s, void* stream);
int gqf_set_tune(gqf_set* s, const uint64_t* keys, const uint64_t* offsets, uint64_t total, uint8_t flags,
                 double* best_ms);
int gqf_set_config(gqf_set* s, int log_region, uint32_t sparse_max);
int gqf_set_get_config(gqf_set* s, int* log_region, uint32_t* sparse_max);
uint64_t gqf_set_export_size(gqf_set* s, uint32_t i);
int gqf_set_export(gqf_set* s, uint32_t i, uint8_t* out, uint64_t size);
int gqf_set_get_status(gqf_set* s, uint32_t* status);

/* The filter's default stream for the reference entry points. */
int gqf_set_stream(QF* qf, void* stream);

/* Files (the reference declares qf_serialize / qf_deserialize,
 * include/gqf_file.cuh:46-49, for host filters): the gqf_export image (the
 * reference's 120-byte metadata and packed 81-byte blocks) written to or read
 * from `path`.  gqf_deserialize allocates a filter of the image's size into
 * *qf.  Both return the bytes written / read, 0 on error. */
uint64_t gqf_serialize(QF* qf, const char* path);
uint64_t gqf_deserialize(QF** qf, const char* path);

/* Point-API lock waits: a lock is tried at most max_spins times (with
 * growing sleeps, up to about a microsecond each) before the operation gives
 * up with QF_TIMEOUT and sets GQF_STATUS_TIMEOUT.  Default 2^20.  The
 * reference spins without a bound (lock_16, src/gqf.cu:2534). */
int gqf_set_lock_wait(QF* qf, uint32_t max_spins);
/* Test hook: marks point-API lock `lock_index` (8192-slot region) held or
 * free, as a thread that died holding it would leave it. */
int gqf_debug_hold_lock(QF* qf, uint64_t lock_index, int held);

/* Region size of the bulk rebuild: 2^log_region quotients (11, 12 or 13).
 * Does not change results, only speed; 0 restores the automatic choice. */
int gqf_set_region_log(QF* qf, int log_region);
int gqf_get_region_log(QF* qf);

/* Regions that receive at most max_keys keys of a batch are updated key by
 * key (the reference's single-key algorithms, one thread per region) instead
 * of rebuilt; 0 rebuilds every touched region; GQF_SPARSE_AUTO (the default)
 * picks nregions / 1400 clamped to [16, 256], for batches averaging at most
 * half that per region (denser batches rebuild every region).  Does not
 * change results, only speed.  gqf_get_sparse_max returns the threshold. */
#define GQF_SPARSE_AUTO 0xFFFFFFFFu
int gqf_set_sparse_max(QF* qf, uint32_t max_keys);
int64_t gqf_get_sparse_max(QF* qf);

/* Geometry: 2^nbits slots, xnslots = nslots + 10 sqrt(nslots) slots in
 * 64-slot blocks (qf_init, src/gqf.cu:1939-1996). */
uint64_t gqf_nslots(QF* qf);
uint64_t gqf_xnslots(QF* qf);
uint64_t gqf_nblocks(QF* qf);
/* Device bytes held by the filter's blocks. */
uint64_t gqf_device_bytes(QF* qf);

/* Status word (GQF_STATUS_*) accumulated since the last clear; synchronises
 * the filter's stream.  Returns 0 on success, nonzero on a CUDA error. */
int gqf_get_status(QF* qf, uint32_t* status);
int gqf_clear_status(QF* qf);

/* Counters since the last gqf_clear_status: [0] regions whose rebuild window
 * was exceeded (applied by the serial path), [1] keys applied serially,
 * [2] regions rebuilt in the full window (the region plus 2048 slots, 1024
 * for 2048-quotient regions) because the first window (the region plus 256
 * slots) could not hold their changes.  Writes min(n, 3) values;
 * synchronises the filter's stream. */
int gqf_get_counters(QF* qf, uint64_t* counters, int n);

/* Empty the filter (asynchronous). */
int gqf_reset(QF* qf);

/* The reference's packed format: the 120-byte qfmetadata header then nblocks
 * 81-byte qfblocks (include/gqf_int.cuh:38-113), exactly the buffer the
 * reference's filter would hold after the same operations.  export_size is
 * the byte count; export writes to a host buffer and synchronises. */
uint64_t gqf_export_size(QF* qf);
int gqf_export(QF* qf, void* host_buf, uint64_t len);
/* Load a packed image (same nbits) into the filter; synchronises. */
int gqf_import(QF* qf, const void* host_buf, uint64_t len);

/* Phase timers: with profiling on, every bulk call brackets its phases with
 * CUDA events on its stream.  gqf_profile_read synchronises and returns, per
 * phase, the summed device milliseconds, the number of calls and the keys
 * processed since profiling was enabled (arrays of GQF_PROF_PHASES). */
#define GQF_PROF_PARTITION 0 /* hash + radix partition by region */
#define GQF_PROF_INSERT 1    /* region rebuild for inserts (both phases + fallback) */
#define GQF_PROF_DELETE 2    /* region rebuild for deletes */
#define GQF_PROF_GET 3       /* probe kernel */
#define GQF_PROF_PHASES 8
int gqf_profile(QF* qf, int enable);
int gqf_profile_read(QF* qf, double* ms, uint64_t* calls, uint64_t* keys);

/* Kernels launched by the library since it was loaded (all filters). */
uint64_t gqf_launch_count(void);

/* Testing support: apply hashes one at a time with the reference's
 * single-key algorithms on the device (op 0 insert count 1, 1 remove one). */
int gqf_debug_serial_apply(QF* qf, const uint64_t* hashes, uint64_t n, int op);

/* Last host-side error message of the calling thread ("" if none). */
const char* gqf_last_error(void);

/* Library version string. */
const char* gqf_version(void);

#ifdef __cplusplus
}
#endif
#endif /* GQF_GB300_H */
