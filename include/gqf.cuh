/*
 * gqf.cuh -- CUDA view of the GB300 counting quotient filter.
 *
 * The reference's include/gqf.cuh exported, besides the host API in gqf.h,
 * device functions that user kernels call directly (include/gqf.cuh:94-103)
 * and the point_bulk_insert kernel (include/gqf.cuh:130).  They are defined
 * in libgqf_gb300_device.a (relocatable device code); link it with
 * `nvcc -rdc=true ... -lgqf_gb300_device`, as the reference's callers linked
 * gqf.o (Makefile:35).
 *
 * Every lock wait is bounded: an operation that cannot take its locks returns
 * QF_TIMEOUT (point_query_concurrent returns 0) and sets GQF_STATUS_TIMEOUT.
 */
#ifndef GQF_GB300_CUH
#define GQF_GB300_CUH

#include "gqf.h"

#ifdef __CUDACC__
#ifdef __cplusplus
extern "C" {
#endif

/* include/gqf.cuh:94: insert one key (count + 1) under the region locks. */
__device__ qf_returns point_insert(QF* qf, uint64_t key, uint8_t value, uint8_t flags);

/* include/gqf.cuh:97: QF_ITEM_FOUND if present (no increment), else insert. */
__device__ qf_returns point_insert_not_exists(QF* qf, uint64_t key, uint8_t value,
                                              uint8_t& returnedVal, uint8_t flags);

/* include/gqf.cuh:100: count of key, no locks. */
__device__ uint64_t point_query(QF* qf, uint64_t key, uint8_t value, uint8_t& returnedVal,
                                uint8_t flags);

/* include/gqf.cuh:103: count of key under the region locks. */
__device__ uint64_t point_query_concurrent(QF* qf, uint64_t key, uint8_t value,
                                           uint8_t& returnedVal, uint8_t flags);

/* include/gqf.cuh:130 */
__global__ void point_bulk_insert(QF* qf, uint64_t* hashes, uint64_t nitems);

#ifdef __cplusplus
}
#endif
#endif /* __CUDACC__ */
#endif /* GQF_GB300_CUH */
