/*
 * knn_gb300_f64.h -- status-returning C API of the double-precision library
 * (libknngb300_double.so).  That library also exports the reference's names
 * with knntype = double (include/cuknns.h compiled with __DOUBLE__), as the
 * reference's libcuknn_double.a does (Makefile:60-64).
 *
 * Results are the exact FP64 top-k by (direct-difference distance, index):
 * FP32 tensor-core candidates, FP64 re-rank, a per-query proof that the
 * shortlist holds the FP64 top-k, and an FP64 search for queries without one.
 * k <= 512.  Layouts as in knn_gb300.h.
 */
#ifndef KNN_GB300_F64_H
#define KNN_GB300_F64_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Device buffers; synchronises `stream` (it reports kernel-side timeouts). */
int knns_search_device_f64(const double *corpus, int64_t N, int64_t ldc, const double *queries, int64_t Q,
                           int64_t ldq, int D, int k, double *dist, int32_t *idx, void *stream);

/* Host buffers: copies in, searches, copies out, synchronises. */
int knns_search_host_f64(const double *corpus, int64_t N, const double *queries, int64_t Q, int D, int k,
                         double *dist, int32_t *idx);

/* Message for the last error raised on the calling thread by this library. */
const char *knns_f64_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* KNN_GB300_F64_H */
