/*
 * cuknns.h -- drop-in C API with the reference's names and signatures.
 *
 * Each declaration below replaces the reference declaration cited beside it
 * (paths within shengren/knn-toolbox).  The float library (libknngb300.so)
 * exports them with knntype = float, as the reference's libcuknn.a does
 * (Makefile:51-57).  Layouts are the reference's: corpus and queries with D
 * as the leading dimension, outputs with k as the leading dimension, indices
 * 0-based and stored as knntype (readme.txt:61-69).  Unlike the reference,
 * results come back sorted ascending by (distance, index), k need not be a
 * power of two, and failures are reported through knns_last_error()
 * (include/knn_gb300.h) instead of being silent.
 */
#ifndef CUKNNS_GB300_DROPIN_H
#define CUKNNS_GB300_DROPIN_H

#ifndef __DOUBLE__
typedef float knntype;
#else
typedef double knntype;
#endif

/* include/cuknns.h:14-16 */
#define MEMTEST_ONLY 10
#define EXACT_KNN 5
#define FORCE_SINGLE_STREAM -5

#ifdef __cplusplus
extern "C" {
#endif

/* include/cuknns.h:18 -- algorithm entry point type stored in a plan */
typedef double (*knnptr2function)(knntype *, knntype *, knntype *, knntype *, int, int, int, int, int);

/* include/cuknns.h:34-41 -- plan; binary layout kept.  numStreams is an
   opaque hint here: the tuned configuration lives in the library's plan
   cache, keyed by (objects, numQueries, dimentions, k). */
typedef struct {
    knnptr2function pt2Function;
    int objects;
    int numQueries;
    int dimentions;
    int k;
    int numStreams;
} knnplan;

/* include/cuknns.h:43-47 */
typedef struct {
    double dst_time;
    double srch_time;
    double knn_time;
} knntimes;

/* include/cuknns.h:75 (src/cuknnBitonic.cu:422) -- returns elapsed seconds
   (host-to-device copies, search and device-to-host copies), FLT_MAX on failure */
double gpuknnsBitonic(knntype *query, knntype *data, knntype *values, knntype *indices, int objects,
                      int numQueries, int attributes, int k, int numStreams);

/* include/cuknns.h:83 (src/cuknnHeap.cu:394) -- same engine, same contract */
double gpuknnsHeap(knntype *query, knntype *data, knntype *values, knntype *indices, int objects,
                   int numQueries, int attributes, int k, int numStreams);

/* include/cuknns.h:85 (src/knnsplan.cu:25) -- measures the engine's
   configurations on random [-50,50) data of the given shape and records the
   fastest; fills every plan field */
void knnsplan(knnplan *plan, long int N, long int Q, long int D, long int k);

/* include/cuknns.h:87 (src/knnsexecute.cu:6) -- runs plan.pt2Function and
   prints "Time Elapsed: <seconds>" like the reference */
void knnsexecute(knnplan plan, knntype *data, knntype *queries, knntype *KNNdist, knntype *KNNidx);

#ifdef __cplusplus
}
#endif

#endif /* CUKNNS_GB300_DROPIN_H */
