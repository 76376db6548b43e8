/*
 * knn_gb300.h -- status-returning C API of the GB300 brute-force kNN engine.
 *
 * The reference (shengren/knn-toolbox) has no error channel: its entry points
 * return void or an elapsed time (include/cuknns.h:75,83,85,87) and never
 * check a CUDA or cuBLAS status.  This header is the engine's native
 * interface; include/cuknns.h keeps the reference's own names and signatures
 * on top of it for drop-in use.
 *
 * Layout conventions (identical to the reference's, readme.txt:61-69):
 *   corpus   N x D, each vector contiguous ("D is the leading dimension"),
 *   queries  Q x D, each vector contiguous,
 *   outputs  Q x k, each query's k results contiguous ("k is the leading
 *            dimension"), sorted ascending by (distance, index), 0-based.
 * Distances are squared L2.  All sizes are element counts.
 */
#ifndef KNN_GB300_H
#define KNN_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define KNNS_OK 0
#define KNNS_ERR_INVALID 1        /* bad argument (sizes, pointers, k > N, ...) */
#define KNNS_ERR_CUDA 2           /* a CUDA runtime call failed */
#define KNNS_ERR_UNSUPPORTED 3    /* shape outside what the kernels handle */
#define KNNS_ERR_DEVICE_TIMEOUT 4 /* a kernel gave up a bounded wait and wound down */
#define KNNS_ERR_NOMEM 5          /* device or host allocation failed */

/* kernel families */
#define KNNS_ALGO_AUTO 0 /* tensor cores when the shape allows, else CUDA cores */
#define KNNS_ALGO_TC 1   /* tcgen05 tensor cores: BF16 keys for data exact in BF16, else 3xTF32; D <= 128
                            with shortlists <= 128 on any corpus, any D (to 2048) and shortlists up to 512
                            on corpora of at least 16384 rows (the 3xTF32 threshold scan) */
#define KNNS_ALGO_SIMT 2 /* CUDA-core FP32 fused distance + shortlist (any D, shortlist <= 512) */

/* precision of the ranking keys */
#define KNNS_PREC_EXACT 0 /* FP32-accurate keys (BF16 products when the data are BF16-exact, else 3xTF32) */
#define KNNS_PREC_BF16 1  /* BF16 keys pick a shortlist of c*k per query, re-ranked by exact distance
                             (tensor cores, D <= 256; c*k <= 128, or up to 512 on corpora of at least
                             16384 rows, where the threshold scan keeps the shortlist) */
#define KNNS_PREC_FP8 2   /* FP8 E4M3 keys (per-row absmax scales, FP32 accumulation) pick the shortlist
                             on the threshold scan, re-ranked by exact distance; same limits as BF16.
                             Where the scan does not run (N below its threshold, KNNS_SCAN_OFF) and
                             for the rare queries the scan hands to its fix-up, BF16 keys are used */

/* threshold scan: the tensor-core pass keeps no shortlist on chip; per-query thresholds
   seeded from nested corpus samples let it collect only the keys that can still enter the
   top-kp (results are the same).  It runs on BF16 / E4M3 keys, or in the exact form on 3xTF32
   keys for data that are not exact in BF16 (the choice is made on the device). */
#define KNNS_SCAN_AUTO 0 /* N >= 131072: BF16 keys for BF16-exact data (always in the BF16 / FP8
                            forms), 3xTF32 keys otherwise; exact form with 16384 <= N < 131072
                            (and re-rank on): the 3xTF32 scan for any data */
#define KNNS_SCAN_ON 1   /* as AUTO, with the BF16 / 3xTF32 pair from N >= 16384 */
#define KNNS_SCAN_OFF 2  /* never used */
#define KNNS_SCAN_TF32 3 /* exact form: the 3xTF32 threshold scan alone for any data when N >= 16384
                            (by default it also serves rows wider than 128 and k above 128); same results */

typedef struct knns_options {
    int algo;        /* KNNS_ALGO_* */
    int splits;      /* corpus splits processed by independent CTAs; 0 = automatic */
    int rerank;      /* 1 (default): shortlist re-ranked by the exact direct-difference distance;
                        0: reference semantics, rank by ||c||^2 - 2 q.c, distance = key + ||q||^2 */
    int kp;          /* shortlist length per query (multiple of 16, >= 32, >= k); 0 = automatic */
    int timing;      /* 1: record CUDA events around each stage (see knns_timing_collect) */
    int pilot;       /* 1 (default): seed per-query thresholds from a pass over a 1/16 corpus sample
                        (large corpora only); results are identical either way */
    int precision;   /* KNNS_PREC_EXACT (default), KNNS_PREC_BF16 or KNNS_PREC_FP8 */
    int shortlist;   /* BF16 / FP8 forms: shortlist factor c, kp = c*k rounded up to 16 (0 = 4) */
    int scan;        /* KNNS_SCAN_* (default AUTO) */
    int scan_boxes;  /* threshold scan: 64-element K boxes per shared-memory ring slot (0 = automatic) */
    int block_rows;  /* host-buffer searches (knns_search_host, gpuknnsBitonic / gpuknnsHeap): corpus rows
                        per device block; 0 = automatic: the whole corpus when it fits in free device memory,
                        else blocks sized to it.  Each block is searched and merged into the running top-k
                        by (distance, index): results are identical to one search over the whole corpus */
    int tf32_only;   /* exact form: 1 = 3xTF32 keys even for data that are exact in BF16 (the BF16
                        tensor-core shortcut and the threshold scan stand down); results are the same,
                        the kernels slower -- a measurement switch for comparing the two key types */
    int scan_accs;   /* threshold scan: tensor-memory accumulators, 2 (tiles of 224 corpus rows; 192
                        above 128 BF16 columns) or 4 (tiles of 96); 0 = automatic */
    int single_stream; /* host-buffer searches on the threshold scan: 1: copy the corpus, then search it
                        on one stream; 0 (default): copy the corpus in blocks on a second stream,
                        prepare each block as it lands on a third while the seeding passes run, and
                        scan each block as soon as it is ready, on two more.  Same results.  Searches
                        of a resident corpus always run on the caller's stream alone */
} knns_options;

typedef struct knns_stats {
    int algo;        /* family that ran */
    int splits;
    int kp;
    int stages;      /* shared-memory pipeline depth of the tensor-core kernel */
    int launches;    /* kernels launched by the call */
    int pilot;       /* 1 when the threshold-seeding pilot pass ran */
    int64_t workspace_bytes;
    int scan;        /* 1 when the threshold-scan path was launched (it runs when the keys are BF16) */
    int scan_splits; /* corpus splits of the main threshold scan */
    int scan_cap;    /* candidate slots per (query, split half) of the main threshold scan */
    int scan_ring;   /* ring slots x boxes per slot, as 100 * slots + boxes */
    int scan_keys;   /* threshold scans launched: 1 BF16 / E4M3 keys, 2 3xTF32 keys, 3 both (the exact
                        form then runs the one that matches the data: BF16 keys for BF16-exact data) */
} knns_stats;

/* Fill *opt with the defaults (automatic algo, splits and shortlist, re-rank on, pilot on). */
void knns_default_options(knns_options *opt);

/*
 * Search with every buffer already in device memory.  Asynchronous on
 * `stream` (a cudaStream_t, NULL = legacy default stream).  ldc / ldq are the
 * row pitches (elements) of corpus and queries; dist / idx are Q x k.
 * `idx` or `dist` may be NULL.  The engine keeps a per-device workspace that
 * grows on demand; calls on one device are serialised on the host, and a
 * later call's stream waits for the previous call's work on the workspace.
 */
int knns_search_device(const float *corpus, int64_t N, int64_t ldc, const float *queries, int64_t Q,
                       int64_t ldq, int D, int k, float *dist, int32_t *idx, const knns_options *opt,
                       void *stream);

/*
 * Search on host buffers: copies corpus and queries to the device, searches,
 * copies results back and synchronises.  Returns KNNS_OK or an error code.
 */
int knns_search_host(const float *corpus, int64_t N, const float *queries, int64_t Q, int D, int k,
                     float *dist, int32_t *idx, const knns_options *opt);

/*
 * Merge of two per-query result lists on the device, by (distance, index): the
 * first `have` entries of run (Q x k) and the first kb entries of blk (Q x kb,
 * indices shifted by `offset`) -> the first min(k, have + kb) entries of their
 * union into out (Q x k; must not alias the inputs).  Both inputs sorted as the
 * search returns them.  It is the exchange step of a corpus split across GPUs
 * (every rank's top-k over its shard, gathered, merged) and of corpus blocks
 * streamed through one GPU -- the reference merges its per-stream corpus chunks
 * on the host instead (mergeResBitonic, src/cuknnBitonic.cu:381-417, called at
 * :586-589).  Asynchronous on `stream`.
 */
int knns_merge_topk(const float *run_d, const int32_t *run_i, int have, const float *blk_d, const int32_t *blk_i,
                    int kb, int32_t offset, int64_t Q, int k, float *out_d, int32_t *out_i, void *stream);

/* Synchronise `stream` and report a kernel-side bounded-wait timeout, if any. */
int knns_check_device(void *stream);

/* Message for the last error raised on the calling thread ("" if none). */
const char *knns_last_error(void);

/* Statistics of the calling thread's last successful search. */
int knns_last_stats(knns_stats *out);

/* Queries of the calling thread's last threshold-scan search that overflowed
 * their candidate segments and were answered by the fix-up pass (0 when the
 * scan did not run).  Diagnostic: synchronises the device. */
int knns_last_fixups(int64_t *out);

/*
 * Stage timings of the searches run with opt->timing = 1 since the last
 * collection, from CUDA events recorded on each search's stream:
 * ms[0] preparation (norms, TF32 split), ms[1] fused distance + shortlist
 * kernel, ms[2] shortlist merge / re-rank.  Synchronises the device; *count
 * receives the number of searches summed.  Resets the accumulator.
 * (The reference kept the same split in knntimes dst_time / srch_time,
 * include/cuknns.h:43-47.)
 */
int knns_timing_collect(double ms[3], int *count);

/*
 * As knns_timing_collect, with five stages: ms[0] preparation, ms[1] threshold
 * seeding (pilot passes and their selections), ms[2] the main fused distance
 * kernel, ms[3] the main merge / selection / re-rank, ms[4] the fix-up of
 * queries whose seeded threshold did not hold.  Resets the accumulator.
 */
int knns_timing_collect5(double ms[5], int *count);

/*
 * Allocation-free search.  No counterpart in the reference: it exists for
 * callers that must not have device memory allocated during a search -- a
 * process whose HBM is already reserved by another allocator (a framework's
 * caching allocator), a latency-critical caller for which cudaMalloc/cudaFree
 * would synchronise the device, or a plug-in host that owns all allocation.
 * Inputs and outputs are the caller's device buffers, as for
 * knns_search_device; the work runs asynchronously on `stream` with the
 * CUDA-core kernel (exact re-rank on, automatic shortlist and splits).
 * Scratch comes from one fixed 8 MiB array in device memory, held by every
 * GPU that loads the library until the process exits; it must hold the corpus
 * norms (4 * roundup(N, 128) bytes), the thresholds (4 * Q bytes) and at least
 * one split of shortlists (8 * Q * kp bytes, kp = k + max(8, k/8) rounded up to
 * 16, at least 32); larger problems are rejected with KNNS_ERR_UNSUPPORTED and
 * a message.  k up to 512 is served, as by knns_search_device's CUDA-core
 * path (the re-rank margin is dropped where it would pass 512 entries).  The
 * first call on a device looks the array's address up (cudaGetSymbolAddress);
 * under CUDA's default lazy module loading that first lookup is also what
 * loads the array into device memory, so the first call can still take
 * 8 MiB of HBM.  Make it -- or call knns_noalloc_prepare -- once per device
 * at start-up, before another allocator takes the HBM and before any stream
 * capture.  Every call shares the array: calls whose GPU work overlaps
 * (other streams, other host threads) race on it and must be serialised by
 * the caller.  The cached address belongs to the device's primary context:
 * do not use the entry point across a cudaDeviceReset.  The function calls
 * no cudaMalloc, cudaFree or allocating library routine.
 */
int knns_search_device_noalloc(const float *corpus, int64_t N, int64_t ldc, const float *queries, int64_t Q,
                               int64_t ldq, int D, int k, float *dist, int32_t *idx, void *stream);

/* Set-up of knns_search_device_noalloc on the current device only: looks up (and so
   loads) its scratch array, which the first search would otherwise do.  Idempotent. */
int knns_noalloc_prepare(void);

/*
 * Resident index (no counterpart in the reference, whose drivers copy the corpus
 * to the device on every call, src/cuknnBitonic.cu:493-512).  knns_index_create
 * prepares a device corpus once -- BF16 copy, row norms, the exactness and
 * integrality flags and, with KNNS_INDEX_TF32, the TF32 hi/lo copies the exact
 * form needs for data that are not BF16-exact -- and synchronises `stream`.
 * The caller keeps the FP32 corpus alive and unchanged while the index is used;
 * searches on it skip the corpus preparation.  D <= 256.
 */
#define KNNS_INDEX_TF32 1
#define KNNS_INDEX_FP8 2 /* also prepare E4M3 codes and row scales (the KNNS_PREC_FP8 form) */
typedef struct knns_index knns_index;
int knns_index_create(const float *corpus, int64_t N, int64_t ldc, int D, int flags, knns_index **out,
                      void *stream);
int knns_index_search(knns_index *index, const float *queries, int64_t Q, int64_t ldq, int k, float *dist,
                      int32_t *idx, const knns_options *opt, void *stream);
void knns_index_destroy(knns_index *index);

/*
 * Shortlist autotuner of the precision forms (precision KNNS_PREC_BF16 or
 * KNNS_PREC_FP8): searches the given device queries (a sample of the
 * workload) with the exact form and with the form's keys at
 * shortlist factors c = 2, 4, 8 (while c*k <= 512), and returns in *c_out the
 * smallest c whose recall@k against the exact form reaches `target` (else the
 * largest tried), its recall in *recall_out.  Synchronises `stream`; needs an
 * index with TF32 copies unless the data are BF16-exact.
 */
int knns_autotune_shortlist(knns_index *index, const float *queries, int64_t Q, int64_t ldq, int k, int precision,
                            double target, int *c_out, double *recall_out, void *stream);

/*
 * Serving form (no counterpart in the reference): a request server over a
 * resident index.  Requests of uneven size (1..max_batch queries, host memory,
 * copied at submit) and k (1..128) arrive at any time from any thread; one worker
 * thread packs pending requests, oldest first, into launches of at most
 * max_batch queries -- in the exact form requests of any k (the launch runs the
 * largest k and each request keeps the first k of its sorted rows), in the
 * BF16 / FP8 forms those that share the oldest request's k (their shortlist is
 * c*k) -- keeps `slots` launches in flight on
 * their own streams and workspaces (a batch formed while another runs overlaps
 * it on the device), and runs each launch as a CUDA graph captured once per
 * (size bucket, k) and slot (buckets: powers of two from 32 to max_batch).  With
 * autotune = 1 the corpus split count of each graph is chosen by timing
 * candidates before capture.  A request's results are the ones a search of that
 * request alone returns (same k, same computation per query).
 */
typedef struct knns_server knns_server;
typedef struct knns_server_config {
    int slots;     /* launches in flight (default 2) */
    int max_batch; /* queries per launch, a power of two (default 1024) */
    int precision; /* KNNS_PREC_* (default exact) */
    int shortlist; /* BF16 / FP8 forms: shortlist factor c (0 = 4) */
    int autotune;  /* 1 (default): time candidate split counts before capturing a graph */
    int reserved[3];
} knns_server_config;
void knns_server_default_config(knns_server_config *cfg);
int knns_server_create(knns_index *index, const knns_server_config *cfg, knns_server **out);
/* Returns the request id (> 0), or minus an error code. */
int64_t knns_server_submit(knns_server *server, const float *queries, int64_t Q, int k);
/* Blocks until the request is answered; dist / idx receive Q x k values (may be NULL). */
int knns_server_wait(knns_server *server, int64_t id, float *dist, int32_t *idx, double *latency_ms);
/* Capture, on every slot, the graphs of each bucket (rounded up to a power of two) x k
   before traffic (otherwise each is captured at its first use).  Call it while no
   request is pending. */
int knns_server_warmup(knns_server *server, const int *buckets, int nb, const int *ks, int nk);
/* out: requests submitted, launches, queries launched, graphs captured. */
int knns_server_stats(knns_server *server, int64_t out[4]);
void knns_server_destroy(knns_server *server);

/* Library version as 10000*major + 100*minor + patch. */
int knns_version(void);

/*
 * Test hook of the bounded waits: the next search on any thread runs its
 * shortlist kernels (the tensor-core path) with every barrier wait bounded by
 * timeout_us and with their copy engines idle, so the waits run out: each
 * kernel records KNNS_ERR_DEVICE_TIMEOUT, winds down (nothing is in flight) and
 * returns; knns_check_device then reports it and the context stays usable.
 * The search's results are undefined.  0 < timeout_us <= 10 s.
 */
int knns_debug_stall_next_search(int64_t timeout_us);

/*
 * Test hook: raw 3xTF32 dot products of the first 128 queries against the
 * first 128 corpus rows, as the tensor-core kernel's accumulator holds them
 * (dump: 128 x 128 floats, device memory).  Synchronous.
 */
int knns_debug_tc_dot_tile(const float *corpus, int64_t N, const float *queries, int64_t Q, int D,
                           float *dump);

/*
 * Test hook: the preparation pass over a device matrix x[n][ld] (D columns),
 * every output in device memory: norms[n] (the float rounding of the double
 * sum of squares in column order), bf16[n][round64(D)] (BF16 copy, zero
 * padded), f8[n][round128(D)] (E4M3 codes) with scales[n] (per-row absmax /
 * 448), words[3] ([0] not BF16-exact, [1] some value not an integer, [2] max
 * |x| as float bits), norm_parts[n][16] (optional: the norm as BF16 parts n1 + n2 + n3,
 * then zeros, the BF16 scan's norm operand).  D <= 384.  Synchronous.
 */
int knns_debug_prep(const float *x, int64_t n, int64_t ld, int D, float *norms, void *bf16, void *f8,
                    float *scales, uint32_t *words, void *norm_parts);

/* The threshold scan's plan for an exact-form search (default options), computed on the host
 * alone (no GPU is touched): the seeding levels, coarsest first, and the main pass.  tf32 = 1
 * gives the 3xTF32 scan's plan, 0 the BF16 scan's; sms is the GPU's SM count. */
#define KNNS_MAX_SEED_LEVELS 6
typedef struct knns_scan_plan_info {
    int kp;                                      /* shortlist length */
    int tile_rows;                               /* corpus rows per tile (MMA N) */
    int levels;
    int64_t level_rows[KNNS_MAX_SEED_LEVELS];    /* sample rows (every level_stride-th corpus row) */
    int64_t level_stride[KNNS_MAX_SEED_LEVELS];
    int level_rank[KNNS_MAX_SEED_LEVELS];        /* rank of the level's threshold among its keys */
    int level_splits[KNNS_MAX_SEED_LEVELS];
    int level_cap[KNNS_MAX_SEED_LEVELS];         /* candidate slots per (query, segment) */
    int splits;                                  /* main pass */
    int64_t split_len;
    int cap;
    int sel_words;                               /* bound on one query's stored main-pass candidates */
} knns_scan_plan_info;
int knns_debug_scan_plan(int64_t N, int64_t Q, int D, int k, int sms, int tf32, knns_scan_plan_info *out);

#ifdef __cplusplus
}
#endif

#endif /* KNN_GB300_H */
