// engine.h -- host engine internals shared by the C ABI translation units.
#pragma once

#include <cstddef>
#include <cstdint>
#include <mutex>
#include <vector>
#include <cuda_runtime.h>

#include "knn_gb300.h"

namespace knn {

struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    int ensure(size_t bytes);
    void release();
};

struct Config {
    int algo = 0;
    int kp = 0;
    int rerank = 1;
    bool pilot = true;
    int precision = 0;
    int splits = 1;
    int64_t split_len = 0;
    int qtile = 128;
    int dp = 0;
    int dpb = 0;
    int stages = 0;
    // E4M3 keys (KNNS_PREC_FP8): the scan's row width in 16-bit units, (D rounded up to 128) / 2
    bool fp8 = false;
    int dpf = 0;
    // exact form on the 3xTF32 threshold scan (rows wider than 128, or shortlists over 128)
    bool tscan = false;
};

struct Engine {
    int device = 0;
    int sms = 1;
    int cc = 0;
    std::mutex mu;
    cudaEvent_t last_done = nullptr;
    DevBuf cn, qn, part, hi, lo, bf, err, thr, loflags, cn_s, thr2, redo;
    // threshold-scan path: BF16 queries, candidate segments and counts, seeded
    // thresholds, sample norms, failed-query list
    DevBuf qbf, cand, cnt, tq, cnv, fail;
    // E4M3 keys: corpus codes and row scales, query scales, sample scales
    DevBuf f8, cs, qs, csv;
    // 3xTF32 scan: the queries' TF32 hi / lo copies and the low-part flags of their tiles; the
    // failed-query list and fix-up thresholds of the scan when it runs beside the BF16 scan
    // (exact form)
    DevBuf qhi, qlo, qlof, tfail, tthr2;
    // per-search flag words: [0] some corpus tile has a TF32 low part, [1] corpus or
    // queries not BF16-exact, [2] some value not an integer, [3] max |x| (float bits), [4] zero,
    // [5] some query tile has a TF32 low part
    DevBuf words;
    DevBuf in_corpus, in_queries, out_dist, out_idx;
    // corpus blocks of host-buffer searches: two running top-k lists (distances, indices)
    DevBuf mrg;
    // host-buffer searches with the threshold scan: the seeding sample (every 32nd corpus row)
    // copied ahead of the corpus, and its norms, BF16 copy, E4M3 codes and scales
    DevBuf smp, smp_cn, smp_bf, smp_f8, smp_cs, smp_np;
    // BF16 threshold scan: the corpus norms as BF16 parts (kNormParts per row) for the MMA
    DevBuf np;
    // stage timing: kTimingEvents events per timed search (start, after prep,
    // after threshold seeding, after the main fused kernel, after the main
    // selection, end)
    static constexpr int kTimingEvents = 6;
    std::vector<cudaEvent_t> tev;
    int tcount = 0;
    int timing_slot(cudaEvent_t out[kTimingEvents]);
    cudaStream_t host_stream();
    cudaEvent_t t0();
    cudaEvent_t t1();
    // blocked searches: the stream that copies a host corpus in, the stream that prepares its
    // blocks, the streams that scan the blocks prepared, and a pool of ordering events (null on
    // failure)
    static constexpr int kScanWorkers = 2;
    cudaStream_t copy_stream();
    cudaStream_t prep_stream();
    cudaStream_t worker_stream(int i);
    cudaEvent_t order_event(int i);

  private:
    cudaStream_t stream_ = nullptr, copy_ = nullptr, prep_ = nullptr, workers_[kScanWorkers] = {};
    cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
    std::vector<cudaEvent_t> order_;
};

// A corpus prepared once and kept resident (the serving index): BF16 copy,
// norms, optional TF32 hi/lo copies with their per-tile low-part flags,
// optional E4M3 codes with per-row scales, and the corpus half of the flag words ([0] low part, [1] not BF16-exact,
// [2] not integer, [3] max |x| bits).  The caller keeps the FP32 corpus alive
// and unchanged while the index is used.
struct PreparedCorpus {
    const float* corpus = nullptr;
    int64_t N = 0, ldc = 0;
    int D = 0, dpb = 0, dp = 0, dpf = 0;
    bool tf32 = false, fp8 = false;
    DevBuf cn, bf, hi, lo, tiles, words, f8, cs, np;
    void release();
};

int set_error(int code, const char* fmt, ...);
void clear_error();
int get_engine(Engine** out);
int auto_kp(int k, int rerank);
int auto_splits(int64_t qtiles, int64_t tiles, int sms, int max_splits);
int resolve_config(const Engine& E, int64_t N, int64_t Q, int D, int k, const knns_options& o, Config* c);
// pc (optional): the corpus arrives prepared (its preparation is skipped).
// capture: the call is being captured into a CUDA graph: no host-side event
// ordering against earlier calls (the caller serialises its stream).
// host_corpus (optional): the corpus is still in host memory (N x D, contiguous rows) and
// `corpus` is its device destination (ldc = D): the search copies it in on the engine's copy
// stream -- the threshold scan's seeding sample first, then blocks aligned to the main scan's
// splits -- and prepares and scans each block as soon as it has landed, so the copy overlaps
// the computation.  Results are identical to a search of the resident corpus.
int run_search(Engine& E, const float* corpus, int64_t N, int64_t ldc, const float* queries, int64_t Q, int64_t ldq,
               int D, int k, float* dist, int32_t* idx, float* idx_f, const knns_options& o, cudaStream_t s,
               knns_stats* st, const PreparedCorpus* pc = nullptr, bool capture = false,
               const float* host_corpus = nullptr);
int prepare_corpus(Engine& E, PreparedCorpus* pc, const float* corpus, int64_t N, int64_t ldc, int D, bool tf32,
                   cudaStream_t s, bool fp8 = false);
int check_device_error(Engine& E, cudaStream_t s);
int search_host(const float* corpus, int64_t N, const float* queries, int64_t Q, int D, int k, float* dist,
                int32_t* idx, float* idx_f_host, const knns_options& o, double* seconds, knns_stats* st);
void remember_stats(const knns_stats& st);

}  // namespace knn

// the resident index behind the opaque knns_index handle
struct knns_index {
    int device = 0;
    knn::PreparedCorpus pc;
};
